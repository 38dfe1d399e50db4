"""Generates tests/golden/ref_echo.npz: echoes computed by the reference's own
generateEchoKernel (code/SAR_BP/CUDA/BPA_CUDA_kernels.cu:3-45), compiled from
the reference source as host code by oracle/ref (make -C oracle/ref echo) and
run on the CPU in FP32.

Two parameter sets, each the reference's default SARParams (BPA_CUDA.h:28-50)
with the record long enough to hold the targets' echoes (its default record of
Nfast = Tr Fr = 300 samples from delay 0 ends before any echo arrives, so the
default echo is all zero) and the aperture La widened so the targets stay in
the azimuth gate:
  "near":    H = 0, Rg0 = 300 m, Mslow = 64, Nfast = 1024, La = 100 m
             (phase 4 pi R / lambda ~ 7e4 rad: FP32 phase error ~ 1e-2 rad);
  "default": H = 5000 m, Rg0 = 10000 m (the defaults), Mslow = 64, Nfast =
             9600, La = 100 m (phase ~ 2.5e6 rad: FP32 phase error ~ 0.25 rad).
Targets: the reference's five (BPA_CUDA.cpp:26-32 layout, offsets from
(Az0, Rg0)); ta = linspace(-La/(2 vr), La/(2 vr), Mslow) and tr = i / Fr in
FP32 as BPA_CUDA.cpp:35-48 computes them.

    python tests/golden/gen_ref_echo_golden.py [<reference checkout>]
(without an argument, oracle/ref's Makefile default is used)
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
OUT = os.path.join(ROOT, "tests", "golden", "ref_echo.npz")
F = np.float32

CASES = {
    "near": dict(H=0.0, Rg0=300.0, Mslow=64, Nfast=1024, La=100.0),
    "default": dict(H=5000.0, Rg0=10000.0, Mslow=64, Nfast=9600, La=100.0),
}


def params(H, Rg0, Mslow, Nfast, La):
    """SARParams fields as float32 / int32 (defaults of BPA_CUDA.h:29-48)."""
    c, fc = F(3e8), F(5.3e9)
    return dict(c=c, fc=fc, lam=F(c / fc), Kr=F(4e12), Tr=F(2.5e-6), Br=F(1e8), Fr=F(1.2e8), vr=F(150.0),
                H=F(H), La=F(La), Rg0=F(Rg0), Az0=F(0.0), Nfast=Nfast, Mslow=Mslow, Ntarget=5)


def inputs(p):
    az0, rg0 = p["Az0"], p["Rg0"]
    pt = np.array([az0 - F(10), rg0 - F(20), 1.0, az0 + F(20), rg0 + F(30), 0.8, az0 - F(30), rg0 + F(10), 1.2,
                   az0 + F(40), rg0 - F(40), 0.9, az0, rg0, 1.5], dtype=np.float32)
    ta_start = F(-p["La"] / (F(2) * p["vr"]))
    ta_end = F(p["La"] / (F(2) * p["vr"]))
    step = F((ta_end - ta_start) / F(p["Mslow"] - 1))
    ta = (ta_start + np.arange(p["Mslow"], dtype=np.float32) * step).astype(np.float32)
    tr = (np.arange(p["Nfast"], dtype=np.float32) * F(F(1) / p["Fr"])).astype(np.float32)
    return pt, ta, tr


def pack(p):
    return struct.pack("<12f3i", p["c"], p["fc"], p["lam"], p["Kr"], p["Tr"], p["Br"], p["Fr"], p["vr"], p["H"],
                       p["La"], p["Rg0"], p["Az0"], p["Nfast"], p["Mslow"], p["Ntarget"])


def main(ref_dir=None):
    cmd = ["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "echo"]
    if ref_dir:
        cmd.append(f"REF={ref_dir}")
    subprocess.run(cmd, check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_echo_host")
    out = {}
    for name, kw in CASES.items():
        p = params(**kw)
        pt, ta, tr = inputs(p)
        with tempfile.TemporaryDirectory() as d:
            fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
            with open(fin, "wb") as f:
                f.write(pack(p) + pt.tobytes() + ta.tobytes() + tr.tobytes())
            subprocess.run([exe, fin, fout], check=True)
            echo = np.fromfile(fout, dtype=np.complex64).reshape(p["Mslow"], p["Nfast"])
        nz = np.count_nonzero(echo)
        print(name, "nonzero samples", nz, "of", echo.size)
        assert nz > 0
        out[f"{name}_params"] = np.frombuffer(pack(p), dtype=np.uint8)
        out[f"{name}_ptarget"] = pt
        out[f"{name}_ta"] = ta
        out[f"{name}_tr"] = tr
        out[f"{name}_echo"] = echo
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SARBP_REFERENCE_DIR"))
