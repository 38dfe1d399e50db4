"""include/sarbp_reference_shim.hpp: the reference's launchGenerateEcho /
launchBackProjection signatures on top of libsarbp.

CPU: the shim compiles into a program written against the reference's
interface and links to libsarbp.so.  GPU: that program runs the reference's
flow (echo generation, then back-projection) and its image focuses the
reference's brightest target (amplitude 1.5 at (Az0, Rg0), BPA_CUDA.cpp:31)
at pixel (Mslow/2, Nfast/2).  Against the reference's own code and the
oracle: the shim's echo matches the echo the reference's generateEchoKernel
computed (tests/golden/ref_echo.npz), and the shim's image of that echo
matches the FP64 oracle under the shim's data model."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sar_cambrianaccelerationcard_gb300")


def build_flow(tmpdir):
    from sar_cambrianaccelerationcard_gb300 import build
    build.build()
    cuda_inc = "/usr/local/cuda/include"
    cuda_lib = "/usr/local/cuda/lib64"
    exe = os.path.join(tmpdir, "ref_flow")
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc,
           os.path.join(ROOT, "tests", "shim", "ref_flow.cpp"), "-o", exe, "-L", PKG, "-lsarbp",
           f"-Wl,-rpath,{PKG}", "-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{cuda_lib}"]
    subprocess.run(cmd, check=True)
    return exe


def test_shim_compiles_and_links(tmp_path):
    exe = build_flow(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_reference_flow_through_shim_focuses(tmp_path):
    exe = build_flow(str(tmp_path))
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    _, i, j, v = out.stdout.split()
    assert abs(int(i) - 128) <= 1 and abs(int(j) - 4800) <= 1, out.stdout
    assert float(v) > 0


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["near", "default"])
def test_shim_echo_matches_reference_kernel(name):
    """sarbp_launch_generate_echo (launchGenerateEcho's signature, FP64 inside)
    against the echo the reference's own generateEchoKernel computed for the
    same SARParams, targets and axes (tests/golden/ref_echo.npz): identical
    gate decisions, and within one FP32 ulp of the reference's phase."""
    torch = pytest.importorskip("torch")
    from ref_echo_case import load, phase_ulp_db
    from sar_cambrianaccelerationcard_gb300 import metrics, sarbp
    case = load(name)
    p = case["params"]
    rp = sarbp.RefParams.from_buffer_copy(case["raw"])
    out = torch.zeros((p["Mslow"], 2 * p["Nfast"]), dtype=torch.float32, device="cuda")
    pt, ta, tr = _dev(torch, case["ptarget"]), _dev(torch, case["ta"]), _dev(torch, case["tr"])
    lib = sarbp.load()
    st = lib.sarbp_launch_generate_echo(out.data_ptr(), pt.data_ptr(), ta.data_ptr(), tr.data_ptr(), ctypes.byref(rp),
                                        p["Mslow"], p["Nfast"])
    assert st == sarbp.OK
    mine = out.cpu().numpy().view(np.complex64)
    ref = case["echo"]
    assert np.array_equal(np.abs(ref) > 0, np.abs(mine) > 0), "gate decisions differ"
    err = metrics.rel_l2_db(mine, ref)
    print(name, f"shim echo vs reference kernel {err:.1f} dB (bound {phase_ulp_db(p):.1f} dB)")
    assert err <= phase_ulp_db(p)


@pytest.mark.gpu
def test_shim_image_matches_oracle(orc):
    """sarbp_launch_back_projection (launchBackProjection's signature) on the
    reference kernel's own echo of its default geometry (64 pulses x 9600
    samples, H = 5 km, Rg0 = 10 km) against the FP64 oracle under the shim's
    data model (tc = 0, t_rec0 = 0, 8x upsampling, ta linspace, 1 m ground
    pixels centred on the scene centre): the whole 64 x 9600 image within
    -60 dB."""
    torch = pytest.importorskip("torch")
    from ref_echo_case import load, oracle_shim_image
    from sar_cambrianaccelerationcard_gb300 import metrics, sarbp
    case = load("default")
    p = case["params"]
    rp = sarbp.RefParams.from_buffer_copy(case["raw"])
    echo = case["echo"]
    d_echo = _dev(torch, echo.view(np.float32))
    d_img = torch.zeros((p["Mslow"], 2 * p["Nfast"]), dtype=torch.float32, device="cuda")
    lib = sarbp.load()
    st = lib.sarbp_launch_back_projection(d_echo.data_ptr(), d_img.data_ptr(), ctypes.byref(rp), p["Mslow"],
                                          p["Nfast"])
    assert st == sarbp.OK
    img = d_img.cpu().numpy().view(np.complex64)
    ref = oracle_shim_image(orc, case, echo)
    err = metrics.rel_l2_db(img, ref)
    pk = np.unravel_index(np.argmax(np.abs(ref)), ref.shape)
    print(f"shim image vs oracle {err:.1f} dB, oracle peak {pk}, shim peak "
          f"{np.unravel_index(np.argmax(np.abs(img)), img.shape)}")
    assert err <= -60.0
