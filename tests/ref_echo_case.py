"""Shared helpers for tests/golden/ref_echo.npz (echoes computed by the
reference's own generateEchoKernel, run as host code; see
tests/golden/gen_ref_echo_golden.py)."""
import os
import struct

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_echo.npz")
FIELDS = ("c", "fc", "lam", "Kr", "Tr", "Br", "Fr", "vr", "H", "La", "Rg0", "Az0", "Nfast", "Mslow", "Ntarget")


def load(name):
    g = np.load(GOLDEN)
    raw = g[f"{name}_params"].tobytes()
    p = dict(zip(FIELDS, struct.unpack("<12f3i", raw)))
    return dict(params=p, raw=raw, ptarget=g[f"{name}_ptarget"], ta=g[f"{name}_ta"], tr=g[f"{name}_tr"],
                echo=g[f"{name}_echo"])


def phase_ulp_db(p):
    """20 log10 of one FP32 ulp of the largest phase the reference's kernel
    forms, 4 pi R / lambda (its echo is computed in FP32): the agreement an
    exact evaluation of the same formula can be expected to reach."""
    r = np.sqrt((p["La"] / 2 + 40.0) ** 2 + (p["Rg0"] + 40.0) ** 2 + p["H"] ** 2)
    phase = np.float32(4.0 * np.pi / p["lam"] * r)
    return float(20.0 * np.log10(np.spacing(phase)))


def oracle_echo(orc, case):
    """The oracle's echo for the case's SARParams, targets and axes."""
    p = case["params"]
    pt = case["ptarget"].reshape(-1, 3).astype(np.float64)
    apc = np.zeros((p["Mslow"], 3))
    apc[:, 0] = p["vr"] * case["ta"].astype(np.float64)
    apc[:, 2] = p["H"]
    tg = np.column_stack([pt[:, 0], pt[:, 1], np.zeros(len(pt)), pt[:, 2]])
    dt = float(np.float32(1.0) / np.float32(p["Fr"]))
    return orc.echo_raw(apc, tg, 0.0, dt, p["Nfast"], p["Kr"], p["Tr"], 0.0, True, p["La"] / 2,
                        p["c"] / p["lam"], p["c"])


def oracle_shim_image(orc, case, echo):
    """The oracle's image under sarbp_launch_back_projection's data model:
    uncentred chirp (tc = 0) over Tr, tr_i = i / Fr (t_rec0 = 0), 8x upsampling,
    APC_m = (vr ta_m, 0, H) with ta = linspace(-La/(2 vr), La/(2 vr), Mslow) in
    FP64, 1 m ground pixels centred on (Az0, Rg0), image [Mslow][Nfast]."""
    p = case["params"]
    fs, tp, kr, c, fc = p["Fr"], p["Tr"], p["Kr"], p["c"], p["fc"]
    na, nr = p["Mslow"], p["Nfast"]
    nc = int(round(tp * fs))
    nfft = 1 << (nr + nc - 2).bit_length()
    shift = nc // 2
    h = orc.chirp(nc, 1.0 / fs, kr, tp, 0.0, False)
    rc = orc.range_compress_raw(echo.astype(np.complex128), h, nfft, shift, 8, 1.0 / nfft, 8 * nr)
    ta0, ta1 = -p["La"] / (2.0 * p["vr"]), p["La"] / (2.0 * p["vr"])
    ta = ta0 + np.arange(na) * ((ta1 - ta0) / (na - 1))
    apc = np.zeros((na, 3))
    apc[:, 0] = p["vr"] * ta
    apc[:, 2] = p["H"]
    origin = np.array([p["Az0"] - na // 2, p["Rg0"] - nr // 2, 0.0])
    return orc.backproject_raw(rc, apc, origin, np.array([0.0, 1.0, 0.0]), np.array([1.0, 0.0, 0.0]),
                               (0, 0, nr, na), fc, c, -shift / fs, 8 * fs)
