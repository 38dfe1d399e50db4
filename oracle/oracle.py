"""ctypes front end of the FP64 CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product library never does.  It builds nothing by itself:
``build()`` runs ``make`` in this directory (gcc + OpenMP).

The functions follow code/SAR_BP/matlab/BPA_SAR.m (see sarbp_oracle.h for the
line map) in two profiles: ``product`` (what the CUDA path computes) and
``matlab`` (the script's own conventions, for pinning).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liborc.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_fft.argtypes = [_dp, ctypes.c_int, ctypes.c_int]
        L.orc_fft.restype = ctypes.c_int
        L.orc_chirp.argtypes = [_dp, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                ctypes.c_double, ctypes.c_double, ctypes.c_int]
        L.orc_range_compress.argtypes = [_dp, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_int, _dp, _dp]
        L.orc_range_compress.restype = ctypes.c_int
        L.orc_echo.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_double,
                               ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                               ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                               ctypes.c_double, _dp]
        L.orc_add_noise.argtypes = [_dp, ctypes.c_int64, ctypes.c_double, ctypes.c_uint64]
        L.orc_noise_sample.argtypes = [ctypes.c_uint64, ctypes.c_int64, _dp, _dp]
        L.orc_mean_power.argtypes = [_dp, ctypes.c_int64]
        L.orc_mean_power.restype = ctypes.c_double
        bp_args = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp,
                   ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                   ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                   ctypes.c_int, _dp]
        L.orc_backproject.argtypes = [_dp] + bp_args
        L.orc_backproject_c64.argtypes = [_fp] + bp_args
        corr_args = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp,
                     ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                     ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                     ctypes.c_int, _dp, _dp]
        L.orc_backproject_corr.argtypes = [_dp] + corr_args + [_dp]
        L.orc_project_weighted.argtypes = [_dp] + corr_args + [_dp, _dp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_get_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _d(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def threads() -> int:
    return int(lib().orc_get_threads())


# ------------------------------------------------------------- primitives --

def fft(x, sign: int = -1) -> np.ndarray:
    y = _c128(x).copy()
    if lib().orc_fft(_d(y.view(np.float64)), y.shape[-1], sign) != 0:
        raise ValueError("orc_fft: size must be a power of two")
    return y


def chirp(n: int, dt: float, kr: float, tp: float, tc: float, strict: bool) -> np.ndarray:
    h = np.zeros(n, dtype=np.complex128)
    lib().orc_chirp(_d(h.view(np.float64)), n, dt, kr, tp, tc, int(strict))
    return h


def range_compress_raw(echo, h, nfft: int, shift: int, L: int, norm: float, nout: int,
                       want_sar1: bool = False):
    echo = _c128(echo)
    h = _c128(h)
    np_, ns = echo.shape
    out = np.zeros((np_, nout), dtype=np.complex128)
    sar1 = np.zeros((np_, nfft), dtype=np.complex128) if want_sar1 else None
    rc = lib().orc_range_compress(_d(echo.view(np.float64)), np_, ns, _d(h.view(np.float64)),
                                  h.shape[0], nfft, shift, L, norm, nout,
                                  _d(out.view(np.float64)),
                                  _d(sar1.view(np.float64)) if sar1 is not None else None)
    if rc != 0:
        raise ValueError("orc_range_compress: bad sizes")
    return (out, sar1) if want_sar1 else out


def echo_raw(apc, targets, t_rec0, dt, ns, kr, tp, tc, strict, beam_hw, fc, c) -> np.ndarray:
    apc = np.ascontiguousarray(apc, dtype=np.float64)
    tg = np.ascontiguousarray(targets, dtype=np.float64)
    np_ = apc.shape[0]
    out = np.zeros((np_, ns), dtype=np.complex128)
    lib().orc_echo(_d(apc), np_, _d(tg), tg.shape[0], t_rec0, dt, ns, kr, tp, tc,
                   int(strict), beam_hw, fc, c, _d(out.view(np.float64)))
    return out


def add_noise(x: np.ndarray, sigma: float, seed: int) -> None:
    assert x.dtype == np.complex128 and x.flags.c_contiguous
    lib().orc_add_noise(_d(x.view(np.float64)), x.size, sigma, ctypes.c_uint64(seed & (2**64 - 1)))


def noise_sample(seed: int, i: int):
    g0 = ctypes.c_double()
    g1 = ctypes.c_double()
    lib().orc_noise_sample(ctypes.c_uint64(seed & (2**64 - 1)), i, ctypes.byref(g0), ctypes.byref(g1))
    return g0.value, g1.value


def mean_power(x: np.ndarray) -> float:
    x = _c128(x)
    return float(lib().orc_mean_power(_d(x.view(np.float64)), x.size))


def backproject_raw(rc, apc, origin, ux, uy, region, fc, c, t0, binrate,
                    interp: int = 0) -> np.ndarray:
    """region = (x0, y0, w, h).  rc may be complex128 or complex64."""
    apc = np.ascontiguousarray(apc, dtype=np.float64)
    o = np.ascontiguousarray(origin, dtype=np.float64)
    a = np.ascontiguousarray(ux, dtype=np.float64)
    b = np.ascontiguousarray(uy, dtype=np.float64)
    x0, y0, w, h = (int(v) for v in region)
    img = np.zeros((h, w), dtype=np.complex128)
    np_, nbins = rc.shape
    args = (np_, nbins, _d(apc), _d(o), _d(a), _d(b), x0, y0, w, h, fc, c, t0, binrate,
            int(interp), _d(img.view(np.float64)))
    if rc.dtype == np.complex64:
        rcc = np.ascontiguousarray(rc)
        lib().orc_backproject_c64(rcc.view(np.float32).ctypes.data_as(_fp), *args)
    else:
        rcc = _c128(rc)
        lib().orc_backproject(_d(rcc.view(np.float64)), *args)
    return img


def _opt(a):
    return None if a is None else _d(np.ascontiguousarray(a, dtype=np.float64))


def backproject_corr_raw(rc, apc, origin, ux, uy, region, fc, c, t0, binrate,
                         drange=None, dphase=None, interp: int = 0) -> np.ndarray:
    """Back-projection with per-pulse range (m) and phase (rad) corrections."""
    apc = np.ascontiguousarray(apc, dtype=np.float64)
    x0, y0, w, h = (int(v) for v in region)
    img = np.zeros((h, w), dtype=np.complex128)
    rcc = _c128(rc)
    np_, nbins = rcc.shape
    dr = None if drange is None else np.ascontiguousarray(drange, dtype=np.float64)
    dp = None if dphase is None else np.ascontiguousarray(dphase, dtype=np.float64)
    lib().orc_backproject_corr(_d(rcc.view(np.float64)), np_, nbins, _d(apc), _opt(origin), _opt(ux), _opt(uy),
                               x0, y0, w, h, fc, c, t0, binrate, int(interp),
                               None if dr is None else _d(dr), None if dp is None else _d(dp),
                               _d(img.view(np.float64)))
    return img


def project_weighted_raw(rc, apc, origin, ux, uy, region, fc, c, t0, binrate, weight,
                         drange=None, dphase=None, interp: int = 0) -> np.ndarray:
    """out[p] = sum over the region of conj(weight) * pulse p's term."""
    apc = np.ascontiguousarray(apc, dtype=np.float64)
    x0, y0, w, h = (int(v) for v in region)
    wt = _c128(weight)
    assert wt.shape == (h, w)
    rcc = _c128(rc)
    np_, nbins = rcc.shape
    out = np.zeros(np_, dtype=np.complex128)
    dr = None if drange is None else np.ascontiguousarray(drange, dtype=np.float64)
    dp = None if dphase is None else np.ascontiguousarray(dphase, dtype=np.float64)
    lib().orc_project_weighted(_d(rcc.view(np.float64)), np_, nbins, _d(apc), _opt(origin), _opt(ux), _opt(uy),
                               x0, y0, w, h, fc, c, t0, binrate, int(interp),
                               None if dr is None else _d(dr), None if dp is None else _d(dp),
                               _d(wt.view(np.float64)), _d(out.view(np.complex128).view(np.float64)))
    return out


# ------------------------------------------------------- product profile --

def echo(scene, noise: bool = True) -> np.ndarray:
    """Noiseless point-target echo plus counter-based complex Gaussian noise at
    scene.snr_db below the mean noiseless power (same stream as the GPU
    synthesiser)."""
    r = scene.radar
    e = echo_raw(scene.apc, scene.targets, scene.t_rec0, 1.0 / r.fs, scene.ns, r.kr, r.tp,
                 r.tp / 2.0, False, 0.0, r.fc, r.c)
    if noise and scene.snr_db is not None:
        from sar_cambrianaccelerationcard_gb300.scenes import noise_sigma
        add_noise(e, noise_sigma(mean_power(e), scene.snr_db), scene.seed)
    return e


def range_compress(scene, echo_data) -> np.ndarray:
    r = scene.radar
    lay = scene.layout
    h = chirp(lay.nc, 1.0 / r.fs, r.kr, r.tp, r.tp / 2.0, False)
    # norm 1/nfft on the L*nfft inverse keeps the compressed amplitude (no 1/L)
    return range_compress_raw(echo_data, h, lay.nfft, lay.shift, r.upsample,
                              1.0 / lay.nfft, lay.nbins)


def backproject(scene, rc, region=None) -> np.ndarray:
    g = scene.grid
    lay = scene.layout
    if region is None:
        region = (0, 0, g.nx, g.ny)
    return backproject_raw(rc, scene.apc, g.origin, g.ux, g.uy, region, scene.radar.fc,
                           scene.radar.c, lay.t0_bins, lay.bin_rate, 0)


def image(scene, echo_data, region=None) -> np.ndarray:
    return backproject(scene, range_compress(scene, echo_data), region)


def backproject_corr(scene, rc, drange=None, dphase=None, region=None) -> np.ndarray:
    g = scene.grid
    lay = scene.layout
    if region is None:
        region = (0, 0, g.nx, g.ny)
    return backproject_corr_raw(rc, scene.apc, g.origin, g.ux, g.uy, region, scene.radar.fc, scene.radar.c,
                                lay.t0_bins, lay.bin_rate, drange, dphase)


def project_weighted(scene, rc, weight, drange=None, dphase=None) -> np.ndarray:
    g = scene.grid
    lay = scene.layout
    return project_weighted_raw(rc, scene.apc, g.origin, g.ux, g.uy, (0, 0, g.nx, g.ny), scene.radar.fc,
                                scene.radar.c, lay.t0_bins, lay.bin_rate, weight, drange, dphase)


def autofocus(scene, rc, iterations: int, dphase=None, drange=None):
    """Sharpness-maximising per-pulse phase estimation, the FP64 statement of
    the product's sarbp_autofocus: each iteration images with the current
    phases, forms W = |I|^2 I, projects it onto every pulse
    (c_p = sum conj(W) term_p) and sets dphase[p] -= arg(c_p), then removes
    the mean.  Returns (dphase, sharpness per iteration, final image)."""
    np_ = rc.shape[0]
    ph = np.zeros(np_) if dphase is None else np.array(dphase, dtype=np.float64)
    sharp = []
    for _ in range(iterations):
        img = backproject_corr(scene, rc, drange, ph)
        a2 = np.abs(img) ** 2
        sharp.append(float(np.sum(a2 * a2)))
        cp = project_weighted(scene, rc, a2 * img, drange, ph)
        ph = ph - np.angle(cp)
        ph -= ph.mean()
    img = backproject_corr(scene, rc, drange, ph)
    a2 = np.abs(img) ** 2
    sharp.append(float(np.sum(a2 * a2)))
    return ph, sharp, img
