"""FP64 restatement of the reference's omega-K (Stolt) imager, test
infrastructure only (tests/, bench.py's CPU legs).

Follows code/SAR_WK/wk_v5.2.3 (process_wk, wk.cc:43-343) step by step, with
numpy's FFTs (any length) in double precision:
  * padding round(na/6) / round(nr/3) rows / columns each side
    (task/preprocess.cc:22-25, PadComplexTensor) and azimuth down-conversion
    by exp(-j 2 pi f_nc ta), ta = (m - NA//2) / PRF (preprocess.cc:35-41);
  * 2-D FFT, range then azimuth (task/fft.cc: cnnlExecFFT over rows, transpose,
    rows, transpose), unnormalised;
  * frequency axes from the fftshifted index (wk.cc:181-205);
  * reference function exp(j theta), theta = 4 pi R0 / c sqrt(max(0, (f0 + fr)^2 -
    c^2 fa^2 / (4 Vr^2))) + pi fr^2 / kr, kr with the parameter file's sign
    (task/compression.cc:17-73 with Kr = -params.Kr; mian_wka_sinc.m step 2);
  * Stolt mapping (task/stolt.cc:324+): delta = (fr_new - fr) Nr / Fr,
    centre = n - delta, taps at clip(floor(centre + k - P/2), 0, Nr - 1),
    weight sin(pi u) / (pi u) with u = centre - tap, summed over the P taps;
  * 2-D IFFT with 1/Nr and 1/Na (fft.cc:224,282).
Differences from the reference, both in the reference's float arithmetic:
the reference computes the down-conversion phase and the Stolt centre in
FP32 (this restatement in FP64), and its sinc is a divide-no-NaN, which gives
the tap at an exact-integer centre weight 0 where sin(pi u)/(pi u) -> 1.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class WkParams:
    fr: float          # range sampling rate (Hz)
    prf: float         # azimuth sampling rate (Hz)
    f0: float          # carrier (Hz)
    r0: float          # reference slant range (m)
    kr: float          # range FM rate (Hz/s), parameter-file sign
    c: float = 299790000.0
    vr: float = 7062.0
    f_nc: float = -6900.0
    taps: int = 6


def radarsat1() -> WkParams:
    """The reference scene's parameters (paras.txt values; Vr, f_nc as wk.cc:60-62)."""
    return WkParams(fr=32317000.0, prf=1256.98, f0=5.3e9, r0=988647.462, kr=-721350000000.0)


def pads(na: int, nr: int):
    # round(Na / 6.0f): float division, half away from zero
    return int(math.floor(float(np.float32(na) / np.float32(6.0)) + 0.5)), \
        int(math.floor(float(np.float32(nr) / np.float32(3.0)) + 0.5))


def padded_size(na: int, nr: int):
    pa, pr = pads(na, nr)
    return na + 2 * pa, nr + 2 * pr


def axes(p: WkParams, NA: int, NR: int):
    n = np.arange(NR)
    fr = (np.where(n < NR // 2, n + NR // 2, n - NR // 2) - NR // 2) * (p.fr / NR)
    m = np.arange(NA)
    fa = p.f_nc + (np.where(m < NA // 2, m + NA // 2, m - NA // 2) - NA // 2) * (p.prf / NA)
    return fr.astype(np.float64), fa.astype(np.float64)


def pad_downconvert(echo, p: WkParams):
    na, nr = echo.shape
    pa, pr = pads(na, nr)
    NA, NR = na + 2 * pa, nr + 2 * pr
    x = np.zeros((NA, NR), dtype=np.complex128)
    x[pa:pa + na, pr:pr + nr] = echo
    ta = (np.arange(NA) - NA // 2) / p.prf
    return x * np.exp(-2j * np.pi * p.f_nc * ta)[:, None]


def rfm_stolt(S, p: WkParams):
    NA, NR = S.shape
    fr, fa = axes(p, NA, NR)
    root = np.sqrt(np.maximum((p.f0 + fr[None, :]) ** 2 - p.c ** 2 / (4.0 * p.vr ** 2) * fa[:, None] ** 2, 0.0))
    theta = 4.0 * np.pi * p.r0 / p.c * root + np.pi * fr[None, :] ** 2 / p.kr
    X = S * np.exp(1j * theta)
    delta = (root - p.f0 - fr[None, :]) * (NR / p.fr)
    centre = np.arange(NR)[None, :] - delta
    rows = np.arange(NA)[:, None]
    out = np.zeros_like(X)
    for k in range(p.taps):
        idx = np.clip(np.floor(centre + (k - 0.5 * p.taps)), 0, NR - 1).astype(np.int64)
        out += X[rows, idx] * np.sinc(centre - idx)
    return out


def wk_image(echo, p: WkParams):
    x = pad_downconvert(np.asarray(echo, dtype=np.complex128), p)
    S = np.fft.fft(np.fft.fft(x, axis=1), axis=0)
    return np.fft.ifft(np.fft.ifft(rfm_stolt(S, p), axis=1), axis=0)
