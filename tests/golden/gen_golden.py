"""Generates tests/golden/bpa_sar_m.npz: golden vectors of the reference's MATLAB
back-projection specification, code/SAR_BP/matlab/BPA_SAR.m.

MATLAB/Octave are not available, so the script is transcribed line by line
into vectorised numpy (numpy.fft has MATLAB's fft/ifft definitions).  The
transcription is deliberately independent of the C oracle (different FFT,
vectorised instead of looped, MATLAB indexing kept literally) so that
agreement between the two pins the oracle's MATLAB profile to the script.

Kept from the script: every parameter (:7-51), the 5 targets (:59-64), the echo
(:80-89, noise line :90 is commented out in the script), the range compression
(:93-100), the 8x upsampling (:106-111) and the upsampled back-projection
(:177-197) with nearest-bin lookup ``round`` (half away from zero) and
1-based ``SAR2(m, nr(m))``.  Only a subset of the 2001 x 1001 image grid
(:127-130) is evaluated to keep the fixture small.

Run from the repository root:  python tests/golden/gen_golden.py
"""
from __future__ import annotations

import math
import os

import numpy as np


def matlab_round(x):
    return np.where(x >= 0, np.floor(x + 0.5), np.ceil(x - 0.5))


def nextpow2(n):
    return int(math.ceil(math.log2(n)))


def run():
    # ---- parameters, BPA_SAR.m:7-51
    c = 3e8
    fc = 1e9
    lam = c / fc
    vr = 100.0
    H = 5000.0
    D = 4.0
    Rg0 = 10e3
    RgL = 1000.0
    R0 = math.sqrt(Rg0 ** 2 + H ** 2)
    La = lam * R0 / D
    Ta = La / vr
    Tw = 5e-6
    Br = 30e6
    Kr = Br / Tw
    Fr = 2 * Br
    Rmin = math.sqrt((Rg0 - RgL / 2) ** 2 + H ** 2)
    Rmax = math.sqrt((Rg0 + RgL / 2) ** 2 + H ** 2 + (La / 2) ** 2)
    Nfast = math.ceil(2 * (Rmax - Rmin) / c * Fr + Tw * Fr)
    Nfast = 2 ** nextpow2(Nfast)
    tr = np.linspace(2 * Rmin / c, 2 * Rmax / c + Tw, Nfast)
    Fr = 1 / ((2 * Rmax / c + Tw - 2 * Rmin / c) / Nfast)
    Az0 = 10e3
    AL = 1000.0
    Azmin = Az0 - AL / 2
    Azmax = Az0 + AL / 2
    Ka = -2 * vr ** 2 / lam / R0
    Ba = abs(Ka * Ta)
    PRF = 1.2 * Ba
    Mslow = math.ceil((Azmax - Azmin + La) / vr * PRF)
    Mslow = 2 ** nextpow2(Mslow)
    ta = np.linspace((Azmin - La / 2) / vr, (Azmax + La / 2) / vr, Mslow)

    # ---- targets, :59-64
    Ptarget = np.array([[Az0 - 10, Rg0 - 20, 1.0],
                        [Az0 + 20, Rg0 + 30, 0.8],
                        [Az0 - 30, Rg0 + 10, 1.2],
                        [Az0 + 40, Rg0 - 40, 0.9],
                        [Az0, Rg0, 1.5]])

    # ---- echo, :80-89
    Srnm = np.zeros((Mslow, Nfast), dtype=np.complex128)
    for k in range(Ptarget.shape[0]):
        sigmak = Ptarget[k, 2]
        Azk = ta * vr - Ptarget[k, 0]
        Rk = np.sqrt(Azk ** 2 + Ptarget[k, 1] ** 2 + H ** 2)
        tauk = 2 * Rk / c
        tk = np.ones((Mslow, 1)) * tr[None, :] - tauk[:, None] * np.ones((1, Nfast))
        phasek = np.pi * Kr * tk ** 2 - (4 * np.pi / lam) * (Rk[:, None] * np.ones((1, Nfast)))
        Srnm = Srnm + sigmak * np.exp(1j * phasek) * ((0 < tk) & (tk < Tw)) * \
            ((np.abs(Azk) < La / 2)[:, None] * np.ones((1, Nfast)))

    # ---- range compression, :93-100
    thr = tr - 2 * Rmin / c
    hrc = np.exp(1j * np.pi * Kr * thr ** 2) * ((0 < thr) & (thr < Tw))
    SRN_FFT = np.fft.fft(Srnm, Nfast, axis=1)
    HRC_FFT = np.fft.fft(hrc, Nfast)
    SSAR = SRN_FFT * np.conj(HRC_FFT)[None, :]
    SAR1 = np.fft.ifft(SSAR, Nfast, axis=1)

    # ---- 8x upsampling, :106-111
    L = 8
    trs_min = tr.min()  # only min(trs) is used downstream
    SAR1f = np.fft.fft(SAR1, Nfast, axis=1)
    half = (Nfast + 1) // 2
    SAR11f = np.concatenate([SAR1f[:, :half], np.zeros((Mslow, (L - 1) * Nfast)),
                             SAR1f[:, half:]], axis=1)
    SAR2 = np.fft.ifft(SAR11f, L * Nfast, axis=1)

    # ---- grid, :127-130 (subset of rows / columns, 0-based indices)
    Rg = Rg0 - 50 + 0.1 * np.arange(1001)
    Az = Az0 - 50 + 0.05 * np.arange(2001)
    rows = np.array([0, 250, 400, 600, 799, 800, 801, 999, 1000, 1001, 1400, 1600, 1800, 2000])
    cols = np.array([0, 100, 199, 200, 201, 300, 499, 500, 501, 600, 700, 800, 1000])

    # ---- back-projection with upsampling, :177-197
    img = np.zeros((rows.size, cols.size), dtype=np.complex128)
    for a, i in enumerate(rows):
        for b, j in enumerate(cols):
            Rt = np.sqrt((vr * ta - Az[i]) ** 2 + Rg[j] ** 2 + H ** 2)
            tau = 2 * Rt / c
            nr = matlab_round((tau - trs_min) * Fr * L).astype(np.int64)
            assert nr.min() >= 1 and nr.max() <= L * Nfast
            rd = SAR2[np.arange(Mslow), nr - 1]
            rd = rd * np.exp(1j * 4 * np.pi * fc / c * Rt)
            img[a, b] = rd.sum()

    prow = np.array([0, 700, 1024, 1500, Mslow - 1])
    return dict(
        c=c, fc=fc, vr=vr, H=H, La=La, Tw=Tw, Kr=Kr, Fr=Fr, L=L, Nfast=Nfast, Mslow=Mslow,
        tr0=tr[0], tr_end=tr[-1], ta=ta, ptarget=Ptarget,
        rg=Rg, az=Az, rows=rows, cols=cols, prow=prow,
        echo_rows=Srnm[prow], sar1_rows=SAR1[prow], sar2_rows=SAR2[prow][:, ::4],
        image=img,
    )


def main():
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bpa_sar_m.npz")
    np.savez_compressed(out, **run())
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
