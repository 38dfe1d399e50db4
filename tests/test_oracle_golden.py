"""Pins the FP64 oracle.

* FFT stage: the reference's own known-answer case
  (code/fft_simple/fft_kt_sample.cc:5-29: 2x4 all-ones -> FFT (4,0,0,0) per row
  -> unnormalised IFFT (4,4,4,4)) and the all-ones 131072-point row of
  code/fft_simple/fft_test.cu:36-40 / fft_test.m:6 (X[0] = N, zeros elsewhere).
* MATLAB profile: golden vectors from the line-by-line transcription of
  code/SAR_BP/matlab/BPA_SAR.m (tests/golden/gen_golden.py): echo (:80-89),
  compressed rows (:100), upsampled rows (:111) and the back-projected image on
  a subset of the script's grid (:177-197).
"""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "bpa_sar_m.npz")


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_fft_known_answer_2x4(orc):
    x = np.ones((2, 4), dtype=np.complex128)
    X = np.stack([orc.fft(r, -1) for r in x])
    assert np.array_equal(X, np.array([[4, 0, 0, 0], [4, 0, 0, 0]], dtype=np.complex128))
    Y = X * np.ones((2, 4))                      # step2 "dotmultiple" with ones
    y = np.stack([orc.fft(r, +1) for r in Y])    # unnormalised inverse
    assert np.array_equal(y, np.full((2, 4), 4.0 + 0j))


def test_fft_all_ones_131072(orc):
    n = 128 * 1024
    X = orc.fft(np.ones(n, dtype=np.complex128), -1)
    assert X[0] == n
    assert np.max(np.abs(X[1:30])) == 0.0
    assert np.max(np.abs(X[1:])) < 1e-6


@pytest.mark.parametrize("n", [2, 8, 64, 1024, 4096])
def test_fft_matches_dft_definition(orc, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    k = np.arange(n)
    W = np.exp(-2j * np.pi * (np.outer(k, k) % n) / n) if n <= 1024 else None
    X = orc.fft(x, -1)
    ref = W @ x if W is not None else np.fft.fft(x)
    assert rel_l2(X, ref) < 1e-13
    assert rel_l2(orc.fft(X, +1) / n, x) < 1e-13


def test_fft_rejects_non_power_of_two(orc):
    with pytest.raises(ValueError):
        orc.fft(np.ones(6, dtype=np.complex128))


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="module")
def matlab_chain(orc, golden):
    g = golden
    Nfast, Mslow, L = int(g["Nfast"]), int(g["Mslow"]), int(g["L"])
    dt = (float(g["tr_end"]) - float(g["tr0"])) / (Nfast - 1)
    apc = np.column_stack([g["vr"] * g["ta"], np.zeros(Mslow), np.full(Mslow, float(g["H"]))])
    tg = np.column_stack([g["ptarget"][:, 0], g["ptarget"][:, 1], np.zeros(5), g["ptarget"][:, 2]])
    echo = orc.echo_raw(apc, tg, float(g["tr0"]), dt, Nfast, float(g["Kr"]), float(g["Tw"]),
                        0.0, True, float(g["La"]) / 2, float(g["fc"]), float(g["c"]))
    h = orc.chirp(Nfast, dt, float(g["Kr"]), float(g["Tw"]), 0.0, True)
    sar2, sar1 = orc.range_compress_raw(echo, h, Nfast, 0, L, 1.0 / (L * Nfast), L * Nfast,
                                        want_sar1=True)
    return dict(apc=apc, echo=echo, sar1=sar1, sar2=sar2)


def test_matlab_profile_echo(golden, matlab_chain):
    e = matlab_chain["echo"][golden["prow"]]
    assert rel_l2(e, golden["echo_rows"]) < 1e-9


def test_matlab_profile_range_compression(golden, matlab_chain):
    assert rel_l2(matlab_chain["sar1"][golden["prow"]], golden["sar1_rows"]) < 1e-9
    assert rel_l2(matlab_chain["sar2"][golden["prow"]][:, ::4], golden["sar2_rows"]) < 1e-9


def test_matlab_profile_backprojection(orc, golden, matlab_chain):
    g = golden
    L = int(g["L"])
    img = np.zeros_like(g["image"])
    origin = np.array([g["az"][0], g["rg"][0], 0.0])
    ux = np.array([0.0, 0.1, 0.0])   # columns step in ground range (Rg)
    uy = np.array([0.05, 0.0, 0.0])  # rows step in azimuth (Az)
    for a, i in enumerate(g["rows"]):
        for b, j in enumerate(g["cols"]):
            img[a, b] = orc.backproject_raw(matlab_chain["sar2"], matlab_chain["apc"], origin, ux, uy,
                                            (int(j), int(i), 1, 1), float(g["fc"]), float(g["c"]),
                                            float(g["tr0"]), float(g["Fr"]) * L, interp=1)[0, 0]
    assert rel_l2(img, g["image"]) < 1e-9
    # The brightest pixel is the 1.5-amplitude target at (Az0, Rg0) (BPA_SAR.m:64),
    # found one 0.1 m range column early (Rg index 499, not 500): the script maps
    # delay tau to the 1-based index round((tau - min(trs))*Fr*L), whose sample
    # lies one upsampled bin before tau.  The product profile uses 0-based bins.
    assert np.unravel_index(np.abs(img).argmax(), img.shape) == (8, 6)
