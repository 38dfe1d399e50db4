"""Oracle (FP64, CPU) checks of the omega-K restatement: the committed
RADARSAT-1 golden crop, the range-term sign pinned by focusing the reference's
own scene, padding sizes, and the Stolt stage's identity when the mapping
vanishes."""
import os

import numpy as np

from oracle import wk
from sar_cambrianaccelerationcard_gb300 import metrics

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "wk_cd_crop.npz")


def test_golden_crop_reproduced():
    g = np.load(GOLDEN)
    img = wk.wk_image(g["echo"].astype(np.complex128), wk.radarsat1())
    assert img.shape == (128, 106)
    assert metrics.rel_l2_db(img.astype(np.complex64), g["image"]) <= -120.0


def test_range_term_sign_focuses_the_reference_scene():
    g = np.load(GOLDEN)
    assert float(g["sharp_file"]) > 10.0 * float(g["sharp_flip"])


def test_padded_sizes():
    assert wk.padded_size(3072, 2048) == (4096, 3414)   # the reference's scene (wk.cc:76-96)
    assert wk.padded_size(9, 9) == (13, 15)             # round half away from zero
    assert wk.padded_size(96, 64) == (128, 106)


def test_stolt_is_identity_without_mapping():
    """With vr -> infinity the mapping fr_new = fr and theta carries only the
    range term: every output takes its own input sample (sinc(0) = 1)."""
    rng = np.random.default_rng(1)
    S = rng.standard_normal((16, 30)) + 1j * rng.standard_normal((16, 30))
    p = wk.WkParams(fr=1e6, prf=100.0, f0=1e9, r0=0.0, kr=1e12, vr=1e30, f_nc=0.0)
    fr, _ = wk.axes(p, 16, 30)
    out = wk.rfm_stolt(S, p)
    ref = S * np.exp(1j * np.pi * fr[None, :] ** 2 / p.kr)
    tol = 1e-9 * np.abs(ref).max()
    assert np.abs(out[:, 1:-1] - ref[:, 1:-1]).max() <= tol
    # the reference clips taps to the row, so at the edges the clipped taps
    # stack on the edge sample: taps floor(n + k - 3), k = 0..5
    assert np.abs(out[:, 0] - 4 * ref[:, 0]).max() <= tol      # k = 0..3 -> index 0
    assert np.abs(out[:, -1] - 3 * ref[:, -1]).max() <= tol    # k = 3..5 -> index NR - 1
