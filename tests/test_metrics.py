"""Known answers for the image metrics (metrics.py).

The reference judges its images by eye: a -3 dB contour of the magnitude
(code/SAR_BP/matlab/BPA_SAR.m:168-175, :213-220).  The metrics that replace it
are pinned here on an analytic point response, img = sinc((x - x0)/rho)
sinc((y - y0)/rho) with a resolution of rho pixels and a sub-pixel position:
  * PSLR of a sinc: first sidelobe 0.21723 of the peak, -13.26 dB (+-0.05);
  * -3 dB width: 0.8859 rho (+-0.01 rho);
  * ISLR: sidelobe / main-lobe energy of sinc^2 over the span the cut covers
    (integrated numerically here; +-0.05 dB);
  * peak position: (x0, y0) within 0.01 pixel.
"""
import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import metrics, scenes

FIRST_SIDELOBE_DB = 20.0 * np.log10(0.217233628)  # -13.2619 dB
HALF_POWER_WIDTH = 0.885893                         # of sinc^2, in resolution cells


def sinc_image(n, rho, x0, y0, amp=1.0 + 0.0j):
    yy, xx = np.mgrid[0:n, 0:n].astype(np.float64)
    return amp * np.sinc((xx - x0) / rho) * np.sinc((yy - y0) / rho)


def islr_expected(rho, lo, hi):
    """10 log10 of the sinc^2 energy outside the main lobe (|u| < rho) over
    its energy inside, for u in [lo, hi)."""
    u = np.linspace(lo, hi, 4_000_001)[:-1]
    s = np.sinc(u / rho) ** 2
    main = np.abs(u) < rho
    return 10.0 * np.log10(s[~main].sum() / s[main].sum())


@pytest.mark.parametrize("rho", [2.0, 3.0, 4.0, 6.0])
@pytest.mark.parametrize("x0,y0", [(128.0, 128.0), (128.3, 127.8), (100.45, 140.1), (60.71, 90.37)])
def test_point_target_on_analytic_sinc(rho, x0, y0):
    img = sinc_image(256, rho, x0, y0, amp=0.7 * np.exp(0.4j))
    t = metrics.point_target(img, int(round(x0)), int(round(y0)))
    assert abs(t.x - x0) <= 0.01 and abs(t.y - y0) <= 0.01, (t.x, t.y)
    assert abs(t.peak - 0.7) <= 1e-3
    for pslr in (t.pslr_range_db, t.pslr_azimuth_db):
        assert abs(pslr - FIRST_SIDELOBE_DB) <= 0.05, pslr
    for w in (t.width_range, t.width_azimuth):
        assert abs(w / rho - HALF_POWER_WIDTH) <= 0.01, w / rho
    # the cuts cover the patch: columns [xc - 32, xc + 32) around the brightest pixel
    xc, yc = int(round(x0)), int(round(y0))
    assert abs(t.islr_range_db - islr_expected(rho, xc - 32 - x0, xc + 32 - x0)) <= 0.05
    assert abs(t.islr_azimuth_db - islr_expected(rho, yc - 32 - y0, yc + 32 - y0)) <= 0.05


def test_point_target_at_image_border():
    """A target 10 pixels from the edge: the patch is clipped, the position and
    PSLR still come out (ISLR then covers the shorter span)."""
    x0, y0 = 10.3, 200.6
    img = sinc_image(256, 3.0, x0, y0)
    t = metrics.point_target(img, 10, 201)
    assert abs(t.x - x0) <= 0.01 and abs(t.y - y0) <= 0.01
    assert abs(t.pslr_azimuth_db - FIRST_SIDELOBE_DB) <= 0.05
    assert abs(t.pslr_range_db - FIRST_SIDELOBE_DB) <= 0.1


def test_rel_l2_known_answers():
    rng = np.random.default_rng(1)
    a = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
    assert metrics.rel_l2_db(1.01 * a, a) == pytest.approx(-40.0, abs=1e-9)
    assert metrics.rel_l2_db(a * np.exp(1e-3j), a) == pytest.approx(20 * np.log10(2 * np.sin(5e-4)), abs=1e-6)
    assert metrics.rel_l2_db(a, a) == float("-inf")
    assert metrics.rel_l2_db(np.zeros(4), np.zeros(4)) == float("-inf")
    assert metrics.rel_l2_db(np.ones(4), np.zeros(4)) == float("inf")


def test_compare_point_targets_sees_a_shift_and_a_sidelobe_change():
    """Identical images compare as zero; a 0.2-pixel shift and a 20% first
    sidelobe (a tapered response) show up in the differences."""
    ref = sinc_image(128, 3.0, 64.2, 63.9)
    same = metrics.compare_point_targets(ref, ref, [(64, 64)])
    assert same["peak_shift_px"] == 0.0 and same["pslr_diff_db"] == 0.0 and same["islr_diff_db"] == 0.0
    moved = metrics.compare_point_targets(sinc_image(128, 3.0, 64.4, 63.9), ref, [(64, 64)])
    assert abs(moved["peak_shift_px"] - 0.2) <= 0.01
    yy, xx = np.mgrid[0:128, 0:128].astype(np.float64)
    tapered = np.sinc((xx - 64.2) / 3.0) ** 2 * np.sinc((yy - 63.9) / 3.0)  # range PSLR -26.5 dB
    diff = metrics.compare_point_targets(tapered, ref, [(64, 64)])
    assert diff["pslr_diff_db"] > 10.0


def test_target_pixels_on_grid():
    s = scenes.config1()
    px = metrics.target_pixels(s)
    assert len(px) == 9
    # the centre target (0, R0, 0) sits on pixel (nx/2, ny/2)
    assert (s.grid.nx // 2, s.grid.ny // 2) in px
