"""Oracle (FP64, CPU) checks of the motion-compensation / autofocus pieces:
per-pulse corrections in back-projection, the weighted projection as the
adjoint and exact sharpness gradient, and the autofocus iteration on a
well-posed scene.  Small cases (64 x 64 pixels at 1 m, 128-256 pulses)."""
import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import metrics, scenes


@pytest.fixture(scope="module")
def scene_rc(orc):
    s = scenes.config1(np_=128, ns=1024, n_img=64, spacing=1.0)
    rc = orc.range_compress(s, orc.echo(s))
    return s, rc


def test_null_corrections_leave_bp_unchanged(orc, scene_rc):
    s, rc = scene_rc
    assert np.array_equal(orc.backproject_corr(s, rc), orc.backproject(s, rc))


def test_phase_correction_is_a_per_pulse_rotation(orc, scene_rc):
    """dphase[p] multiplies pulse p's contribution by exp(j dphase[p])."""
    s, rc = scene_rc
    ph = np.random.default_rng(1).uniform(-np.pi, np.pi, s.np_)
    a = orc.backproject_corr(s, rc, None, ph)
    b = orc.backproject(s, rc * np.exp(1j * ph)[:, None])
    assert metrics.rel_l2_db(a, b) <= -200.0


def test_range_correction_equals_moved_antenna(orc, scene_rc):
    """A range correction equal to the change of |apc - pixel| when the
    antenna moves along the line of sight to the scene centre reproduces the
    moved-antenna image at the scene centre."""
    s, rc = scene_rc
    dr = np.full(s.np_, 0.3)
    img = orc.backproject_corr(s, rc, dr, None, region=(24, 24, 16, 16))
    centre = np.array([0.0, s.radar.r0, 0.0])
    u = (s.apc - centre) / np.linalg.norm(s.apc - centre, axis=1)[:, None]
    moved = scenes.Scene(**{**s.__dict__, "apc": s.apc + 0.3 * u})
    ref = orc.backproject(moved, rc, region=(24, 24, 16, 16))
    # exact at the centre pixel, close nearby (the line of sight varies slowly)
    assert metrics.rel_l2_db(img[8, 8], ref[8, 8]) <= -60.0
    assert metrics.rel_l2_db(img, ref) <= -30.0


def test_projection_is_the_adjoint(orc, scene_rc):
    """sum_x conj(W) BP(x) == sum_p out[p] (same corrections)."""
    s, rc = scene_rc
    rng = np.random.default_rng(2)
    w = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
    ph = rng.uniform(-1, 1, s.np_)
    dr = rng.uniform(-0.2, 0.2, s.np_)
    img = orc.backproject_corr(s, rc, dr, ph)
    out = orc.project_weighted(s, rc, w, dr, ph)
    lhs = np.vdot(w, img)
    assert abs(lhs - out.sum()) <= 1e-9 * abs(lhs)


def test_sharpness_gradient(orc, scene_rc):
    """d/d dphase[p] sum |I|^4 = -4 Im(out[p]) with weight |I|^2 I."""
    s, rc = scene_rc
    ph = np.random.default_rng(3).normal(0, 0.3, s.np_)
    img = orc.backproject_corr(s, rc, None, ph)
    out = orc.project_weighted(s, rc, np.abs(img) ** 2 * img, None, ph)

    def sharp(v):
        j = orc.backproject_corr(s, rc, None, v)
        return np.sum(np.abs(j) ** 4)

    for p in (5, 64, 100):
        h = 1e-5
        e = np.zeros(s.np_)
        e[p] = h
        num = (sharp(ph + e) - sharp(ph - e)) / (2 * h)
        assert abs(num - (-4 * out[p].imag)) <= 1e-5 * abs(num)


def test_autofocus_recovers_quadratic_and_random_phase(orc):
    s, rc, eps = autofocus_case(orc)
    base = orc.backproject(s, rc)
    ph, sharp, img = orc.autofocus(s, rc * np.exp(1j * eps)[:, None], 6)
    assert sharp[-1] > 2.0 * sharp[0]
    res = ph + eps
    k = np.arange(s.np_)
    A = np.vstack([np.ones_like(k), k]).T
    res -= A @ np.linalg.lstsq(A, res, rcond=None)[0]
    assert res.std() < 0.02
    g = np.vdot(img, base)
    assert metrics.rel_l2_db(img * g / abs(g), base) <= -30.0


def autofocus_case(orc):
    """A dominant scatterer with two weaker ones (256 pulses, 64 x 64 at 1 m,
    30 dB SNR) and a per-pulse phase error: 2 rad quadratic across the aperture
    plus N(0, 0.4 rad)."""
    s = scenes.config1(np_=256, ns=1024, n_img=64, spacing=1.0)
    s.targets = np.array([[0.0, s.radar.r0, 0.0, 10.0], [10.0, s.radar.r0 + 5, 0.0, 1.0],
                          [-12.0, s.radar.r0 - 8, 0.0, 1.0]])
    rc = orc.range_compress(s, orc.echo(s))
    k = np.arange(s.np_)
    eps = 8.0 * (k / (s.np_ - 1) - 0.5) ** 2 + np.random.default_rng(3).normal(0, 0.4, s.np_)
    return s, rc, eps
