"""GPU parity of the motion-compensation / autofocus hooks against the FP64
oracle: back-projection with per-pulse range and phase corrections (every
mode), the weighted projection (adjoint) and the sharpness autofocus.

Tolerances (relative L2): SPLIT / FP16STORE -60 dB, FP64 -100 dB, FP32 (the
plain comparator) -20 dB; projection -60 dB; autofocus phases within 0.02 rad
of the oracle's after the same iterations."""
import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import metrics, sarbp, scenes

from test_oracle_autofocus import autofocus_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sarbp.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def case(orc):
    s = scenes.config1(np_=256, ns=1024, n_img=96)
    rc = orc.range_compress(s, orc.echo(s))
    rng = np.random.default_rng(11)
    dr = rng.uniform(-0.3, 0.3, s.np_)
    ph = rng.uniform(-np.pi, np.pi, s.np_)
    return s, rc, dr, ph


def bp_gpu(ctx, s, rc, mode, dr=None, ph=None):
    r, g, lay = sarbp.scene_args(s)
    if mode == sarbp.MODE_FP16STORE:
        h = rc.astype(np.complex64).view(np.float32).reshape(rc.shape[0], -1, 2)
        scale = np.maximum(np.abs(h).max(axis=(1, 2)), 1e-30).astype(np.float32) / 2.0 ** 14
        scale = (2.0 ** np.ceil(np.log2(scale))).astype(np.float32)
        h16 = (h / scale[:, None, None]).astype(np.float16)
        return ctx.backproject(r, h16, s.apc, g, mode, lay.t0_bins, lay.bin_rate, scale=scale, drange=dr, dphase=ph)
    return ctx.backproject(r, rc.astype(np.complex64), s.apc, g, mode, lay.t0_bins, lay.bin_rate,
                           drange=dr, dphase=ph)


@pytest.mark.parametrize("mode,tol", [(sarbp.MODE_SPLIT, -60.0), (sarbp.MODE_FP16STORE, -60.0),
                                      (sarbp.MODE_FP64, -100.0), (sarbp.MODE_FP32, -20.0)])
def test_backprojection_with_corrections(ctx, orc, case, mode, tol):
    s, rc, dr, ph = case
    ref = orc.backproject_corr(s, rc.astype(np.complex64), dr, ph)
    img = bp_gpu(ctx, s, rc, mode, dr, ph)
    err = metrics.rel_l2_db(img, ref)
    print("mode", mode, "corrected BP rel-L2 dB", err)
    assert err <= tol


def test_zero_corrections_are_bit_identical(ctx, case):
    s, rc, _, _ = case
    z = np.zeros(s.np_)
    a = bp_gpu(ctx, s, rc, sarbp.MODE_SPLIT)
    b = bp_gpu(ctx, s, rc, sarbp.MODE_SPLIT, z, z)
    assert np.array_equal(a, b)


def test_device_correction_arrays(ctx, case):
    torch = pytest.importorskip("torch")
    s, rc, dr, ph = case
    host = bp_gpu(ctx, s, rc, sarbp.MODE_SPLIT, dr, ph)
    dev = bp_gpu(ctx, s, rc, sarbp.MODE_SPLIT, torch.from_numpy(dr).cuda(), torch.from_numpy(ph).cuda())
    assert np.array_equal(host, dev)


@pytest.mark.parametrize("mode", [sarbp.MODE_SPLIT, sarbp.MODE_FP16STORE])
def test_weighted_projection(ctx, orc, case, mode):
    s, rc, dr, ph = case
    r, g, lay = sarbp.scene_args(s)
    rng = np.random.default_rng(5)
    w = (rng.standard_normal((g.ny, g.nx)) + 1j * rng.standard_normal((g.ny, g.nx))).astype(np.complex64)
    ref = orc.project_weighted(s, rc.astype(np.complex64), w, dr, ph)
    if mode == sarbp.MODE_FP16STORE:
        h = rc.astype(np.complex64).view(np.float32).reshape(rc.shape[0], -1, 2)
        scale = (2.0 ** np.ceil(np.log2(np.abs(h).max(axis=(1, 2)) / 2.0 ** 14))).astype(np.float32)
        out = ctx.project_weighted(r, (h / scale[:, None, None]).astype(np.float16), s.apc, g, mode, lay.t0_bins,
                                   lay.bin_rate, w, scale=scale, drange=dr, dphase=ph)
    else:
        out = ctx.project_weighted(r, rc.astype(np.complex64), s.apc, g, mode, lay.t0_bins, lay.bin_rate, w,
                                   drange=dr, dphase=ph)
    err = metrics.rel_l2_db(out, ref)
    print("projection rel-L2 dB", err)
    assert err <= -60.0
    # adjoint identity on the GPU's own image: sum_x conj(W) I = sum_p out[p]
    img = bp_gpu(ctx, s, rc, mode, dr, ph)
    lhs = np.vdot(w.astype(np.complex128), img.astype(np.complex128))
    assert abs(lhs - out.sum()) <= 1e-3 * abs(lhs)


@pytest.mark.parametrize("np_", [253, 17, 1])
def test_weighted_projection_odd_pulse_counts(ctx, orc, np_):
    """Pulses are summed in pairs: odd chunk tails (253 = 15 x 16 + 13 over
    several segments, 17, a single pulse) against the oracle."""
    s = scenes.config1(np_=np_, ns=1024, n_img=96)
    rc = orc.range_compress(s, orc.echo(s)).astype(np.complex64)
    r, g, lay = sarbp.scene_args(s)
    rng = np.random.default_rng(np_)
    w = (rng.standard_normal((g.ny, g.nx)) + 1j * rng.standard_normal((g.ny, g.nx))).astype(np.complex64)
    ref = orc.project_weighted(s, rc, w, None, None)
    out = ctx.project_weighted(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, w)
    assert out.shape == (np_,)
    err = metrics.rel_l2_db(out, ref)
    print("projection rel-L2 dB", np_, err)
    assert err <= -60.0


def test_projection_is_deterministic(ctx, case):
    s, rc, dr, ph = case
    r, g, lay = sarbp.scene_args(s)
    w = np.ones((g.ny, g.nx), dtype=np.complex64)
    a = ctx.project_weighted(r, rc.astype(np.complex64), s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, w)
    b = ctx.project_weighted(r, rc.astype(np.complex64), s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, w)
    assert np.array_equal(a, b)


def test_autofocus_matches_oracle_and_recovers(ctx, orc):
    s, rc, eps = autofocus_case(orc)
    rce = rc * np.exp(1j * eps)[:, None]
    r, g, lay = sarbp.scene_args(s)
    iters = 6
    ph, sharp, img = ctx.autofocus(r, rce.astype(np.complex64), s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins,
                                   lay.bin_rate, iters)
    ph_ref, sharp_ref, _ = orc.autofocus(s, rce.astype(np.complex64), iters)
    print("max |phase - oracle| rad", np.abs(ph - ph_ref).max(), "sharpness", sharp[0], "->", sharp[-1])
    assert np.abs(ph - ph_ref).max() <= 0.02
    assert np.allclose(sharp, sharp_ref, rtol=1e-3)
    res = ph + eps
    k = np.arange(s.np_)
    A = np.vstack([np.ones_like(k), k]).T
    res -= A @ np.linalg.lstsq(A, res, rcond=None)[0]
    assert res.std() < 0.02
    base = orc.backproject(s, rc)
    gph = np.vdot(img, base)
    assert metrics.rel_l2_db(img * gph / abs(gph), base) <= -30.0


def test_autofocus_rejects_bad_arguments(ctx, case):
    s, rc, _, _ = case
    r, g, lay = sarbp.scene_args(s)
    with pytest.raises(sarbp.SarbpError):
        ctx.autofocus(r, rc.astype(np.complex64), s.apc, g, sarbp.MODE_FP32, lay.t0_bins, lay.bin_rate, 2)
    with pytest.raises(sarbp.SarbpError):
        ctx.autofocus(r, rc.astype(np.complex64), s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, 2,
                      dphase=np.full(s.np_, np.nan))
