"""Seeded random geometries against the FP64 CPU oracle (BPA_SAR.m:80-111,
177-197 restated in oracle/).

The configured workloads all image a flat grid aligned with a straight or
gently curved track.  Here every case draws its own geometry:
  * pulses 64-640 and grid sides 33-300 (ragged: not multiples of the 32 x 64
    pixel tile or the 16-pulse chunk), pixel spacing 0.2-1.5 m;
  * platform speed 80-250 m/s and PRF 300-800 Hz, a straight or curved track
    (sinusoidal cross-track error of random amplitude and period, jitter),
    the antenna at 0-4 km altitude;
  * the grid rotated by any angle about the vertical, half the cases also
    tilted out of the ground plane, its centre 2-8 km away in ground range and
    up to 50 m off broadside;
  * the recorded swath covers every pixel for every pulse with a random margin,
    in half the cases 1000-3500 samples longer with the scene anywhere inside
    (samples per pulse ragged; 4096- and 8192-point range transforms).
Five isolated point targets with sub-pixel offsets, 30 dB SNR; both sides take
the oracle's FP64 echo cast to complex64.

Checked per case: split FP32 and FP16 storage within -60 dB relative L2 of the
oracle (the accuracy target), FP64 mode within -100 dB; and the checked
kernels (every window index clamped, any change reported) report nothing and
give the same image bits as the production kernels, so the window each tile
stages holds every bin its pixels read on these geometries too.
"""
import math

import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import metrics, sarbp, scenes

N_CASES = 16
TOL_DB = {"split": -60.0, "fp16store": -60.0, "fp64": -100.0}


def random_scene(seed):
    rng = np.random.default_rng(7000 + seed)
    radar = scenes.Radar()
    radar.v = float(rng.uniform(80.0, 250.0))
    radar.prf = float(rng.uniform(300.0, 800.0))
    np_ = int(rng.integers(64, 641))
    nx, ny = int(rng.integers(33, 301)), int(rng.integers(33, 301))
    spacing = float(rng.uniform(0.2, 1.5))
    altitude = 0.0 if rng.random() < 0.4 else float(rng.uniform(500.0, 4000.0))
    ground_range = float(rng.uniform(2000.0, 8000.0))
    if rng.random() < 0.5:
        apc = scenes.curved_track(radar, np_, amp=float(rng.uniform(0.1, 2.0)), period=float(rng.uniform(50.0, 400.0)),
                                  jitter=float(rng.uniform(0.0, 0.05)), seed=seed)
    else:
        apc = scenes.straight_track(radar, np_)
    apc[:, 2] += altitude
    th = float(rng.uniform(0.0, 2.0 * math.pi))
    ux = spacing * np.array([math.cos(th), math.sin(th), 0.0])
    uy = spacing * np.array([-math.sin(th), math.cos(th), 0.0])
    if rng.random() < 0.5:  # tilt the grid plane about the track direction
        a = float(rng.uniform(-0.4, 0.4))
        rot = np.array([[1.0, 0.0, 0.0], [0.0, math.cos(a), -math.sin(a)], [0.0, math.sin(a), math.cos(a)]])
        ux, uy = rot @ ux, rot @ uy
    centre = np.array([float(rng.uniform(-50.0, 50.0)), ground_range, 0.0])
    grid = scenes.Grid(origin=centre - (nx // 2) * ux - (ny // 2) * uy, ux=ux, uy=uy, nx=nx, ny=ny)
    # swath: every pixel of the grid (edges sampled densely) for every pulse
    e = np.linspace(0.0, 1.0, 33)
    fx = np.concatenate([e * (nx - 1), e * (nx - 1), np.zeros(33), np.full(33, nx - 1.0), [0.5 * (nx - 1)]])
    fy = np.concatenate([np.zeros(33), np.full(33, ny - 1.0), e * (ny - 1), e * (ny - 1), [0.5 * (ny - 1)]])
    pts = grid.pixel(fx, fy)
    rng_m = np.linalg.norm(pts[None, :, :] - apc[:, None, :], axis=2)
    rmin, rmax = float(rng_m.min()), float(rng_m.max())
    margin = float(rng.uniform(0.0, 1e-6))
    # half the cases record a longer swath with the scene anywhere inside it
    extra = int(rng.integers(0, 64)) if rng.random() < 0.5 else int(rng.integers(1000, 3500))
    before = int(rng.integers(0, extra + 1))
    t_rec0 = 2.0 * rmin / radar.c - margin - before / radar.fs
    ns = int(math.ceil((2.0 * (rmax - rmin) / radar.c + radar.tp + 2.0 * margin) * radar.fs)) + extra
    targets = scenes.isolated_targets(grid, seed=seed)
    return scenes.Scene(name=f"random{seed}", radar=radar, np_=np_, ns=ns, apc=apc, grid=grid, targets=targets,
                        t_rec0=t_rec0, snr_db=30.0, seed=seed)


def test_generator_stays_in_the_tested_ranges():
    nffts = set()
    for seed in range(N_CASES):
        s = random_scene(seed)
        assert s.layout.nfft <= 16384 and 64 <= s.np_ <= 640, (seed, s.ns, s.np_)
        assert 33 <= s.grid.nx <= 300 and 33 <= s.grid.ny <= 300
        nffts.add(s.layout.nfft)
    assert nffts == {4096, 8192}


@pytest.fixture(scope="module")
def contexts():  # the production and the checked kernels side by side
    plain = sarbp.Context(0)
    checked = sarbp.Context(0)
    checked.debug_set(sarbp.DEBUG_BP_CHECKED, 1)
    yield plain, checked
    plain.close()
    checked.close()


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(N_CASES))
def test_random_geometry_vs_oracle(contexts, orc, seed):
    plain, checked = contexts
    s = random_scene(seed)
    e64 = orc.echo(s).astype(np.complex64)
    ref = orc.image(s, e64.astype(np.complex128))
    errs = {}
    for name in ("split", "fp16store", "fp64"):
        img = sarbp.image_scene(plain, s, e64, sarbp.MODES[name])
        errs[name] = metrics.rel_l2_db(img, ref)
        if name != "fp64":
            img_checked = sarbp.image_scene(checked, s, e64, sarbp.MODES[name])
            assert np.array_equal(img, img_checked), f"{s.name} {name}: checked kernel differs"
    print(s.name, f"np {s.np_} ns {s.ns} grid {s.grid.nx}x{s.grid.ny}",
          " ".join(f"{k} {v:.1f} dB" for k, v in errs.items()))
    for name, err in errs.items():
        assert err <= TOL_DB[name], (s.name, name, err)


def coarse_scene(spacing, seed):
    """Coarse pixels with the grid at 45 degrees to the track, 5 km slant range
    (3 km altitude): both tile sides reach along the line of sight."""
    radar = scenes.Radar()
    np_, n = 256, 160
    apc = scenes.straight_track(radar, np_)
    apc[:, 2] += 3000.0
    th = math.pi / 4
    ux = spacing * np.array([math.cos(th), math.sin(th), 0.0])
    uy = spacing * np.array([-math.sin(th), math.cos(th), 0.0])
    centre = np.array([0.0, 4000.0, 0.0])
    grid = scenes.Grid(origin=centre - (n // 2) * ux - (n // 2) * uy, ux=ux, uy=uy, nx=n, ny=n)
    corners = grid.pixel(np.array([0.0, n - 1, 0.0, n - 1]), np.array([0.0, 0.0, n - 1, n - 1]))
    r = np.linalg.norm(corners[None, :, :] - apc[:, None, :], axis=2)
    t_rec0 = 2.0 * float(r.min()) / radar.c - 2e-7
    ns = int(math.ceil((2.0 * (float(r.max()) - float(r.min())) / radar.c + radar.tp + 4e-7) * radar.fs))
    return scenes.Scene(name=f"coarse{spacing:g}m", radar=radar, np_=np_, ns=ns, apc=apc, grid=grid,
                        targets=scenes.isolated_targets(grid, seed=seed), t_rec0=t_rec0, snr_db=30.0, seed=seed)


@pytest.mark.gpu
@pytest.mark.parametrize("spacing", [2.0, 3.0, 4.0])
def test_coarse_pixels_inside_and_outside_the_split_envelope(contexts, orc, spacing):
    """The split modes expand the differential range in a series about each
    tile centre; the planner takes the tallest tile (32 x 64, 32 x 32 or
    32 x 16 pixels) whose remainder stays below 5e-7 m and refuses the call
    when even the smallest does not, which at 5 km bounds the pixel spacing
    near 2.9 m.  Inside (2 m): within the accuracy target.  Outside (3 and
    4 m): SARBP_ERR_UNSUPPORTED with the reason, and the FP64 mode images the
    same scene within -100 dB of the oracle."""
    plain, _ = contexts
    s = coarse_scene(spacing, seed=int(spacing * 10))
    e64 = orc.echo(s).astype(np.complex64)
    ref = orc.image(s, e64.astype(np.complex128))
    if spacing <= 2.9:
        errs = {name: metrics.rel_l2_db(sarbp.image_scene(plain, s, e64, sarbp.MODES[name]), ref)
                for name in ("split", "fp16store")}
        print(s.name, f"ns {s.ns}", " ".join(f"{k} {v:.1f} dB" for k, v in errs.items()))
        for name, err in errs.items():
            assert err <= TOL_DB[name], (s.name, name, err)
        return
    for name in ("split", "fp16store"):
        with pytest.raises(sarbp.SarbpError) as e:
            sarbp.image_scene(plain, s, e64, sarbp.MODES[name])
        assert e.value.status == sarbp.ERR_UNSUPPORTED and "differential-range series" in str(e.value)
    err = metrics.rel_l2_db(sarbp.image_scene(plain, s, e64, sarbp.MODE_FP64), ref)
    print(s.name, f"ns {s.ns} split refused, fp64 {err:.1f} dB")
    assert err <= TOL_DB["fp64"]


@pytest.mark.gpu
@pytest.mark.parametrize("step_updates", [0, 1 << 24])
def test_served_random_geometries_vs_oracle(contexts, orc, step_updates):
    """Six of the random geometries served together in one mix (the server
    plans each job at submit and advances it in per-step pulse slices: 128
    pulses, or about 2^24 pixel*pulse updates per job and step): every image
    within -60 dB of the oracle and within -100 dB of the same job's one-shot
    image (only the sub-aperture summation order differs)."""
    plain, _ = contexts
    cases = []
    for seed in range(6):
        s = random_scene(seed)
        e64 = orc.echo(s).astype(np.complex64)
        cases.append((s, e64, orc.image(s, e64.astype(np.complex128)),
                      sarbp.image_scene(plain, s, e64, sarbp.MODE_SPLIT)))
    with sarbp.Server(0, max_jobs=6, hbm_budget_bytes=8 << 30, pulses_per_step=128,
                      step_updates=step_updates) as srv:
        tickets = []
        for s, e64, _, _ in cases:
            r, g, _ = sarbp.scene_args(s)
            tickets.append(srv.submit(r, g, e64, s.apc, sarbp.MODE_SPLIT))
        results = [srv.wait(t, 120000) for t in tickets]
    for (s, _, ref, one_shot), (st, stats, img) in zip(cases, results):
        assert st == sarbp.OK, s.name
        err, vs_one = metrics.rel_l2_db(img, ref), metrics.rel_l2_db(img, one_shot)
        print(s.name, f"steps {stats.steps} served vs oracle {err:.1f} dB, vs one-shot {vs_one:.1f} dB")
        assert err <= -60.0 and vs_one <= -100.0, (s.name, err, vs_one)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(6))
def test_corrected_backprojection_on_random_geometries(contexts, orc, seed):
    """Per-pulse range and phase corrections (the motion-compensation hook,
    sarbp_backproject_ex) on the random geometries, against the oracle's
    corrected back-projection of the oracle's own range compression: a smooth
    range error of up to 0.3 m plus 1 cm jitter and an arbitrary phase per
    pulse.  Split within -60 dB, FP64 within -100 dB; the checked kernel
    reports no clamp (the staged windows follow the corrected ranges) and gives
    the same bits."""
    plain, checked = contexts
    s = random_scene(seed)
    rng = np.random.default_rng(900 + seed)
    t = np.arange(s.np_) / s.np_
    drange = 0.3 * np.sin(2 * math.pi * (t * rng.uniform(0.5, 3.0) + rng.uniform())) + rng.normal(0, 0.01, s.np_)
    dphase = rng.uniform(-math.pi, math.pi, s.np_)
    e64 = orc.echo(s).astype(np.complex64)
    rc = orc.range_compress(s, e64.astype(np.complex128))
    ref = orc.backproject_corr(s, rc, drange, dphase)
    r, g, lay = sarbp.scene_args(s)
    rc32 = rc.astype(np.complex64)
    errs = {}
    for name in ("split", "fp64"):
        img = plain.backproject(r, rc32, s.apc, g, sarbp.MODES[name], lay.t0_bins, lay.bin_rate,
                                drange=drange, dphase=dphase)
        errs[name] = metrics.rel_l2_db(img, ref)
        if name == "split":
            again = checked.backproject(r, rc32, s.apc, g, sarbp.MODES[name], lay.t0_bins, lay.bin_rate,
                                        drange=drange, dphase=dphase)
            assert np.array_equal(img, again), s.name
    print(s.name, "corrected:", " ".join(f"{k} {v:.1f} dB" for k, v in errs.items()))
    assert errs["split"] <= TOL_DB["split"] and errs["fp64"] <= TOL_DB["fp64"], (s.name, errs)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(4))
def test_weighted_projection_on_random_geometries(contexts, orc, seed):
    """The weighted projection (the adjoint of back-projection that drives the
    sharpness autofocus, sarbp_project_weighted) on the random geometries with
    per-pulse corrections and random complex weights, against the oracle's
    projection: within -60 dB, and the adjoint identity
    sum_x conj(W) I = sum_p out[p] holds on the GPU's own image to 1e-3."""
    plain, _ = contexts
    s = random_scene(seed)
    rng = np.random.default_rng(1900 + seed)
    drange = rng.normal(0, 0.05, s.np_)
    dphase = rng.uniform(-math.pi, math.pi, s.np_)
    e64 = orc.echo(s).astype(np.complex64)
    rc = orc.range_compress(s, e64.astype(np.complex128)).astype(np.complex64)
    r, g, lay = sarbp.scene_args(s)
    w = (rng.standard_normal((g.ny, g.nx)) + 1j * rng.standard_normal((g.ny, g.nx))).astype(np.complex64)
    ref = orc.project_weighted(s, rc, w, drange, dphase)
    out = plain.project_weighted(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, w,
                                 drange=drange, dphase=dphase)
    err = metrics.rel_l2_db(out, ref)
    img = plain.backproject(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate,
                            drange=drange, dphase=dphase)
    lhs = np.vdot(w.astype(np.complex128), img.astype(np.complex128))
    print(s.name, f"projection vs oracle {err:.1f} dB, adjoint mismatch {abs(lhs - out.sum()) / abs(lhs):.1e}")
    assert err <= -60.0
    assert abs(lhs - out.sum()) <= 1e-3 * abs(lhs)


def _plan(ctx, s, mode=sarbp.MODE_SPLIT):
    r, g, lay = sarbp.scene_args(s)
    v = sarbp.RcView()
    v.data, v.scale, v.storage, v.np, v.nbins = None, None, sarbp.STORE_C64, s.np_, lay.nbins
    v.t0_bins, v.bin_rate = lay.t0_bins, lay.bin_rate
    return ctx.bp_plan(r, v, s.apc, g, mode)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [3, 5, 11])
def test_linear_phase_form_on_large_tiles(orc, seed):
    """Tiles with half-diagonals beyond 12 m (0.61-1.46 m pixels): the series
    form's FP32 differential range costs phase accuracy in proportion to the
    tile's extent; the linear-term form (phase increments per pixel step
    reduced modulo 2 pi per pulse, FP32 only for the nonlinear remainder) does
    not.  The planner picks it there; forced either way, both stay within the
    -60 dB target and the linear-term form is at least 10 dB closer to the
    oracle."""
    s = random_scene(seed)
    e64 = orc.echo(s).astype(np.complex64)
    ref = orc.image(s, e64.astype(np.complex128))
    errs, forms = {}, {}
    for form in (-1, 1, 0):
        with sarbp.Context(0) as ctx:
            ctx.debug_set(sarbp.DEBUG_BP_LINEAR_PHASE, form)
            forms[form] = _plan(ctx, s).linear_phase
            errs[form] = metrics.rel_l2_db(sarbp.image_scene(ctx, s, e64, sarbp.MODE_SPLIT), ref)
    print(s.name, "series", f"{errs[-1]:.1f}", "linear-term", f"{errs[1]:.1f}", "planner", f"{errs[0]:.1f} dB")
    assert forms == {-1: 0, 1: 1, 0: 1}
    assert errs[-1] <= -60.0 and errs[1] <= -60.0
    assert errs[1] <= errs[-1] - 10.0
    assert errs[0] == errs[1]


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [3, 5, 11])
def test_linear_phase_form_in_the_projection(orc, seed):
    """The weighted projection takes the planner's phase form too: on tiles
    beyond 12 m the linear-term form is closer to the oracle's projection than
    the series form (GB300: -95 to -106 dB against -64 to -72 dB), both stay
    within -60 dB, and the adjoint identity with the back-projection of the
    same form holds to 1e-5 (the series form's, with its larger phase error, to
    1e-3)."""
    s = random_scene(seed)
    rng = np.random.default_rng(2900 + seed)
    e64 = orc.echo(s).astype(np.complex64)
    rc = orc.range_compress(s, e64.astype(np.complex128)).astype(np.complex64)
    r, g, lay = sarbp.scene_args(s)
    w = (rng.standard_normal((g.ny, g.nx)) + 1j * rng.standard_normal((g.ny, g.nx))).astype(np.complex64)
    zeros = np.zeros(s.np_)
    ref = orc.project_weighted(s, rc, w, zeros, zeros)
    errs, adj, forms = {}, {}, {}
    for form in (-1, 1, 0):
        with sarbp.Context(0) as ctx:
            ctx.debug_set(sarbp.DEBUG_BP_LINEAR_PHASE, form)
            forms[form] = _plan(ctx, s).linear_phase
            out = ctx.project_weighted(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, w)
            img = ctx.backproject(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate)
        errs[form] = metrics.rel_l2_db(out, ref)
        lhs = np.vdot(w.astype(np.complex128), img.astype(np.complex128))
        adj[form] = abs(lhs - out.sum()) / abs(lhs)
    print(s.name, "projection vs oracle: series", f"{errs[-1]:.1f}", "linear-term", f"{errs[1]:.1f}",
          "planner", f"{errs[0]:.1f} dB; adjoint mismatch", f"{adj[-1]:.1e} / {adj[1]:.1e}")
    assert forms == {-1: 0, 1: 1, 0: 1}
    assert errs[-1] <= -60.0 and errs[1] <= -60.0
    assert errs[1] <= errs[-1] - 20.0
    assert errs[0] == errs[1]
    assert adj[-1] <= 1e-3 and adj[1] <= 1e-5


@pytest.mark.gpu
def test_linear_phase_form_on_config2_tiles(orc):
    """Config 2's geometry (0.25 m pixels, 8.8 m half-diagonal tiles) keeps the
    series form; forced to the linear-term form it is at least as accurate."""
    s = scenes.config2(np_=512, n_img=256)
    s.targets = scenes.isolated_targets(s.grid, seed=21)
    e64 = orc.echo(s).astype(np.complex64)
    ref = orc.image(s, e64.astype(np.complex128))
    errs = {}
    for form in (0, 1):
        with sarbp.Context(0) as ctx:
            ctx.debug_set(sarbp.DEBUG_BP_LINEAR_PHASE, form)
            assert _plan(ctx, s).linear_phase == form
            errs[form] = metrics.rel_l2_db(sarbp.image_scene(ctx, s, e64, sarbp.MODE_SPLIT), ref)
    print("config-2 geometry: series", f"{errs[0]:.1f}", "linear-term", f"{errs[1]:.1f} dB")
    assert errs[0] <= -75.0 and errs[1] <= errs[0] + 1.0
