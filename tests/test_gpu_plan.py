"""Back-projection planning (sarbp_bp_plan): the geometry extremes the planner
sizes tiles and staging windows from are reduced on the device for the
one-shot calls and on the host for the serving loop; both must give the same
bits, so that a job plans (and rounds) the same either way.  Also: the
config-5 sub-aperture x tile launches keep two CTAs per SM with FP16 rows, and
a non-finite APC is rejected by both reductions."""
import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import sarbp, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sarbp.Context(0)
    yield c
    c.close()


def view(s, storage=sarbp.STORE_C64, np_=None):
    _, _, lay = sarbp.scene_args(s)
    v = sarbp.RcView()
    v.storage, v.np, v.nbins = storage, s.np_ if np_ is None else np_, lay.nbins
    v.t0_bins, v.bin_rate = lay.t0_bins, lay.bin_rate
    return v


def sub_grid(g, x0, y0, nx, ny):
    gs = sarbp.Grid()
    for i in range(3):
        gs.origin[i] = g.origin[i] + x0 * g.ux[i] + y0 * g.uy[i]
        gs.ux[i], gs.uy[i] = g.ux[i], g.uy[i]
    gs.nx, gs.ny = nx, ny
    return gs


def skewed_scene():
    s = scenes.config1(np_=512, ns=2048, n_img=300, spacing=0.5)
    g = s.grid
    g.uy = g.uy + 0.2 * g.ux  # non-orthogonal axes
    g.nx, g.ny = 301, 157
    return s


FIELDS = ("tile_x", "tile_y", "window", "series_terms", "segments", "ctas_per_sm", "pulse_chunk", "smem_bytes",
          "rmin", "rmax", "cos_x", "cos_y")


def plan_case(case):
    if case == "config2":
        s = scenes.config2()
        r, g, _ = sarbp.scene_args(s)
        apc, v = s.apc, view(s)
    elif case == "ground":
        s = scenes.ground_scene()
        r, g, _ = sarbp.scene_args(s)
        apc, v = s.apc, view(s)
    elif case == "skewed":
        s = skewed_scene()
        r, g, _ = sarbp.scene_args(s)
        apc, v = s.apc, view(s)
    else:
        s = scenes.config5()
        r, g0, _ = sarbp.scene_args(s)
        g = sub_grid(g0, 0, 0, 4096, 4096)
        apc, v = np.ascontiguousarray(s.apc[12288:]), view(s, sarbp.STORE_C32H, 4096)
    mode = sarbp.MODE_FP16STORE if v.storage == sarbp.STORE_C32H else sarbp.MODE_SPLIT
    return r, g, np.ascontiguousarray(apc, dtype=np.float64), v, mode


def brute_extremes(apc, g):
    """Every (pulse, lattice point) of the planner's 9 x 9 lattice, one IEEE
    operation at a time in the planner's order: range and the two direction
    cosines |axis.w| / (R |axis|) (numpy ufuncs round each operation and do not
    fuse multiply-adds)."""
    o, ux, uy = (np.array(x, dtype=np.float64) for x in (g.origin, g.ux, g.uy))
    dot = lambda a, b: (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]
    lux, luy = np.sqrt(dot(ux, ux)), np.sqrt(dot(uy, uy))
    k = np.arange(9)
    fx = ((g.nx - 1) * k).astype(np.float64) / 8.0
    fy = ((g.ny - 1) * k).astype(np.float64) / 8.0
    P = (o[None, None, :] + fx[:, None, None] * ux[None, None, :]) + fy[None, :, None] * uy[None, None, :]
    w = P[None, :, :, :] - apc[:, None, None, :]
    R = np.sqrt(dot(w, w))
    with np.errstate(divide="ignore", invalid="ignore"):
        cx = np.where(R > 0, np.abs(dot(ux, w)) / (R * lux), 0.0) if lux > 0 else np.zeros_like(R)
        cy = np.where(R > 0, np.abs(dot(uy, w)) / (R * luy), 0.0) if luy > 0 else np.zeros_like(R)
    return R.min(), R.max(), cx.max(), cy.max()


@pytest.mark.parametrize("case", ["config2", "ground", "skewed", "config5_corner"])
def test_extremes_equal_brute_force(ctx, case):
    """Both reductions skip the cosine divisions that a division-free
    comparison rules out and take the square root of the squared-range
    extremes; their results are the exact extremes of the per-point formula."""
    r, g, apc, v, mode = plan_case(case)
    want = brute_extremes(apc, g)
    for host in (False, True):
        info = ctx.bp_plan(r, v, apc, g, mode, host_reduction=host)
        got = (info.rmin, info.rmax, info.cos_x, info.cos_y)
        assert got == want, (host, got, want)


@pytest.mark.parametrize("case", ["config2", "ground", "skewed", "config5_corner"])
def test_host_and_device_extremes_agree(ctx, case):
    r, g, apc, v, mode = plan_case(case)
    dev = ctx.bp_plan(r, v, apc, g, mode)
    host = ctx.bp_plan(r, v, apc, g, mode, host_reduction=True)
    for f in FIELDS:
        assert getattr(dev, f) == getattr(host, f), f
    # device-resident APC: the same plan
    torch = pytest.importorskip("torch")
    d_apc = torch.from_numpy(np.ascontiguousarray(apc)).cuda()
    dev2 = ctx.bp_plan(r, v, d_apc, g, mode)
    for f in FIELDS:
        assert getattr(dev2, f) == getattr(dev, f), f
    assert dev.rmin < dev.rmax and 0 < dev.cos_x <= 1 and 0 <= dev.cos_y <= 1
    assert dev.window % 4 == 0 and dev.ctas_per_sm >= 1
    print(case, {f: getattr(dev, f) for f in FIELDS})


def test_config5_batches_keep_two_ctas(ctx):
    """The 16 sub-aperture (4096 pulses) x tile (4096^2) launches of config 5:
    windows of 92-140 bins, all at two resident CTAs per SM with FP16 rows."""
    s = scenes.config5()
    r, g, _ = sarbp.scene_args(s)
    wins = []
    for ty in (0, 4096):
        for tx in (0, 4096):
            gs = sub_grid(g, tx, ty, 4096, 4096)
            for p0 in range(0, s.np_, 4096):
                info = ctx.bp_plan(r, view(s, sarbp.STORE_C32H, 4096), np.ascontiguousarray(s.apc[p0:p0 + 4096]), gs,
                                   sarbp.MODE_FP16STORE)
                wins.append(info.window)
                assert info.ctas_per_sm >= 2, (tx, ty, p0, info.window, info.smem_bytes)
    assert max(wins) > 116  # wider than two complex64 CTAs would allow
    print("config 5 windows", sorted(wins))


def test_nonfinite_apc_rejected(ctx):
    s = scenes.config1(np_=64, ns=1024, n_img=32)
    r, g, _ = sarbp.scene_args(s)
    apc = s.apc.copy()
    apc[17, 1] = np.nan
    for host in (False, True):
        with pytest.raises(sarbp.SarbpError):
            ctx.bp_plan(r, view(s), apc, g, sarbp.MODE_SPLIT, host_reduction=host)


@pytest.mark.parametrize("case,storage,chunk", [("config1", sarbp.STORE_C64, 8), ("config1", sarbp.STORE_C32H, 16),
                                                 ("ground", sarbp.STORE_C64, 8), ("config2", sarbp.STORE_C64, 16)])
def test_wide_windows_keep_two_ctas(ctx, case, storage, chunk):
    """Windows past the two-CTA limit of 16-pulse chunks (config 1: 128 bins of
    complex64 at 0.5 m; the ground scene: 220 bins at 1 m) stage 8-pulse chunks."""
    s = {"config1": scenes.config1, "ground": scenes.ground_scene, "config2": scenes.config2}[case]()
    r, g, _ = sarbp.scene_args(s)
    mode = sarbp.MODE_FP16STORE if storage == sarbp.STORE_C32H else sarbp.MODE_SPLIT
    info = ctx.bp_plan(r, view(s, storage), s.apc, g, mode)
    print(case, info.window, info.pulse_chunk, info.ctas_per_sm, info.smem_bytes)
    assert info.pulse_chunk == chunk
    assert info.ctas_per_sm == 2


@pytest.mark.parametrize("form", [-1, 1], ids=["series", "linear"])
@pytest.mark.parametrize("storage", [sarbp.STORE_C64, sarbp.STORE_C32H])
def test_chunk_size_does_not_change_results(ctx, storage, form):
    """Pixels accumulate pulses in the same order whatever the staging chunk, so
    16-, 8- and 4-pulse chunks give the same bits (back-projection and the
    weighted projection, in both phase forms, 16-pulse chunks compiled in; 300
    pulses: ragged last chunks)."""
    s = scenes.config1(np_=300, ns=1024, n_img=96)
    r, g, lay = sarbp.scene_args(s)
    echo = sarbp.synthesize(ctx, s)
    rc = ctx.range_compress(r, echo, storage=storage)
    data, scale = rc if storage == sarbp.STORE_C32H else (rc, None)
    mode = sarbp.MODE_FP16STORE if storage == sarbp.STORE_C32H else sarbp.MODE_SPLIT
    w = (np.random.default_rng(4).standard_normal((g.ny, g.nx)) + 0j).astype(np.complex64)
    imgs, projs = {}, {}
    try:
        ctx.debug_set(sarbp.DEBUG_BP_LINEAR_PHASE, form)
        for c in ("16", "8", "4"):
            ctx.debug_set(sarbp.DEBUG_BP_CHUNK, int(c))
            info = ctx.bp_plan(r, view(s, storage), s.apc, g, mode)
            assert info.pulse_chunk == int(c) and info.linear_phase == (1 if form > 0 else 0)
            imgs[c] = ctx.backproject(r, data, s.apc, g, mode, lay.t0_bins, lay.bin_rate, scale=scale)
            projs[c] = ctx.project_weighted(r, data, s.apc, g, mode, lay.t0_bins, lay.bin_rate, w, scale=scale)
    finally:
        ctx.debug_set(sarbp.DEBUG_BP_CHUNK, 0)
        ctx.debug_set(sarbp.DEBUG_BP_LINEAR_PHASE, 0)
    for c in ("8", "4"):
        assert np.array_equal(imgs[c], imgs["16"])
        assert np.array_equal(projs[c], projs["16"])
    assert np.abs(imgs["16"]).max() > 0


def test_wide_coarse_grid_plans_and_matches_fp64(ctx):
    """A 4 km-wide range extent at 1 m pixels from 5 km range: the series bound
    taken at the nearest tile centre admits 32 x 32 tiles with 4 terms (the
    bound at the farthest range rejected every tile), the window (236 bins, past
    the 116-bin two-CTA limit of 16-pulse chunks) stages 8-pulse chunks at two
    CTAs per SM, and the near-range corner (largest
    relative tile size) matches the FP64 mode within -65 dB."""
    radar = scenes.Radar()
    grid = scenes.centred_grid(radar, 4096, 256, 1.0)
    s = scenes.Scene(name="coarse", radar=radar, np_=512, ns=8192, apc=scenes.straight_track(radar, 512), grid=grid,
                     targets=scenes.random_targets(grid, 50, 3), t_rec0=scenes.centred_record_start(radar, 8192),
                     snr_db=None, seed=3)
    r, g, lay = sarbp.scene_args(s)
    info = ctx.bp_plan(r, view(s), s.apc, g, sarbp.MODE_SPLIT)
    assert (info.tile_x, info.tile_y, info.series_terms) == (32, 32, 4)
    print("coarse grid plan", info.window, info.pulse_chunk, info.ctas_per_sm)
    assert info.window > 116 and info.pulse_chunk in (8, 4) and info.ctas_per_sm == 2
    rc = ctx.range_compress(r, sarbp.synthesize(ctx, s))
    img = ctx.backproject(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate)
    corner = sub_grid(g, 0, 0, 256, 256)
    ref = ctx.backproject(r, rc, s.apc, corner, sarbp.MODE_FP64, lay.t0_bins, lay.bin_rate)
    err = 20 * np.log10(np.linalg.norm(img[:256, :256] - ref) / np.linalg.norm(ref))
    print("coarse grid near-range corner rel-L2 dB", err)
    assert err <= -65.0


def expected_segments(tiles, npl, npix, sms):
    """The planner's rule restated: the fewest segments giving 12 waves of CTAs
    (two per SM), at least 64 pulses per segment, no empty segment, partial
    images within 1 GiB."""
    best = 1
    for s in range(1, 65):
        if s > 1 and (npl // s < 64 or s * npix * 8 > 2 ** 30):
            break
        n = (npl + s - 1) // s
        pps = (n + 15) // 16 * 16
        if s > 1 and (s - 1) * pps >= npl:
            continue
        best = s
        if tiles * s >= 12 * 2 * sms:
            break
    return best


@pytest.mark.parametrize("n_img,np_", [(4096, 4096), (2048, 4096), (1024, 4096), (512, 512), (256, 100)])
def test_segments_fill_waves(ctx, n_img, np_):
    """Pulse segments follow the 12-wave rule: config 2 keeps one segment, a
    1024^2 image of 4096 pulses on 152 SMs takes 8, short apertures stop at 64
    pulses per segment."""
    torch = pytest.importorskip("torch")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    s = scenes.config2(n_img=n_img) if np_ == 4096 else scenes.config1(np_=np_, ns=1024, n_img=n_img)
    r, g, _ = sarbp.scene_args(s)
    info = ctx.bp_plan(r, view(s), s.apc, g, sarbp.MODE_SPLIT)
    tiles = ((g.nx + info.tile_x - 1) // info.tile_x) * ((g.ny + info.tile_y - 1) // info.tile_y)
    assert info.segments == expected_segments(tiles, np_, g.nx * g.ny, sms)
    if sms == 152:
        assert info.segments == {4096: 1, 2048: 2, 1024: 8, 512: 8, 256: 1}[n_img]


def test_forced_segments_agree(ctx):
    """Segment counts only regroup the per-pixel pulse sums: 1, 3 and 7
    segments (uneven last segments) agree with the planner's choice to FP32
    rounding.  The weighted projection sums each pulse inside one CTA per tile
    whatever the segments, so it is bit-identical."""
    s = scenes.config1(np_=700, ns=1024, n_img=128)
    r, g, lay = sarbp.scene_args(s)
    rc = ctx.range_compress(r, sarbp.synthesize(ctx, s))
    w = (np.random.default_rng(9).standard_normal((g.ny, g.nx)) + 0j).astype(np.complex64)
    auto = ctx.bp_plan(r, view(s), s.apc, g, sarbp.MODE_SPLIT).segments
    ref = ctx.backproject(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate)
    pref = ctx.project_weighted(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, w)
    try:
        for n in ("1", "3", "7"):
            ctx.debug_set(sarbp.DEBUG_BP_SEGMENTS, int(n))
            assert ctx.bp_plan(r, view(s), s.apc, g, sarbp.MODE_SPLIT).segments == int(n)
            img = ctx.backproject(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate)
            prj = ctx.project_weighted(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, w)
            err = 20 * np.log10(np.linalg.norm(img - ref) / np.linalg.norm(ref))
            print("segments", n, "vs", auto, "image rel-L2 dB", err)
            assert err <= -110.0
            assert np.array_equal(prj, pref)
    finally:
        ctx.debug_set(sarbp.DEBUG_BP_SEGMENTS, 0)
