"""GPU parity: the CUDA path (through the C ABI) against the FP64 oracle on
config-1 scenes (512 pulses x 1024 samples, 3x3 targets, 30 dB SNR).

Tolerances (relative L2, 20 log10 ||gpu - oracle|| / ||oracle||):
  range compression, complex64 storage   <= -110 dB  (FP32 FFT vs FP64)
  range compression, FP16 storage        <= -60 dB   (11-bit significand)
  back-projection SPLIT / FP16STORE      <= -60 dB   (the imaging target)
  back-projection FP64                   <= -100 dB  (complex64 data and output)
  point targets: peak position within 0.05 px, PSLR and ISLR within 0.1 dB.
"""
import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import metrics, sarbp, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sarbp.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def c1(orc):
    scene = scenes.config1()
    echo = orc.echo(scene)                    # FP64 echo with noise
    echo64 = echo.astype(np.complex64)        # what the GPU gets
    rc = orc.range_compress(scene, echo64.astype(np.complex128))
    img = orc.backproject(scene, rc)
    return dict(scene=scene, echo=echo64, rc=rc, img=img)


def test_range_compression_c64(ctx, c1):
    s = c1["scene"]
    r, g, lay = sarbp.scene_args(s)
    rc = ctx.range_compress(r, c1["echo"])
    err = metrics.rel_l2_db(rc, c1["rc"])
    print("rc c64 rel-L2 dB", err)
    assert rc.shape == (s.np_, lay.nbins)
    assert err <= -110.0


def test_range_compression_fp16(ctx, c1):
    s = c1["scene"]
    r, g, lay = sarbp.scene_args(s)
    h, scale = ctx.range_compress(r, c1["echo"], storage=sarbp.STORE_C32H)
    assert h.shape == (s.np_, lay.nbins, 2)
    m, e = np.frexp(scale)
    assert np.all(m == 0.5), "scales are powers of two"
    assert np.abs(h.astype(np.float32)).max() <= 2.0 ** 14
    rc = (h[..., 0].astype(np.float64) + 1j * h[..., 1].astype(np.float64)) * scale[:, None]
    err = metrics.rel_l2_db(rc, c1["rc"])
    print("rc fp16 rel-L2 dB", err)
    assert err <= -60.0


@pytest.mark.parametrize("mode,tol", [("split", -60.0), ("fp64", -100.0)])
def test_backprojection_on_oracle_data(ctx, orc, c1, mode, tol):
    """BP stage alone: both sides back-project the same complex64 rc data."""
    s = c1["scene"]
    r, g, lay = sarbp.scene_args(s)
    rc32 = c1["rc"].astype(np.complex64)
    ref = orc.backproject(s, rc32)
    img = ctx.backproject(r, rc32, s.apc, g, sarbp.MODES[mode], lay.t0_bins, lay.bin_rate)
    err = metrics.rel_l2_db(img, ref)
    print(mode, "bp rel-L2 dB", err, "bp ms", ctx.timings()[1])
    assert err <= tol


def test_backprojection_fp32_is_worse_than_split(ctx, orc, c1):
    """Plain FP32 (absolute ranges in FP32) is the accuracy comparator: it must
    still focus, and it is expected to miss the -60 dB target."""
    s = c1["scene"]
    r, g, lay = sarbp.scene_args(s)
    rc32 = c1["rc"].astype(np.complex64)
    ref = orc.backproject(s, rc32)
    img = ctx.backproject(r, rc32, s.apc, g, sarbp.MODE_FP32, lay.t0_bins, lay.bin_rate)
    err = metrics.rel_l2_db(img, ref)
    print("fp32 bp rel-L2 dB", err)
    assert err < 0.0
    pk = np.unravel_index(np.argmax(np.abs(img)), img.shape)
    assert any(abs(pk[0] - y) <= 1 and abs(pk[1] - x) <= 1 for (x, y) in metrics.target_pixels(s))


@pytest.mark.parametrize("mode", ["split", "fp16store"])
def test_full_chain_c1_c3(ctx, c1, mode):
    """Config 1 (SPLIT) and config 3 (FP16 storage): echo in, image out, vs oracle."""
    s = c1["scene"]
    img = sarbp.image_scene(ctx, s, c1["echo"], sarbp.MODES[mode])
    err = metrics.rel_l2_db(img, c1["img"])
    cmp = metrics.compare_point_targets(img, c1["img"], metrics.target_pixels(s))
    print(mode, "image rel-L2 dB", err, "shift", cmp["peak_shift_px"], "pslr", cmp["pslr_diff_db"],
          "islr", cmp["islr_diff_db"])
    assert err <= -60.0
    assert cmp["peak_shift_px"] <= 0.05
    assert cmp["pslr_diff_db"] <= 0.1
    assert cmp["islr_diff_db"] <= 0.1


def test_synthesiser_matches_oracle(ctx, orc):
    s = scenes.config1(np_=64, ns=1024)
    gpu = sarbp.synthesize(ctx, s)
    ref = orc.echo(s)
    err = metrics.rel_l2_db(gpu, ref)
    print("synth rel-L2 dB", err)
    assert err <= -120.0
    clean = ctx.synthesize_echo(sarbp.radar_struct(s.radar, s.t_rec0), s.apc, s.ns, s.targets, None)
    assert metrics.rel_l2_db(clean, orc.echo(s, noise=False)) <= -120.0


def test_ragged_sizes(ctx, orc):
    """Grid not a multiple of the tile, ns not a power of two, odd pulse count."""
    s = scenes.config1(np_=77, ns=1000, n_img=10)
    s.grid = scenes.centred_grid(s.radar, 45, 71, 0.5)
    echo = orc.echo(s).astype(np.complex64)
    ref = orc.image(s, echo.astype(np.complex128))
    img = sarbp.image_scene(ctx, s, echo, sarbp.MODE_SPLIT)
    assert img.shape == (71, 45)
    assert metrics.rel_l2_db(img, ref) <= -60.0


def test_empty_inputs(ctx):
    s = scenes.config1(np_=16, ns=256, n_img=32)
    r, g, lay = sarbp.scene_args(s)
    img = np.full((32, 32), 7 + 7j, dtype=np.complex64)
    out = ctx.backproject(r, np.zeros((0, lay.nbins), np.complex64), np.zeros((0, 3)), g, sarbp.MODE_SPLIT,
                          lay.t0_bins, lay.bin_rate, image=img)
    assert np.all(out == 0)
    g0 = sarbp.grid_struct(scenes.centred_grid(s.radar, 0, 0, 0.5))
    ctx.backproject(r, np.zeros((16, lay.nbins), np.complex64), s.apc, g0, sarbp.MODE_SPLIT, lay.t0_bins,
                    lay.bin_rate, image=np.zeros((0, 0), np.complex64))


def test_accumulate_is_linear_over_subapertures(ctx, c1):
    s = c1["scene"]
    r, g, lay = sarbp.scene_args(s)
    rc32 = np.ascontiguousarray(c1["rc"].astype(np.complex64))
    full = ctx.backproject(r, rc32, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate)
    k = 200
    part = ctx.backproject(r, np.ascontiguousarray(rc32[:k]), np.ascontiguousarray(s.apc[:k]), g,
                           sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate)
    part = ctx.backproject(r, np.ascontiguousarray(rc32[k:]), np.ascontiguousarray(s.apc[k:]), g,
                           sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, image=part, accumulate=True)
    assert metrics.rel_l2_db(part, full) <= -110.0


def test_invalid_arguments(ctx, c1):
    s = c1["scene"]
    r, g, lay = sarbp.scene_args(s)
    rc32 = c1["rc"].astype(np.complex64)
    with pytest.raises(sarbp.SarbpError) as e:
        ctx.backproject(r, rc32, s.apc, g, 9, lay.t0_bins, lay.bin_rate)
    assert e.value.status == sarbp.ERR_INVALID_ARGUMENT
    with pytest.raises(sarbp.SarbpError) as e:
        ctx.backproject(r, rc32, s.apc, g, sarbp.MODE_FP16STORE, lay.t0_bins, lay.bin_rate)
    assert e.value.status == sarbp.ERR_INVALID_ARGUMENT
    with pytest.raises(sarbp.SarbpError) as e:
        ctx.backproject(r, np.ascontiguousarray(rc32[:, :-2]), s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins,
                        lay.bin_rate)
    assert e.value.status == sarbp.ERR_UNSUPPORTED
    bad = s.apc.copy()
    bad[3, 1] = np.nan
    with pytest.raises(sarbp.SarbpError) as e:
        ctx.backproject(r, rc32, bad, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate)
    assert e.value.status == sarbp.ERR_INVALID_ARGUMENT
    with pytest.raises(sarbp.SarbpError) as e:   # range FFT beyond 32768 points
        ctx.range_compress(r, np.zeros((2, 40000), np.complex64))
    assert e.value.status == sarbp.ERR_UNSUPPORTED
    # the context stays usable after errors
    img = ctx.backproject(r, rc32[:8].copy(), s.apc[:8].copy(), g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate)
    assert np.isfinite(img).all()


def test_device_pointer_path(ctx, c1):
    """Device-resident buffers (torch CUDA tensors): asynchronous call on a stream."""
    torch = pytest.importorskip("torch")
    s = c1["scene"]
    r, g, lay = sarbp.scene_args(s)
    host = sarbp.image_scene(ctx, s, c1["echo"], sarbp.MODE_SPLIT)
    echo = torch.from_numpy(c1["echo"].view(np.float32)).cuda()
    apc = torch.from_numpy(s.apc).cuda()
    img = torch.zeros((g.ny, g.nx * 2), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        ctx.check(ctx.lib.sarbp_image(ctx.h, sarbp.ctypes.byref(r), echo.data_ptr(), s.np_, s.ns, apc.data_ptr(),
                                      sarbp.ctypes.byref(g), sarbp.MODE_SPLIT, img.data_ptr(),
                                      sarbp.ctypes.c_void_p(stream.cuda_stream)), "image")
    stream.synchronize()
    ctx.synchronize()
    dev = img.cpu().numpy().view(np.complex64)
    assert np.array_equal(dev, host)


def test_reference_shim_default_params_give_zero_image(ctx):
    """The reference program's own scene (SARParams defaults, BPA_CUDA.cpp:26-48)
    produces an all-zero echo: targets at ~11.2 km delay 74.5 us, far past the
    2.5 us record.  Through the shim the image is all-zero as well, as the
    reference's own output is."""
    torch = pytest.importorskip("torch")
    p = sarbp.RefParams.defaults()
    M, N = p.Mslow, p.Nfast
    ptarget = torch.tensor([p.Az0 - 10, p.Rg0 - 20, 1.0, p.Az0 + 20, p.Rg0 + 30, 0.8, p.Az0 - 30, p.Rg0 + 10, 1.2,
                            p.Az0 + 40, p.Rg0 - 40, 0.9, p.Az0, p.Rg0, 1.5], dtype=torch.float32, device="cuda")
    ta = torch.linspace(-p.La / (2 * p.vr), p.La / (2 * p.vr), M, dtype=torch.float32, device="cuda")
    tr = torch.arange(N, dtype=torch.float32, device="cuda") / p.Fr
    srnm = torch.zeros((M, N * 2), dtype=torch.float32, device="cuda")
    lib = sarbp.load()
    assert lib.sarbp_launch_generate_echo(srnm.data_ptr(), ptarget.data_ptr(), ta.data_ptr(), tr.data_ptr(),
                                          sarbp.ctypes.byref(p), M, N) == 0
    assert float(srnm.abs().max()) == 0.0
    image = torch.full((M, N * 2), 3.0, dtype=torch.float32, device="cuda")
    assert lib.sarbp_launch_back_projection(srnm.data_ptr(), image.data_ptr(), sarbp.ctypes.byref(p), M, N) == 0
    assert float(image.abs().max()) == 0.0


def test_ground_geometry_coarse_pixels(ctx, orc):
    """Antenna at 5 km altitude, 1 m ground pixels (the reference program's
    geometry): the planner picks shorter tiles; still within -60 dB."""
    s = scenes.ground_scene()
    echo = orc.echo(s).astype(np.complex64)
    ref = orc.image(s, echo.astype(np.complex128))
    for mode in ("split", "fp16store"):
        img = sarbp.image_scene(ctx, s, echo, sarbp.MODES[mode])
        err = metrics.rel_l2_db(img, ref)
        print("ground", mode, err)
        assert err <= -60.0


@pytest.mark.parametrize("storage", [sarbp.STORE_C64, sarbp.STORE_C32H])
def test_chunked_host_upload_is_bit_exact(ctx, storage):
    """A host echo is uploaded in pulse chunks (2500 pulses: 8 chunks of 313,
    the last 309) overlapped with range compression; rows and FP16 scales equal
    those from a device-resident echo, and so does the image."""
    torch = pytest.importorskip("torch")
    s = scenes.config1(np_=2500, ns=1024, n_img=128)
    r, g, lay = sarbp.scene_args(s)
    rng = np.random.default_rng(9)
    echo = (rng.standard_normal((s.np_, s.ns)) + 1j * rng.standard_normal((s.np_, s.ns))).astype(np.complex64)
    host = ctx.range_compress(r, echo, storage=storage)
    d_echo = torch.from_numpy(echo.view(np.float32)).cuda()
    esize = 8 if storage == sarbp.STORE_C64 else 4
    d_rc = torch.empty((s.np_, lay.nbins * esize // 4), dtype=torch.float32, device="cuda")
    d_scale = torch.empty(s.np_, dtype=torch.float32, device="cuda")
    ctx.check(ctx.lib.sarbp_range_compress(ctx.h, sarbp.ctypes.byref(r), d_echo.data_ptr(), s.np_, s.ns, storage,
                                           d_rc.data_ptr(), d_scale.data_ptr() if storage == sarbp.STORE_C32H else None,
                                           None), "rc device")
    ctx.synchronize()
    if storage == sarbp.STORE_C64:
        assert np.array_equal(d_rc.cpu().numpy().view(np.complex64), host)
    else:
        h, scale = host
        assert np.array_equal(d_rc.cpu().numpy().view(np.float16).reshape(h.shape), h)
        assert np.array_equal(d_scale.cpu().numpy(), scale)
    mode = sarbp.MODE_SPLIT if storage == sarbp.STORE_C64 else sarbp.MODE_FP16STORE
    img_host = sarbp.image_scene(ctx, s, echo, mode)
    img_dev = torch.zeros((g.ny, g.nx * 2), dtype=torch.float32, device="cuda")
    apc = torch.from_numpy(s.apc).cuda()
    ctx.check(ctx.lib.sarbp_image(ctx.h, sarbp.ctypes.byref(r), d_echo.data_ptr(), s.np_, s.ns, apc.data_ptr(),
                                  sarbp.ctypes.byref(g), mode, img_dev.data_ptr(), None), "image device")
    ctx.synchronize()
    assert np.array_equal(img_dev.cpu().numpy().view(np.complex64), img_host)


def test_pinned_host_image_written_in_place(ctx, c1):
    """A pinned (device-mapped) host image is written by the back-projection
    itself, with no download: same bits as the device-buffer path; with no
    pulses the image is cleared."""
    torch = pytest.importorskip("torch")
    s = c1["scene"]
    r, g, lay = sarbp.scene_args(s)
    ref = sarbp.image_scene(ctx, s, c1["echo"], sarbp.MODE_SPLIT)  # pageable: downloaded
    pinned = torch.full((g.ny, g.nx * 2), 7.0, dtype=torch.float32, pin_memory=True)
    echo = torch.from_numpy(c1["echo"].view(np.float32)).pin_memory()
    ctx.check(ctx.lib.sarbp_image(ctx.h, sarbp.ctypes.byref(r), echo.data_ptr(), s.np_, s.ns, s.apc.ctypes.data,
                                  sarbp.ctypes.byref(g), sarbp.MODE_SPLIT, pinned.data_ptr(), None), "image pinned")
    assert np.array_equal(pinned.numpy().view(np.complex64), ref)
    ctx.check(ctx.lib.sarbp_image(ctx.h, sarbp.ctypes.byref(r), echo.data_ptr(), 0, s.ns, s.apc.ctypes.data,
                                  sarbp.ctypes.byref(g), sarbp.MODE_SPLIT, pinned.data_ptr(), None), "image np=0")
    assert not pinned.numpy().any()


def test_error_after_upload_leaves_nothing_in_flight(ctx, c1):
    """A grid the planner cannot serve (on top of the flight track) fails after
    the echo upload and range compression were queued; the call returns the
    status with no copy left reading the caller's pinned echo, and the context
    stays usable."""
    torch = pytest.importorskip("torch")
    s = c1["scene"]
    r, g, lay = sarbp.scene_args(s)
    echo = torch.from_numpy(c1["echo"].view(np.float32)).pin_memory()
    bad = sarbp.scene_args(s)[1]
    for i in range(3):
        bad.origin[i] = float(s.apc[s.np_ // 2][i]) - 0.5 * (bad.nx * bad.ux[i] + bad.ny * bad.uy[i])
    img = np.zeros((bad.ny, bad.nx), dtype=np.complex64)
    with pytest.raises(sarbp.SarbpError) as ex:
        ctx.check(ctx.lib.sarbp_image(ctx.h, sarbp.ctypes.byref(r), echo.data_ptr(), s.np_, s.ns, s.apc.ctypes.data,
                                      sarbp.ctypes.byref(bad), sarbp.MODE_SPLIT, img.ctypes.data, None), "image")
    assert ex.value.status == sarbp.ERR_UNSUPPORTED
    del echo  # the caller may release its buffer right after the error
    again = sarbp.image_scene(ctx, s, c1["echo"], sarbp.MODE_SPLIT)
    assert np.array_equal(again, sarbp.image_scene(ctx, s, c1["echo"], sarbp.MODE_SPLIT))


def test_nonfinite_apc_fails_after_upload_is_queued(ctx, c1):
    """sarbp_image queues the echo upload and range compression before it waits
    for the planning extremes; a non-finite APC is found there and returns
    SARBP_ERR_INVALID_ARGUMENT with no copy left reading the caller's pinned
    echo, and the context stays usable."""
    torch = pytest.importorskip("torch")
    s = c1["scene"]
    r, g, _ = sarbp.scene_args(s)
    echo = torch.from_numpy(c1["echo"].view(np.float32)).pin_memory()
    bad = s.apc.copy()
    bad[s.np_ // 3, 0] = np.inf
    img = np.zeros((g.ny, g.nx), dtype=np.complex64)
    with pytest.raises(sarbp.SarbpError) as ex:
        ctx.check(ctx.lib.sarbp_image(ctx.h, sarbp.ctypes.byref(r), echo.data_ptr(), s.np_, s.ns, bad.ctypes.data,
                                      sarbp.ctypes.byref(g), sarbp.MODE_SPLIT, img.ctypes.data, None), "image")
    assert ex.value.status == sarbp.ERR_INVALID_ARGUMENT
    del echo
    again = sarbp.image_scene(ctx, s, c1["echo"], sarbp.MODE_SPLIT)
    assert np.isfinite(again).all() and np.abs(again).max() > 0
