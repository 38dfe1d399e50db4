"""GPU parity of the omega-K imager and its batched DFT against FP64 numpy /
the omega-K oracle (oracle/wk.py).

Tolerances (relative L2): DFT <= -110 dB (FP32 transforms of up to 16384
points); omega-K image <= -80 dB against the FP64 restatement (FP32 FFTs, FP64
phases, FP32 Stolt weights)."""
import os

import numpy as np
import pytest

from oracle import wk
from sar_cambrianaccelerationcard_gb300 import metrics, sarbp

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "wk_cd_crop.npz")


@pytest.fixture(scope="module")
def ctx():
    c = sarbp.Context(0)
    yield c
    c.close()


def rand(shape, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize("n", [2, 8, 64, 512, 4096, 16384, 3, 5, 7, 100, 106, 214, 854, 1000, 3414, 8191])
def test_dft_rows(ctx, n):
    rows = max(1, min(64, 65536 // n))
    x = rand((rows, n), n)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    got = ctx.dft(x.copy())
    err = metrics.rel_l2_db(got, ref)
    back = ctx.dft(got.copy(), inverse=True)
    err_inv = metrics.rel_l2_db(back, x.astype(np.complex128))
    print(f"dft n {n}: forward {err:.1f} dB, round trip {err_inv:.1f} dB")
    assert err <= -110.0
    assert err_inv <= -110.0


def test_dft_rejects_unsupported(ctx):
    with pytest.raises(sarbp.SarbpError):
        ctx.dft(np.zeros((2, 8193), dtype=np.complex64))


def test_wk_golden_crop(ctx):
    """The reference's RADARSAT-1 echo (96 x 64 crop): GPU against the FP64 image."""
    g = np.load(GOLDEN)
    img = ctx.wk_image(wk.radarsat1(), g["echo"])
    err = metrics.rel_l2_db(img, g["image"])
    print("wk golden crop rel-L2 dB", err)
    assert img.shape == (128, 106)
    assert err <= -80.0


@pytest.mark.parametrize("shape,taps", [((768, 512), 6), ((300, 200), 6), ((128, 96), 5), ((64, 256), 8)])
def test_wk_matches_oracle(ctx, shape, taps):
    p = wk.radarsat1()
    p.taps = taps
    echo = rand(shape, 7 + taps)
    ref = wk.wk_image(echo.astype(np.complex128), p)
    img = ctx.wk_image(p, echo)
    err = metrics.rel_l2_db(img, ref)
    print(f"wk {shape} taps {taps} rel-L2 dB {err:.1f}")
    assert err <= -80.0


def test_wk_fp64_stolt_path(ctx):
    """An airborne L-band case (f0 1.3 GHz, Vr 120 m/s, zero Doppler centroid):
    the mapping is no longer a small correction (c^2 fa^2 / (4 Vr^2) up to 0.4 of
    (f0 + fr)^2), so the Stolt stage runs in FP64."""
    p = wk.WkParams(fr=100e6, prf=1000.0, f0=1.3e9, r0=3000.0, kr=5e12, vr=120.0, f_nc=0.0)
    echo = rand((192, 160), 21)
    ref = wk.wk_image(echo.astype(np.complex128), p)
    img = ctx.wk_image(p, echo)
    err = metrics.rel_l2_db(img, ref)
    print("wk fp64 stolt rel-L2 dB", err)
    assert err <= -80.0


def test_wk_tables_follow_parameters(ctx):
    """The omega-K tables are built once per (parameters, padded size) and
    reused: alternating two parameter sets and two sizes on one context, and
    trimming its buffers in between, gives each call the image a fresh
    context gives."""
    a = wk.radarsat1()
    b = wk.WkParams(fr=100e6, prf=1000.0, f0=1.3e9, r0=3000.0, kr=5e12, vr=120.0, f_nc=0.0)
    e1, e2 = rand((192, 128), 31), rand((160, 96), 32)
    fresh = sarbp.Context(0)
    try:
        want = {(k, i): fresh.wk_image(p, e) for k, p in (("a", a), ("b", b)) for i, e in ((1, e1), (2, e2))}
    finally:
        fresh.close()
    order = [("a", 1), ("a", 1), ("b", 1), ("a", 1), ("a", 2), ("b", 2), ("trim", 0), ("b", 2), ("a", 1)]
    for k, i in order:
        if k == "trim":
            ctx.check(ctx.lib.sarbp_trim(ctx.h), "trim")
            continue
        img = ctx.wk_image(a if k == "a" else b, e1 if i == 1 else e2)
        assert np.array_equal(img, want[(k, i)]), (k, i)


def test_wk_device_pointers(ctx):
    torch = pytest.importorskip("torch")
    p = wk.radarsat1()
    echo = rand((192, 128), 3)
    host = ctx.wk_image(p, echo)
    NA, NR, _ = ctx.wk_padded_size(192, 128)
    d_echo = torch.from_numpy(echo.view(np.float32)).cuda()
    d_img = torch.empty((NA, NR * 2), dtype=torch.float32, device="cuda")
    w = sarbp.wk_params(p)
    ctx.check(ctx.lib.sarbp_wk_image(ctx.h, sarbp.ctypes.byref(w), d_echo.data_ptr(), 192, 128, d_img.data_ptr(), None),
              "wk device")
    ctx.synchronize()
    dev = d_img.cpu().numpy().view(np.complex64)
    assert np.array_equal(dev, host)


def test_wk_rejects_bad_arguments(ctx):
    p = wk.radarsat1()
    with pytest.raises(sarbp.SarbpError):
        q = wk.radarsat1()
        q.taps = 0
        ctx.wk_image(q, rand((64, 64), 1))
    with pytest.raises(sarbp.SarbpError):
        q = wk.radarsat1()
        q.prf = float("nan")
        ctx.wk_image(q, rand((64, 64), 1))
    with pytest.raises(sarbp.SarbpError):  # padded range size 10924 > 8192 and not a power of two
        ctx.wk_image(p, rand((8, 6554), 1))


@pytest.mark.parametrize("shape", [(1024, 854), (4096, 96), (512, 512), (300, 200), (100, 64), (64, 33), (1, 7), (7, 1)])
def test_dft2d(ctx, shape):
    """sarbp_dft2d (perform2DFFT / perform2DIFFT): against numpy fft2 / ifft2 in
    FP64, both the column kernel (power-of-two column lengths 512..4096) and the
    transpose path."""
    x = rand(shape, shape[0] * 7 + shape[1])
    ref = np.fft.fft2(x.astype(np.complex128))
    got = ctx.dft2d(x.copy())
    assert metrics.rel_l2_db(got, ref) <= -105.0
    back = ctx.dft2d(got.copy(), inverse=True)
    assert metrics.rel_l2_db(back, x.astype(np.complex128)) <= -105.0
    assert metrics.rel_l2_db(ctx.dft2d(ref.astype(np.complex64), inverse=True), x.astype(np.complex128)) <= -105.0


@pytest.mark.parametrize("shape", [(768, 512), (300, 200)])
def test_wk_stages_match_oracle_and_pipeline(ctx, shape):
    """preprocess -> dft2d -> focus -> inverse dft2d: each stage against its FP64
    restatement, and the staged result bit-identical to sarbp_wk_image (the same
    kernels on the same values)."""
    p = wk.radarsat1()
    echo = rand(shape, 31)
    x = ctx.wk_preprocess(p, echo)
    x_ref = wk.pad_downconvert(echo.astype(np.complex128), p)
    assert metrics.rel_l2_db(x, x_ref) <= -130.0
    S = ctx.dft2d(x.copy())
    F = ctx.wk_focus(p, S)
    F_ref = wk.rfm_stolt(S.astype(np.complex128), p)
    assert metrics.rel_l2_db(F, F_ref) <= -80.0
    img = ctx.dft2d(F.copy(), inverse=True)
    assert np.array_equal(img, ctx.wk_image(p, echo))
    assert metrics.rel_l2_db(img, wk.wk_image(echo.astype(np.complex128), p)) <= -80.0


def test_stage_entry_points_device_pointers_and_errors(ctx):
    """Device-resident buffers give the host path's bits (sarbp_dft2d in place,
    sarbp_wk_focus in place as documented); invalid arguments return a status."""
    torch = pytest.importorskip("torch")
    p = wk.radarsat1()
    echo = rand((192, 128), 5)
    NA, NR, _ = ctx.wk_padded_size(192, 128)
    host_x = ctx.wk_preprocess(p, echo)
    w = sarbp.wk_params(p)
    d_echo = torch.from_numpy(echo.view(np.float32)).cuda()
    d_x = torch.empty((NA, NR * 2), dtype=torch.float32, device="cuda")
    ctx.check(ctx.lib.sarbp_wk_preprocess(ctx.h, sarbp.ctypes.byref(w), d_echo.data_ptr(), 192, 128, d_x.data_ptr(),
                                          None), "preprocess device")
    ctx.check(ctx.lib.sarbp_dft2d(ctx.h, d_x.data_ptr(), NA, NR, 0, None), "dft2d device")
    ctx.check(ctx.lib.sarbp_wk_focus(ctx.h, sarbp.ctypes.byref(w), d_x.data_ptr(), NA, NR, d_x.data_ptr(), None),
              "focus in place")
    ctx.synchronize()
    host_f = ctx.wk_focus(p, ctx.dft2d(host_x.copy()))
    assert np.array_equal(d_x.cpu().numpy().view(np.complex64), host_f)
    with pytest.raises(sarbp.SarbpError):
        ctx.dft2d(np.zeros((0, 8), dtype=np.complex64))
    with pytest.raises(sarbp.SarbpError):
        ctx.dft2d(np.zeros((4, 8193), dtype=np.complex64))  # 8193 is neither a power of two nor <= 8192
    q = wk.radarsat1()
    q.vr = float("nan")
    with pytest.raises(sarbp.SarbpError):
        ctx.wk_preprocess(q, echo)
    with pytest.raises(sarbp.SarbpError):
        ctx.wk_focus(p, np.zeros((8, 40000), dtype=np.complex64))  # Stolt row too large for shared memory
