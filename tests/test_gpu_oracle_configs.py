"""The CUDA path against the FP64 CPU oracle at the geometries of the larger
workloads, reduced so the oracle finishes in seconds (BPA_SAR.m:80-111,
177-197 restated in oracle/):

  * config 2's radar and track (4096 pulses x 8192 samples, 4096^2 at 0.25 m,
    200 targets, 20 dB clutter), reduced to 1024 pulses x 8192 samples imaged
    onto a 256^2 grid at 0.25 m with five isolated targets: split FP32, FP16
    storage and plain FP32;
  * config 5's curved track (0.5 m / 200 m sinusoid + 2 cm jitter, 16384
    samples per pulse: 32768-point range FFTs on the split path), reduced to
    1024 pulses onto a 256^2 grid, FP16 storage, back-projected in
    sub-apertures of 256 pulses x 2 x 2 image tiles as the full-size run is.

Both sides take the oracle's FP64 echo (cast to complex64 for the GPU).
Tolerances (the accuracy target of the split and FP16-storage modes):
  relative L2 <= -60 dB; point targets: peak position within 0.05 pixel,
  PSLR and ISLR within 0.1 dB of the oracle's (range and azimuth cuts).
Plain FP32 BP is the accuracy comparator: it must focus every target, and
misses -60 dB by design.
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


def c2_tile(np_=1024):
    s = scenes.config2(np_=np_, n_img=256)
    s.targets = scenes.isolated_targets(s.grid, seed=21)
    return s


def c5_tile(np_=1024):
    s = scenes.config5(np_=np_, n_img=256)
    s.targets = scenes.isolated_targets(s.grid, seed=51)
    return s


def oracle_chain(orc, s):
    echo = orc.echo(s)
    e64 = echo.astype(np.complex64)
    rc = orc.range_compress(s, e64.astype(np.complex128))
    return e64, rc, orc.backproject(s, rc)


def check_against_oracle(img, ref, s, label):
    err = metrics.rel_l2_db(img, ref)
    cmp = metrics.compare_point_targets(img, ref, metrics.target_pixels(s))
    print(label, f"rel-L2 {err:.1f} dB, peak shift {cmp['peak_shift_px']:.4f} px, "
                 f"PSLR {cmp['pslr_diff_db']:.4f} dB, ISLR {cmp['islr_diff_db']:.4f} dB")
    assert len(cmp["targets"]) == len(s.targets)
    assert err <= -60.0
    assert cmp["peak_shift_px"] <= 0.05
    assert cmp["pslr_diff_db"] <= 0.1
    assert cmp["islr_diff_db"] <= 0.1
    return err, cmp


@pytest.fixture(scope="module")
def c2(orc):
    s = c2_tile()
    e64, rc, ref = oracle_chain(orc, s)
    return dict(scene=s, echo=e64, rc=rc, ref=ref)


@pytest.mark.parametrize("mode", ["split", "fp16store"])
def test_config2_geometry_full_chain_vs_oracle(ctx, c2, mode):
    s = c2["scene"]
    img = sarbp.image_scene(ctx, s, c2["echo"], sarbp.MODES[mode])
    check_against_oracle(img, c2["ref"], s, f"config-2 tile {mode}")


def test_config2_geometry_plain_fp32_focuses(ctx, c2):
    s = c2["scene"]
    r, g, lay = sarbp.scene_args(s)
    rc32 = c2["rc"].astype(np.complex64)
    img = ctx.backproject(r, rc32, s.apc, g, sarbp.MODE_FP32, lay.t0_bins, lay.bin_rate)
    err = metrics.rel_l2_db(img, c2["ref"])
    print(f"config-2 tile plain fp32 rel-L2 {err:.1f} dB")
    assert err < -3.0
    for (x, y) in metrics.target_pixels(s):
        t = metrics.point_target(img, x, y)
        assert abs(t.x - x) <= 1.5 and abs(t.y - y) <= 1.5


def test_config5_curved_track_batched_fp16store_vs_oracle(ctx, orc):
    s = c5_tile()
    assert s.layout.nfft == 32768
    e64, rc, ref = oracle_chain(orc, s)
    r, g, lay = sarbp.scene_args(s)
    h, scale = ctx.range_compress(r, e64, storage=sarbp.STORE_C32H)
    half, sub = s.grid.nx // 2, 256
    img = np.zeros((s.grid.ny, s.grid.nx), np.complex64)
    for ty in range(2):
        for tx in range(2):
            tile = scenes.Grid(origin=s.grid.origin + tx * half * s.grid.ux + ty * half * s.grid.uy,
                               ux=s.grid.ux, uy=s.grid.uy, nx=half, ny=half)
            acc = np.zeros((half, half), np.complex64)
            for p0 in range(0, s.np_, sub):
                acc = ctx.backproject(r, np.ascontiguousarray(h[p0:p0 + sub]), np.ascontiguousarray(s.apc[p0:p0 + sub]),
                                      sarbp.grid_struct(tile), sarbp.MODE_FP16STORE, lay.t0_bins, lay.bin_rate,
                                      scale=np.ascontiguousarray(scale[p0:p0 + sub]), image=acc, accumulate=p0 > 0)
            img[ty * half:(ty + 1) * half, tx * half:(tx + 1) * half] = acc
    check_against_oracle(img, ref, s, "config-5 tile fp16store, 256-pulse sub-apertures x 2x2 tiles")
