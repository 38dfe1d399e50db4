"""Config-5 pieces: the split range FFT (ns = 16384 -> nfft = 32768, two CTAs per
pulse and a 2-CTA cluster per upsampling phase) against the FP64 oracle, and
curved-track FP16-storage back-projection processed in sub-aperture and
image-tile batches against the FP64 GPU comparator."""
import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import metrics, sarbp, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sarbp.Context(0)
    yield c
    c.close()


def c5_scene(np_, n_img, ns=16384):
    s = scenes.config5(np_=np_, ns=ns, n_img=n_img, n_targets=40)
    return s


def test_split_range_fft_matches_oracle(ctx, orc):
    s = c5_scene(np_=6, n_img=64)
    assert s.layout.nfft == 32768
    echo = orc.echo(s).astype(np.complex64)
    ref = orc.range_compress(s, echo.astype(np.complex128))
    r, g, lay = sarbp.scene_args(s)
    rc = ctx.range_compress(r, echo)
    err = metrics.rel_l2_db(rc, ref)
    print("split rc c64 rel-L2 dB", err)
    assert err <= -110.0
    h, scale = ctx.range_compress(r, echo, storage=sarbp.STORE_C32H)
    assert np.all(np.frexp(scale)[0] == 0.5)
    rc16 = (h[..., 0].astype(np.float64) + 1j * h[..., 1].astype(np.float64)) * scale[:, None]
    err16 = metrics.rel_l2_db(rc16, ref)
    print("split rc fp16 rel-L2 dB", err16)
    assert err16 <= -60.0


def test_curved_track_batched_fp16store_vs_fp64(ctx):
    """1024 pulses of the curved track (0.5 m / 200 m sinusoid + 2 cm jitter),
    768^2 image: sub-apertures of 256 pulses x 4 image tiles, accumulated, equal
    the single-call image and stay within -60 dB of the FP64 comparator."""
    s = c5_scene(np_=1024, n_img=768)
    echo = sarbp.synthesize(ctx, s)
    r, g, lay = sarbp.scene_args(s)
    h, scale = ctx.range_compress(r, echo, storage=sarbp.STORE_C32H)
    rc64 = ctx.range_compress(r, echo)
    full = ctx.backproject(r, h, s.apc, g, sarbp.MODE_FP16STORE, lay.t0_bins, lay.bin_rate, scale=scale)
    ref = ctx.backproject(r, rc64, s.apc, g, sarbp.MODE_FP64, lay.t0_bins, lay.bin_rate)
    err = metrics.rel_l2_db(full, ref)
    print("curved fp16store vs fp64 rel-L2 dB", err)
    assert err <= -60.0
    tiled = np.zeros_like(full)
    half = s.grid.nx // 2
    for ty in range(2):
        for tx in range(2):
            sub = scenes.Grid(origin=s.grid.origin + tx * half * s.grid.ux + ty * half * s.grid.uy,
                              ux=s.grid.ux, uy=s.grid.uy, nx=half, ny=half)
            gs = sarbp.grid_struct(sub)
            img = np.zeros((half, half), np.complex64)
            for p0 in range(0, s.np_, 256):
                img = ctx.backproject(r, np.ascontiguousarray(h[p0:p0 + 256]),
                                      np.ascontiguousarray(s.apc[p0:p0 + 256]), gs, sarbp.MODE_FP16STORE,
                                      lay.t0_bins, lay.bin_rate, scale=np.ascontiguousarray(scale[p0:p0 + 256]),
                                      image=img, accumulate=p0 > 0)
            tiled[ty * half:(ty + 1) * half, tx * half:(tx + 1) * half] = img
    assert metrics.rel_l2_db(tiled, full) <= -100.0
