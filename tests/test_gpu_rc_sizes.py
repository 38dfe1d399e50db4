"""Range compression at every supported FFT size (64 ... 32768 points) and
several upsampling factors, against the FP64 oracle.

Each size exercises a different stage sequence of the shared-memory FFT
(radix-8 stages closed by a radix-8, -4 or -2 stage; twiddles computed once per
thread, per butterfly, or with the low table level fixed per thread; two-level
or direct upsampling ramp; the split path at 32768).  Random complex echoes,
4 pulses.  Tolerances as for config 1: complex64 storage <= -110 dB,
FP16 storage <= -60 dB relative L2.
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


def scene_for(nfft: int, L: int) -> scenes.Scene:
    # short chirp for the small transforms, the configs' 10 us chirp from 2048 up
    tp = 0.2e-6 if nfft <= 1024 else 10e-6
    radar = scenes.Radar(tp=tp, upsample=L)
    nc = int(round(radar.tp * radar.fs))
    ns = nfft - nc  # nextpow2(ns + nc - 1) == nfft
    s = scenes.config1(np_=4, ns=ns, n_img=8)
    s.radar = radar
    s.t_rec0 = scenes.centred_record_start(radar, ns)
    assert s.layout.nfft == nfft
    return s


def random_echo(np_: int, ns: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((np_, ns)) + 1j * rng.standard_normal((np_, ns))).astype(np.complex64)


CASES = [(n, 8) for n in (64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384, 32768)] + \
        [(4096, 1), (4096, 4), (16384, 16), (1024, 2)]


@pytest.mark.parametrize("nfft,L", CASES)
def test_range_compression_sizes(ctx, orc, nfft, L):
    s = scene_for(nfft, L)
    echo = random_echo(s.np_, s.ns, nfft + L)
    ref = orc.range_compress(s, echo.astype(np.complex128))
    r, _, lay = sarbp.scene_args(s)
    rc = ctx.range_compress(r, echo)
    err = metrics.rel_l2_db(rc, ref)
    h, scale = ctx.range_compress(r, echo, storage=sarbp.STORE_C32H)
    rc16 = (h[..., 0].astype(np.float64) + 1j * h[..., 1].astype(np.float64)) * scale[:, None]
    err16 = metrics.rel_l2_db(rc16, ref)
    print(f"nfft {nfft} L {L}: c64 {err:.1f} dB, fp16 {err16:.1f} dB")
    assert rc.shape == (s.np_, lay.nbins)
    assert err <= -110.0
    assert err16 <= -60.0
