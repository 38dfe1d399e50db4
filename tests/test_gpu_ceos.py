"""GPU CEOS raw-data decode against the reader restatement (oracle/ceos.py):
bit-exact (integer decode times the same float gain), across block
boundaries and the spliced replica, host and device input; and the reference's
own RADARSAT-1 samples decoded and imaged by the omega-K path against the
committed FP64 image."""
import os

import numpy as np
import pytest

from oracle import ceos, wk
from sar_cambrianaccelerationcard_gb300 import metrics, sarbp

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def ctx():
    c = sarbp.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def raw_file():
    rng = np.random.default_rng(9)
    lay = ceos.CeosLayout()
    n, m = 53, 2048
    v = (2 * rng.integers(-8, 8, (n, m)) + 1) + 1j * (2 * rng.integers(-8, 8, (n, m)) + 1)
    codes = rng.integers(0, 64, n)
    return lay, ceos.write(v, codes, lay, first_cell=1049, seed=5)


@pytest.mark.parametrize("first,cnt,c0,nc,agc", [(0, 53, 1049, 2048, True), (6, 9, 1049, 2048, False),
                                                  (7, 1, 0, 9288, True), (13, 40, 2000, 17, True)])
def test_decode_matches_reader(ctx, raw_file, first, cnt, c0, nc, agc):
    lay, raw = raw_file
    ref, ref_a = ceos.read(raw, lay, first, cnt, c0, nc, apply_agc=agc)
    got, got_a = ctx.ceos_decode(raw, first, cnt, c0, nc, apply_agc=agc)
    assert np.array_equal(got, ref)
    assert np.array_equal(got_a, ref_a)


def test_gain_table_follows_layout(ctx, raw_file):
    """The AGC gain table is uploaded when the layout's gain changes and reused
    otherwise: alternating gains on one context match the reader each time."""
    import dataclasses
    lay, raw = raw_file
    for g in (1.5, 2.25, 2.25, 1.5, 0.75):
        lg = dataclasses.replace(lay, gain=g)
        ref, _ = ceos.read(raw, lg, 2, 20, 1049, 2048, apply_agc=True)
        got, _ = ctx.ceos_decode(raw, 2, 20, 1049, 2048, layout=lg, apply_agc=True)
        assert np.array_equal(got, ref), g


def test_decode_device_input(ctx, raw_file):
    torch = pytest.importorskip("torch")
    lay, raw = raw_file
    host, _ = ctx.ceos_decode(raw, 3, 30, 1049, 2048)
    dev_raw = torch.from_numpy(raw).cuda()
    dev, _ = ctx.ceos_decode(dev_raw, 3, 30, 1049, 2048)
    assert np.array_equal(dev, host)


def test_reference_scene_decode_and_image(ctx):
    """CEOS bytes holding the reference's RADARSAT-1 samples (96 lines x 64
    cells of its extracted scene) and attenuation codes decode to exactly
    those samples, and the omega-K image of the decode matches the FP64 image
    of the reference's samples."""
    g = np.load(os.path.join(GOLD, "wk_cd_crop.npz"))
    agc = np.load(os.path.join(GOLD, "ceos_agc.npz"))["agc_db"]
    raw = ceos.write(g["echo"], agc, ceos.CeosLayout(), first_cell=1049 + 1000, seed=6)
    echo, a = ctx.ceos_decode(raw, 0, 96, 1049 + 1000, 64, apply_agc=False)
    assert np.array_equal(echo, g["echo"]) and np.array_equal(a, agc)
    img = ctx.wk_image(wk.radarsat1(), echo)
    assert metrics.rel_l2_db(img, g["image"]) <= -80.0
    gained, _ = ctx.ceos_decode(raw, 0, 96, 1049 + 1000, 64, apply_agc=True)
    ref, _ = ceos.read(raw, ceos.CeosLayout(), 0, 96, 1049 + 1000, 64, apply_agc=True)
    assert np.array_equal(gained, ref)


def test_decode_rejects_bad_requests(ctx, raw_file):
    lay, raw = raw_file
    with pytest.raises(sarbp.SarbpError):
        ctx.ceos_decode(raw, 0, 4, 9000, 300)            # cells beyond the line
    with pytest.raises(sarbp.SarbpError):
        ctx.ceos_decode(raw, 50, 20, 0, 16)              # lines beyond the file's blocks
    with pytest.raises(sarbp.SarbpError):
        ctx.ceos_decode(raw[:100000], 0, 8, 0, 16)       # raw shorter than the first block
