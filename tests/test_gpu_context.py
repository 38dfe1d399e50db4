"""Context memory accounting: sarbp_device_bytes counts every buffer the
context holds, and sarbp_trim releases every call-sized buffer (range
compression, back-projection, projection, autofocus, omega-K and DFT
scratch), leaving only the persistent words and tables; the next call
re-grows what it needs."""
import numpy as np
import pytest

from oracle import wk
from sar_cambrianaccelerationcard_gb300 import sarbp, scenes

pytestmark = pytest.mark.gpu


def test_trim_releases_all_scratch():
    ctx = sarbp.Context(0)
    try:
        base = ctx.lib.sarbp_device_bytes(ctx.h)
        s = scenes.config1(np_=128, ns=1024, n_img=64)
        r, g, lay = sarbp.scene_args(s)
        echo = sarbp.synthesize(ctx, s)
        img = sarbp.image_scene(ctx, s, echo, sarbp.MODE_SPLIT)
        rc = ctx.range_compress(r, echo)
        w = (np.abs(img) ** 2 * img).astype(np.complex64)
        ctx.project_weighted(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, w)
        ctx.autofocus(r, rc, s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, 2)
        rng = np.random.default_rng(2)
        e = (rng.standard_normal((96, 64)) + 1j * rng.standard_normal((96, 64))).astype(np.complex64)
        ctx.wk_image(wk.radarsat1(), e)
        ctx.dft(e.copy())
        ctx.dft(np.ascontiguousarray(e[:, :61]))  # a Bluestein length
        grown = ctx.lib.sarbp_device_bytes(ctx.h)
        assert grown > base + (4 << 20)
        ctx.check(ctx.lib.sarbp_trim(ctx.h), "trim")
        trimmed = ctx.lib.sarbp_device_bytes(ctx.h)
        # what stays: the check word, the power scalar, the planning extremes and
        # the range-compression tables of the last layout
        assert trimmed < (2 << 20), trimmed
        # the next call re-grows and still works
        again = sarbp.image_scene(ctx, s, echo, sarbp.MODE_SPLIT)
        assert np.array_equal(again, img)
    finally:
        ctx.close()
