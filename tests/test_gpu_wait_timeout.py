"""Failure detection without a GPU fault: the back-projection kernels' bounded
staging waits.

Every CTA waits on an mbarrier for each pulse chunk's TMA copies, with a time
limit.  A test-only switch (sarbp_debug_set(SARBP_DEBUG_WAIT_FAULT_CHUNK, k))
arms chunk k's barrier in every CTA with 16 bytes more than its copies bring,
so that phase cannot complete and every CTA's wait runs out after the
(shortened) limit.  The kernel then raises the timeout bit and, before it
exits, waits for the copies still in flight: chunks k and k + 1, each on its
own phase parity (chunk k is phase k / 3 of ring stage k % 3, so chunks 3..5
complete odd phases).  The injected fault's 16 bytes are delivered there, as a
late copy would.

Checked: the call returns SARBP_ERR_TIMEOUT with the timeout bit set and the
drain bit clear (every copy landed before the CTAs released their shared
memory), and the same context then images bit-identically to a fresh one.
The waits are limited to 200 us here; nothing hangs and nothing traps.
"""
import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import sarbp, scenes

pytestmark = pytest.mark.gpu

WAIT_TIMEOUT_BIT = 1
DRAIN_TIMEOUT_BIT = 16


@pytest.fixture(scope="module")
def case():
    s = scenes.config1(np_=512, ns=1024, n_img=256)  # one segment: 32 chunks of 16 pulses per CTA
    with sarbp.Context(0) as ctx:
        echo = sarbp.synthesize(ctx, s)
        r, g, lay = sarbp.scene_args(s)
        rc = ctx.range_compress(r, echo)
        h, scale = ctx.range_compress(r, echo, storage=sarbp.STORE_C32H)
        ref = {m: ctx.backproject(r, rc if m != sarbp.MODE_FP16STORE else h, s.apc, g, m, lay.t0_bins, lay.bin_rate,
                                  scale=scale if m == sarbp.MODE_FP16STORE else None)
               for m in (sarbp.MODE_SPLIT, sarbp.MODE_FP16STORE, sarbp.MODE_FP64)}
    return dict(scene=s, rc=rc, h=h, scale=scale, ref=ref)


def _bp(ctx, case, mode):
    s = case["scene"]
    r, g, lay = sarbp.scene_args(s)
    fp16 = mode == sarbp.MODE_FP16STORE
    return ctx.backproject(r, case["h"] if fp16 else case["rc"], s.apc, g, mode, lay.t0_bins, lay.bin_rate,
                           scale=case["scale"] if fp16 else None)


@pytest.mark.parametrize("mode", [sarbp.MODE_SPLIT, sarbp.MODE_FP16STORE, sarbp.MODE_FP64])
@pytest.mark.parametrize("fault_chunk", [0, 3, 4, 31])
def test_wait_runs_out_then_drains_and_recovers(case, mode, fault_chunk):
    with sarbp.Context(0) as ctx:
        ctx.debug_set(sarbp.DEBUG_BP_SEGMENTS, 1)
        ctx.debug_set(sarbp.DEBUG_WAIT_LIMIT_NS, 200_000)
        ctx.debug_set(sarbp.DEBUG_WAIT_FAULT_CHUNK, fault_chunk)
        with pytest.raises(sarbp.SarbpError) as e:
            _bp(ctx, case, mode)
        assert e.value.status == sarbp.ERR_TIMEOUT, str(e.value)
        flags = ctx.debug_get(sarbp.DEBUG_DEVICE_FLAGS)
        assert flags & WAIT_TIMEOUT_BIT, hex(flags)
        assert not flags & DRAIN_TIMEOUT_BIT, f"a copy was still in flight after the drain ({flags:#x})"
        # the context recovers: defaults back, same bits as a context that never faulted
        ctx.debug_set(sarbp.DEBUG_WAIT_FAULT_CHUNK, -1)
        ctx.debug_set(sarbp.DEBUG_WAIT_LIMIT_NS, 0)
        ctx.debug_set(sarbp.DEBUG_BP_SEGMENTS, 0)
        img = _bp(ctx, case, mode)
    assert np.array_equal(img, case["ref"][mode])


def test_projection_wait_runs_out(case):
    """The weighted projection runs the same staged loop: the same fault gives
    the same status, and the context projects correctly afterwards."""
    s = case["scene"]
    r, g, lay = sarbp.scene_args(s)
    w = (np.random.default_rng(5).standard_normal((g.ny, g.nx)) + 0j).astype(np.complex64)
    with sarbp.Context(0) as ctx:
        ref = ctx.project_weighted(r, case["rc"], s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, w)
        ctx.debug_set(sarbp.DEBUG_WAIT_LIMIT_NS, 200_000)
        ctx.debug_set(sarbp.DEBUG_WAIT_FAULT_CHUNK, 2)
        with pytest.raises(sarbp.SarbpError) as e:
            ctx.project_weighted(r, case["rc"], s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, w)
        assert e.value.status == sarbp.ERR_TIMEOUT
        flags = ctx.debug_get(sarbp.DEBUG_DEVICE_FLAGS)
        assert flags & WAIT_TIMEOUT_BIT and not flags & DRAIN_TIMEOUT_BIT, hex(flags)
        ctx.debug_set(sarbp.DEBUG_WAIT_FAULT_CHUNK, -1)
        ctx.debug_set(sarbp.DEBUG_WAIT_LIMIT_NS, 0)
        again = ctx.project_weighted(r, case["rc"], s.apc, g, sarbp.MODE_SPLIT, lay.t0_bins, lay.bin_rate, w)
    assert np.array_equal(again, ref)


def test_debug_switches_validate_and_read_back():
    with sarbp.Context(0) as ctx:
        for key, bad in ((sarbp.DEBUG_BP_CHUNK, 5), (sarbp.DEBUG_BP_SEGMENTS, 65), (sarbp.DEBUG_WAIT_LIMIT_NS, -1),
                         (sarbp.DEBUG_BP_LINEAR_PHASE, 2), (99, 0)):
            with pytest.raises(sarbp.SarbpError) as e:
                ctx.debug_set(key, bad)
            assert e.value.status == sarbp.ERR_INVALID_ARGUMENT
        ctx.debug_set(sarbp.DEBUG_BP_CHUNK, 8)
        assert ctx.debug_get(sarbp.DEBUG_BP_CHUNK) == 8
        assert ctx.debug_get(sarbp.DEBUG_WAIT_FAULT_CHUNK) == -1
        ctx.debug_set(sarbp.DEBUG_BP_LINEAR_PHASE, -1)
        assert ctx.debug_get(sarbp.DEBUG_BP_LINEAR_PHASE) == -1
        assert ctx.debug_get(sarbp.DEBUG_DEVICE_FLAGS) == 0
