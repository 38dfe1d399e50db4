"""Contexts on several host threads at once (one context per thread, as the
header prescribes).

Two threads image different scenes over and over on their own contexts: the
same back-projection and range-compression kernels run concurrently with
different staging windows, so different dynamic shared-memory sizes.  Every
image must equal the one the scene gives on a single thread, bit for bit, and
no call may fail (each kernel's shared-memory limit is raised once per device,
not per launch, so one thread cannot lower it under another's launch).
"""
import threading

import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import sarbp, scenes

pytestmark = pytest.mark.gpu


def test_two_threads_with_different_windows():
    a = scenes.config1(np_=256, ns=1024, n_img=256)
    b = scenes.ground_scene(np_=256, ns=2048, n_img=192)
    cases = []
    with sarbp.Context(0) as ctx:
        for s in (a, b):
            echo = sarbp.synthesize(ctx, s)
            refs = {m: sarbp.image_scene(ctx, s, echo, m) for m in (sarbp.MODE_SPLIT, sarbp.MODE_FP16STORE)}
            cases.append((s, echo, refs))
        smem = []
        for s, _, _ in cases:
            r, g, lay = sarbp.scene_args(s)
            v = sarbp.RcView()
            v.data, v.scale, v.storage, v.np, v.nbins = None, None, sarbp.STORE_C64, s.np_, lay.nbins
            v.t0_bins, v.bin_rate = lay.t0_bins, lay.bin_rate
            smem.append(ctx.bp_plan(r, v, s.apc, g, sarbp.MODE_SPLIT).smem_bytes)
    assert smem[0] != smem[1], f"the two scenes should stage different shared-memory sizes ({smem})"
    errors = []

    def worker(case, rounds):
        s, echo, refs = case
        try:
            with sarbp.Context(0) as ctx:
                for k in range(rounds):
                    mode = sarbp.MODE_SPLIT if k % 2 == 0 else sarbp.MODE_FP16STORE
                    img = sarbp.image_scene(ctx, s, echo, mode)
                    if not np.array_equal(img, refs[mode]):
                        errors.append(f"{s.name} round {k}: image differs")
        except Exception as e:  # reported on the main thread
            errors.append(f"{s.name}: {e}")

    threads = [threading.Thread(target=worker, args=(c, 12)) for c in cases]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
