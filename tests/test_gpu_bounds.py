"""Evidence for the unclamped back-projection inner loop.

The production SPLIT / FP16STORE kernels index the staged range window
without a per-update clamp: the window is sized (and checked per tile and
pulse by the producer) so that every bin a pixel needs lies inside it.  The
checked kernels (sarbp_debug_set(SARBP_DEBUG_BP_CHECKED, 1)) keep a clamp
on every index and report through the context if they ever changed one.  Over
straight, curved and ragged geometries they must report nothing and produce the
same image bit for bit.
"""
import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import sarbp, scenes

pytestmark = pytest.mark.gpu


def scenes_to_check():
    a = scenes.config1(np_=256, ns=1024)
    b = scenes.config2(np_=512, ns=4096, n_img=512)
    c = scenes.config2(np_=512, ns=4096, n_img=300)
    c.apc = scenes.curved_track(c.radar, c.np_, seed=5)
    d = scenes.config1(np_=100, ns=700)
    d.grid = scenes.centred_grid(d.radar, 77, 130, 0.5)
    e = scenes.ground_scene()  # 1 m ground pixels from 5 km altitude: shorter tiles
    return [a, b, c, d, e]


@pytest.mark.parametrize("mode", ["split", "fp16store"])
def test_checked_kernel_never_clamps(mode):
    checked = sarbp.Context(0)
    checked.debug_set(sarbp.DEBUG_BP_CHECKED, 1)
    results = []
    for s in scenes_to_check():  # the clamped kernel runs first and must report nothing
        echo = sarbp.synthesize(checked, s)
        results.append((s, echo, sarbp.image_scene(checked, s, echo, sarbp.MODES[mode])))
    plain = sarbp.Context(0)
    for s, echo, b in results:
        a = sarbp.image_scene(plain, s, echo, sarbp.MODES[mode])
        assert np.array_equal(a, b), s.name
    checked.close()
    plain.close()
