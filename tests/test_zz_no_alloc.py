"""sarbp_range_compress_noalloc: range compression with no device allocation.

Callers that cannot call cudaMalloc while running (their allocator already
holds the GPU's memory, or their loop must not stall on an allocation) use this
entry point; its scratch is a fixed device array inside the library.  These
tests call it through the C ABI:
  * twice in a row with different radar layouts (so the second call must
    replace the tables the first one left in the shared array), each output
    checked against sarbp_range_compress on the same input: bit-identical,
    since both run the same kernels on the same tables;
  * on 32768-point range FFTs (the split path: two CTAs per forward transform,
    2-CTA clusters per inverse, bounds after the spectra in the array) over
    pulses that need several batches of the array, both storages;
  * after a warm-up (np = 0 calls: set-up only), calls that switch layouts
    leave the device's free memory unchanged: nothing is allocated.
The file is collected last and passes both alone and after the other tests.
"""
import ctypes

import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import metrics, sarbp, scenes

pytestmark = pytest.mark.gpu


def _compress_both(ctx, torch, scene, storage):
    r = sarbp.radar_struct(scene.radar, scene.t_rec0)
    lay = scene.layout
    echo = sarbp.synthesize(ctx, scene)
    echo_d = torch.from_numpy(echo.view(np.float32)).cuda()
    esize = 2 if storage == sarbp.STORE_C64 else 1  # float32 words per bin
    ref = torch.zeros((scene.np_, lay.nbins * esize), dtype=torch.float32, device="cuda")
    out = torch.full_like(ref, 123.0)
    ref_sc = torch.zeros(scene.np_, dtype=torch.float32, device="cuda")
    out_sc = torch.full_like(ref_sc, 7.0)
    ctx.check(ctx.lib.sarbp_range_compress(ctx.h, ctypes.byref(r), echo_d.data_ptr(), scene.np_, scene.ns,
                                           storage, ref.data_ptr(), ref_sc.data_ptr(), None), "range_compress")
    ctx.synchronize()
    lib = sarbp.load()
    st = lib.sarbp_range_compress_noalloc(ctypes.byref(r), echo_d.data_ptr(), scene.np_, scene.ns, storage,
                                          out.data_ptr(), out_sc.data_ptr(), None)
    assert st == sarbp.OK, lib.sarbp_status_string(st)
    torch.cuda.synchronize()
    return ref.cpu().numpy(), out.cpu().numpy(), ref_sc.cpu().numpy(), out_sc.cpu().numpy()


@pytest.mark.parametrize("storage", [sarbp.STORE_C64, sarbp.STORE_C32H])
def test_noalloc_matches_allocating_path_twice(storage):
    torch = pytest.importorskip("torch")
    ctx = sarbp.Context(0)
    # call 1: 512 pulses x 1024 samples (nfft 4096); call 2: 300 pulses x 700 samples (nfft 2048)
    first = scenes.config1(np_=512, ns=1024)
    second = scenes.config1(np_=300, ns=700)
    for scene in (first, second):
        ref, out, rsc, osc = _compress_both(ctx, torch, scene, storage)
        if storage == sarbp.STORE_C64:
            a = ref.view(np.complex64)
            b = out.view(np.complex64)
            assert metrics.rel_l2_db(b, a) <= -110.0
            assert np.array_equal(a, b)
        else:
            assert np.array_equal(rsc, osc)
            assert np.array_equal(ref, out)
    ctx.close()


def test_noalloc_rejects_host_pointers_and_oversize():
    lib = sarbp.load()
    s = scenes.config1(np_=4, ns=256)
    r = sarbp.radar_struct(s.radar, s.t_rec0)
    host_echo = np.zeros((4, 256), np.complex64)
    host_out = np.zeros((4, 8 * 256), np.complex64)
    assert lib.sarbp_range_compress_noalloc(ctypes.byref(r), host_echo.ctypes.data, 4, 256, 0,
                                            host_out.ctypes.data, None, None) == sarbp.ERR_INVALID_ARGUMENT
    # a range FFT beyond 32768 points is rejected before touching any memory
    assert lib.sarbp_range_compress_noalloc(ctypes.byref(r), host_echo.ctypes.data, 4, 40000, 0,
                                            host_out.ctypes.data, None, None) == sarbp.ERR_UNSUPPORTED


def _setup(ctx, torch, scene, storage):
    """Echo on the device, the allocating path's output for reference, and
    output buffers for the no-allocation calls (all allocated up front)."""
    r = sarbp.radar_struct(scene.radar, scene.t_rec0)
    lay = scene.layout
    echo_d = torch.from_numpy(sarbp.synthesize(ctx, scene).view(np.float32)).cuda()
    words = 2 if storage == sarbp.STORE_C64 else 1
    ref = torch.zeros((scene.np_, lay.nbins * words), dtype=torch.float32, device="cuda")
    ref_sc = torch.zeros(scene.np_, dtype=torch.float32, device="cuda")
    ctx.check(ctx.lib.sarbp_range_compress(ctx.h, ctypes.byref(r), echo_d.data_ptr(), scene.np_, scene.ns,
                                           storage, ref.data_ptr(), ref_sc.data_ptr(), None), "range_compress")
    out = torch.full_like(ref, 123.0)
    out_sc = torch.full_like(ref_sc, 7.0)
    return dict(scene=scene, r=r, storage=storage, echo=echo_d, ref=ref, ref_sc=ref_sc, out=out, out_sc=out_sc)


def _noalloc(lib, c, np_=None):
    s = c["scene"]
    n = s.np_ if np_ is None else np_
    return lib.sarbp_range_compress_noalloc(ctypes.byref(c["r"]), c["echo"].data_ptr() if n else None, n, s.ns,
                                            c["storage"], c["out"].data_ptr() if n else None,
                                            c["out_sc"].data_ptr() if n else None, None)


def test_noalloc_split_fft_and_no_device_memory_after_warmup():
    torch = pytest.importorskip("torch")
    lib = sarbp.load()
    ctx = sarbp.Context(0)
    # 40 pulses of 16384 samples: nfft 32768, about 13 pulse spectra per batch
    # of the array -> 4 batches; and a 4096-point layout to switch to and from
    big = scenes.config5(np_=40, ns=16384, n_img=64, n_targets=20)
    small = scenes.config1(np_=96, ns=1024)
    assert big.layout.nfft == 32768 and small.layout.nfft == 4096
    cases = [_setup(ctx, torch, sc, st) for st in (sarbp.STORE_C64, sarbp.STORE_C32H) for sc in (big, small)]
    torch.cuda.synchronize()
    # warm-up: set-up only (symbol lookup, tables, kernels loaded), no output written
    for c in cases:
        assert _noalloc(lib, c, np_=0) == sarbp.OK
    torch.cuda.synchronize()
    assert all(float(c["out"][0, 0]) == 123.0 for c in cases)
    free0 = torch.cuda.mem_get_info()[0]
    for c in cases:  # every call switches layout or storage: tables rebuilt in the fixed array
        assert _noalloc(lib, c) == sarbp.OK, lib.sarbp_status_string(_noalloc(lib, c))
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, f"device memory changed by {free0 - free1} bytes"
    for c in cases:
        assert torch.equal(c["out"], c["ref"]), (c["scene"].name, c["storage"])
        if c["storage"] == sarbp.STORE_C32H:
            assert torch.equal(c["out_sc"], c["ref_sc"])
    ctx.close()
