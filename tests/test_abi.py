"""C ABI of libsarbp.so, checked without a GPU: the library builds and loads,
exports every entry point include/sarbp.h declares, its structs have the
header's layout (compiled probe), host-only calls work, and device calls
fail cleanly with a status code when no GPU is present."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sarbp.h")


@pytest.fixture(scope="module")
def lib():
    from sar_cambrianaccelerationcard_gb300 import build, sarbp
    build.build()
    return sarbp.load()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sarbp_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("sarbp_create", "sarbp_image", "sarbp_backproject", "sarbp_range_compress",
              "sarbp_launch_back_projection", "sarbp_synthesize_echo"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(sarbp_[a-z0-9_]+)\b", out))
    assert set(declared_functions()) <= exported


def test_binding_covers_every_declared_symbol():
    from sar_cambrianaccelerationcard_gb300 import sarbp
    assert set(declared_functions()) == set(sarbp.SIGNATURES)


def test_struct_layouts_match_header(tmp_path):
    """Compile a probe against include/sarbp.h and compare sizes/offsets with ctypes."""
    from sar_cambrianaccelerationcard_gb300 import sarbp
    src = tmp_path / "probe.c"
    src.write_text(r'''
#include <stdio.h>
#include <stddef.h>
#include "sarbp.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(sarbp_radar), sizeof(sarbp_grid), sizeof(sarbp_rc_layout),
         sizeof(sarbp_rc_view), sizeof(sarbp_target), sizeof(sarbp_ref_params), sizeof(sarbp_complex64));
  printf("%zu %zu %zu %zu\n", offsetof(sarbp_radar, upsample), offsetof(sarbp_grid, nx),
         offsetof(sarbp_rc_view, t0_bins), offsetof(sarbp_ref_params, Nfast));
  return 0;
}''')
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    lines = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    sizes = [int(v) for v in lines[0].split()]
    offs = [int(v) for v in lines[1].split()]
    assert sizes == [ctypes.sizeof(sarbp.Radar), ctypes.sizeof(sarbp.Grid), ctypes.sizeof(sarbp.RcLayout),
                     ctypes.sizeof(sarbp.RcView), ctypes.sizeof(sarbp.Target), ctypes.sizeof(sarbp.RefParams), 8]
    assert offs == [sarbp.Radar.upsample.offset, sarbp.Grid.nx.offset, sarbp.RcView.t0_bins.offset,
                    sarbp.RefParams.Nfast.offset]
    # the reference's SARParams is 12 floats + 3 ints (BPA_CUDA.h:28-50)
    assert sizes[5] == 60


def test_abi_version_and_status_strings(lib):
    from sar_cambrianaccelerationcard_gb300 import sarbp
    header = open(HEADER).read()
    version = int(re.search(r"#define SARBP_ABI_VERSION (\d+)", header).group(1))
    assert lib.sarbp_abi_version() == version == sarbp.ABI_VERSION
    assert lib.sarbp_status_string(0) == b"ok"
    assert lib.sarbp_status_string(2) == b"unsupported"
    assert lib.sarbp_status_string(999) == b"unknown status"


def test_rc_layout_matches_scene_definition(lib):
    from sar_cambrianaccelerationcard_gb300 import sarbp, scenes
    for cfg, (nfft, nbins) in ((scenes.config1(), (4096, 8192)), (scenes.config2(n_img=64, np_=8), (16384, 65536))):
        r = sarbp.radar_struct(cfg.radar, cfg.t_rec0)
        lay = sarbp.RcLayout()
        assert lib.sarbp_rc_layout_get(ctypes.byref(r), cfg.ns, ctypes.byref(lay)) == 0
        want = cfg.layout
        assert (lay.nc, lay.nfft, lay.shift, lay.nbins) == (want.nc, want.nfft, want.shift, want.nbins)
        assert (lay.nfft, lay.nbins) == (nfft, nbins)
        assert lay.t0_bins == pytest.approx(want.t0_bins, rel=0, abs=1e-18)
        assert lay.bin_rate == want.bin_rate


def test_rc_layout_rejects_bad_radar(lib):
    from sar_cambrianaccelerationcard_gb300 import sarbp, scenes
    lay = sarbp.RcLayout()
    r = sarbp.radar_struct(scenes.Radar(), 0.0)
    assert lib.sarbp_rc_layout_get(ctypes.byref(r), 0, ctypes.byref(lay)) == sarbp.ERR_INVALID_ARGUMENT
    r.upsample = 3
    assert lib.sarbp_rc_layout_get(ctypes.byref(r), 100, ctypes.byref(lay)) == sarbp.ERR_INVALID_ARGUMENT
    r.upsample = 8
    r.fs = -1.0
    assert lib.sarbp_rc_layout_get(ctypes.byref(r), 100, ctypes.byref(lay)) == sarbp.ERR_INVALID_ARGUMENT
    assert lib.sarbp_rc_layout_get(None, 100, ctypes.byref(lay)) == sarbp.ERR_INVALID_ARGUMENT


def test_null_context_calls_fail_cleanly(lib):
    from sar_cambrianaccelerationcard_gb300 import sarbp
    assert lib.sarbp_destroy(None) == sarbp.ERR_INVALID_ARGUMENT
    assert lib.sarbp_synchronize(None) == sarbp.ERR_INVALID_ARGUMENT
    assert lib.sarbp_image(None, None, None, 0, 0, None, None, 0, None, None) == sarbp.ERR_INVALID_ARGUMENT
    assert lib.sarbp_kernel_launches(None) == 0
    assert lib.sarbp_create(None, 0) == sarbp.ERR_INVALID_ARGUMENT


def test_create_without_gpu_reports_no_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from sar_cambrianaccelerationcard_gb300 import sarbp
    h = ctypes.c_void_p()
    assert lib.sarbp_create(ctypes.byref(h), 0) == sarbp.ERR_NO_DEVICE
    with pytest.raises(sarbp.SarbpError):
        sarbp.Context(0)
