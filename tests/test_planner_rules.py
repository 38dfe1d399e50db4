"""The back-projection planner's rules, checked on the CPU.

A small C++ harness (compiled here with g++) calls the library's own planner,
sarbp::plan_bp with the host geometry extremes, exactly as the serving loop
does, on scenes built in Python.  No GPU is needed: planning is host code.

Pinned:
  * config 2's geometry (0.25 m pixels) takes 32 x 64 tiles, 3 series terms and
    the series phase form; config 1's (0.5 m pixels, 17.5 m tile half-diagonal)
    the linear-term form;
  * the linear-term form starts at 12 m of tile half-diagonal, and the debug
    switch forces either form;
  * the split modes' envelope: the smallest tile (32 x 16) must keep the
    differential-range series remainder below 5e-7 m, so grids at 45 degrees
    to the track are refused past about 1.4 m pixels at 2 km slant range and
    2.9 m at 5 km (both sides of each bound are checked), while the FP64 mode
    plans them;
  * the staging-window bound, common to every mode: at 10 km the smallest
    tile's window outgrows shared memory past about 5 m pixels.
"""
import math
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from sar_cambrianaccelerationcard_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sar_cambrianaccelerationcard_gb300")
LIB = os.path.join(PKG, "libsarbp.so")

HARNESS = r"""
#include <cstdio>
#include <string>
#include <vector>
#include "sarbp_internal.h"
int main() {
    double rd[7];   // c fc fs kr tp tc t_rec0
    int ri[2];      // upsample, np
    double view[2]; // t0_bins, bin_rate
    int vi[2];      // nbins, mode
    int force;
    double gv[9];
    int gn[2];
    if (fread(rd, 8, 7, stdin) != 7 || fread(ri, 4, 2, stdin) != 2 || fread(view, 8, 2, stdin) != 2 ||
        fread(vi, 4, 2, stdin) != 2 || fread(&force, 4, 1, stdin) != 1 || fread(gv, 8, 9, stdin) != 9 ||
        fread(gn, 4, 2, stdin) != 2)
        return 1;
    const int np = ri[1];
    std::vector<double> apc(3 * (size_t)np);
    if (fread(apc.data(), 8, apc.size(), stdin) != apc.size()) return 1;
    sarbp_radar r{};
    r.c = rd[0]; r.fc = rd[1]; r.fs = rd[2]; r.kr = rd[3]; r.tp = rd[4]; r.tc = rd[5]; r.t_rec0 = rd[6];
    r.upsample = ri[0];
    sarbp_rc_view v{};
    v.storage = SARBP_STORE_C64; v.np = np; v.nbins = vi[0]; v.t0_bins = view[0]; v.bin_rate = view[1];
    sarbp_grid g{};
    for (int k = 0; k < 3; ++k) { g.origin[k] = gv[k]; g.ux[k] = gv[3 + k]; g.uy[k] = gv[6 + k]; }
    g.nx = gn[0]; g.ny = gn[1];
    sarbp::BpExtremes ex;
    sarbp::bp_extremes_host(apc.data(), np, g, ex);
    sarbp::Tuning tune;
    tune.linear_phase = force;
    sarbp::BpPlan p;
    std::string why;
    const bool ok = sarbp::plan_bp(152, r, v, ex, np, g, vi[1], 0, p, why, &tune);
    int tx = 0, ty = 0;
    if (ok) sarbp::bp_tile_dims(p.pix, &tx, &ty);
    printf("%d %d %d %d %d %d|%s\n", ok ? 1 : 0, tx, ty, ok ? p.nterms : 0, ok ? p.lin : 0, ok ? p.win : 0, why.c_str());
    return 0;
}
"""


def cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


@pytest.fixture(scope="module")
def planner(tmp_path_factory):
    inc = cuda_include()
    if not (shutil.which("g++") and inc and os.path.exists(LIB)):
        pytest.skip("needs g++, the CUDA headers and the built library")
    d = tmp_path_factory.mktemp("planner")
    src, exe = d / "harness.cpp", d / "harness"
    src.write_text(HARNESS)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(PKG, "csrc"),
                    "-I", inc, str(src), "-o", str(exe), LIB, f"-Wl,-rpath,{PKG}"], check=True)

    def plan(scene, mode=2, force=0):
        rad, g, lay = scene.radar, scene.grid, scene.layout
        data = struct.pack("7d", rad.c, rad.fc, rad.fs, rad.kr, rad.tp, rad.tp / 2.0, scene.t_rec0)
        data += struct.pack("2i", rad.upsample, scene.np_)
        data += struct.pack("2d", lay.t0_bins, lay.bin_rate) + struct.pack("2i", lay.nbins, mode)
        data += struct.pack("i", force) + struct.pack("9d", *g.origin, *g.ux, *g.uy) + struct.pack("2i", g.nx, g.ny)
        data += np.ascontiguousarray(scene.apc, dtype=np.float64).tobytes()
        out = subprocess.run([str(exe)], input=data, capture_output=True, check=True).stdout.decode()
        nums, why = out.strip().split("|", 1)
        ok, tx, ty, nterms, lin, win = (int(x) for x in nums.split())
        return dict(ok=bool(ok), tile=(tx, ty), nterms=nterms, lin=lin, win=win, why=why)

    return plan


def rotated_scene(spacing, slant_range, n=128, theta=math.pi / 4, np_=256):
    """A grid at `theta` to the track, centred at `slant_range` (3/5 of it in
    altitude), the swath covering it."""
    radar = scenes.Radar()
    apc = scenes.straight_track(radar, np_)
    alt = 0.6 * slant_range
    apc[:, 2] += alt
    ux = spacing * np.array([math.cos(theta), math.sin(theta), 0.0])
    uy = spacing * np.array([-math.sin(theta), math.cos(theta), 0.0])
    centre = np.array([0.0, math.sqrt(slant_range ** 2 - alt ** 2), 0.0])
    grid = scenes.Grid(origin=centre - (n // 2) * ux - (n // 2) * uy, ux=ux, uy=uy, nx=n, ny=n)
    c = grid.pixel(np.array([0.0, n - 1, 0.0, n - 1]), np.array([0.0, 0.0, n - 1, n - 1]))
    rr = np.linalg.norm(c[None, :, :] - apc[:, None, :], axis=2)
    t_rec0 = 2.0 * float(rr.min()) / radar.c - 2e-7
    ns = int(math.ceil((2.0 * (float(rr.max()) - float(rr.min())) / radar.c + radar.tp + 4e-7) * radar.fs))
    return scenes.Scene(name="rot", radar=radar, np_=np_, ns=ns, apc=apc, grid=grid, targets=np.zeros((0, 4)),
                        t_rec0=t_rec0, snr_db=None, seed=0)


def test_configured_geometries(planner):
    c2 = planner(scenes.config2(np_=512, n_img=512))
    assert c2["ok"] and c2["tile"] == (32, 64) and c2["nterms"] == 3 and c2["lin"] == 0, c2
    c1 = planner(scenes.config1())
    assert c1["ok"] and c1["tile"] == (32, 64) and c1["lin"] == 1, c1


def test_linear_phase_threshold_and_switch(planner):
    # 32 x 64 tiles: half-diagonal = spacing * hypot(15.5, 31.5)
    h = math.hypot(15.5, 31.5)
    below = scenes.config1(spacing=11.9 / h)
    above = scenes.config1(spacing=12.1 / h)
    assert planner(below)["lin"] == 0 and planner(above)["lin"] == 1
    assert planner(above, force=-1)["lin"] == 0 and planner(below, force=1)["lin"] == 1
    assert planner(above, mode=0)["lin"] == 0  # FP64 mode: no phase form to choose


@pytest.mark.parametrize("slant_range,limit", [(2000.0, 1.38), (5000.0, 2.89)])
def test_split_envelope(planner, slant_range, limit):
    inside = planner(rotated_scene(0.95 * limit, slant_range))
    outside = planner(rotated_scene(1.05 * limit, slant_range))
    assert inside["ok"], inside
    assert not outside["ok"] and "differential-range series" in outside["why"], outside
    assert planner(rotated_scene(1.05 * limit, slant_range), mode=0)["ok"]


def test_window_bound_all_modes(planner):
    # 10 km: the smallest tile's staging window outgrows shared memory (chunk 4,
    # one CTA per SM) before the series bound, for every mode alike
    inside, outside = rotated_scene(0.95 * 5.04, 10000.0), rotated_scene(1.05 * 5.04, 10000.0)
    for mode in (0, 1, 2, 3):
        assert planner(inside, mode=mode)["ok"], mode
        out = planner(outside, mode=mode)
        assert not out["ok"] and "shared memory" in out["why"], (mode, out)
