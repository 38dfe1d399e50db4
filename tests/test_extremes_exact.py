"""The planner's geometry extremes (range extremes and the largest
line-of-sight cosines over a 9 x 9 grid lattice and every pulse) skip the
cosine quotients that a division-free comparison rules out, and take the range
extremes as square roots of the squared ones.  This checks, on the CPU, that
the reduction the library runs on the host and the device (the header-only
helpers in csrc/sarbp_internal.h, compiled here with g++ and no fused
multiply-adds) gives the exact extremes of the per-point formula, evaluated
point by point in numpy, over randomised tracks and grids."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "sar_cambrianaccelerationcard_gb300", "csrc")

HARNESS = r"""
#include <cstdio>
#include <vector>
#include "sarbp_internal.h"
using namespace sarbp;
int main() {
    int np;
    sarbp_grid g{};
    if (fread(&np, 4, 1, stdin) != 1) return 1;
    double gv[9];
    int n2[2];
    if (fread(gv, 8, 9, stdin) != 9 || fread(n2, 4, 2, stdin) != 2) return 1;
    for (int k = 0; k < 3; ++k) { g.origin[k] = gv[k]; g.ux[k] = gv[3 + k]; g.uy[k] = gv[6 + k]; }
    g.nx = n2[0]; g.ny = n2[1];
    std::vector<double> apc(3 * (size_t)np);
    if (fread(apc.data(), 8, apc.size(), stdin) != apc.size()) return 1;
    const double lux = std::sqrt(ext_dot(g.ux, g.ux)), luy = std::sqrt(ext_dot(g.uy, g.uy));
    double P[kLattice * kLattice][3];
    for (int k = 0; k < kLattice * kLattice; ++k) ext_lattice(g, k / kLattice, k % kLattice, P[k]);
    ExtAcc acc;
    ext_acc_init(acc);
    for (int i = 0; i < np; ++i)
        for (int k = 0; k < kLattice * kLattice; ++k) ext_acc_point(acc, g, lux, luy, P[k], &apc[3 * (size_t)i]);
    BpExtremes e{};
    ext_ranges(acc.r2min, acc.r2max, e);
    const double out[4] = {e.rmin, e.rmax, acc.cx.best, acc.sy.best};
    fwrite(out, 8, 4, stdout);
    return 0;
}
"""


def cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    inc = cuda_include()
    if shutil.which("g++") is None or inc is None:
        pytest.skip("g++ or the CUDA headers are not available")
    d = tmp_path_factory.mktemp("ext")
    src, exe = d / "h.cpp", d / "h"
    src.write_text(HARNESS)
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I", inc, "-I", os.path.join(ROOT, "include"),
                    "-I", CSRC, str(src), "-o", str(exe)], check=True)
    return str(exe)


def brute(apc, origin, ux, uy, nx, ny):
    dot = lambda a, b: (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]
    lux, luy = np.sqrt(dot(ux, ux)), np.sqrt(dot(uy, uy))
    k = np.arange(9)
    fx = ((nx - 1) * k).astype(np.float64) / 8.0
    fy = ((ny - 1) * k).astype(np.float64) / 8.0
    P = (origin[None, None, :] + fx[:, None, None] * ux[None, None, :]) + fy[None, :, None] * uy[None, None, :]
    w = P[None] - apc[:, None, None, :]
    R = np.sqrt(dot(w, w))
    with np.errstate(divide="ignore", invalid="ignore"):
        cx = np.where(R > 0, np.abs(dot(ux, w)) / (R * lux), 0.0)
        cy = np.where(R > 0, np.abs(dot(uy, w)) / (R * luy), 0.0)
    return R.min(), R.max(), cx.max(), cy.max()


def run(exe, apc, origin, ux, uy, nx, ny):
    blob = struct.pack("<i", apc.shape[0]) + np.concatenate([origin, ux, uy]).astype("<f8").tobytes() + \
        struct.pack("<ii", nx, ny) + apc.astype("<f8").tobytes()
    out = subprocess.run([exe], input=blob, capture_output=True, check=True).stdout
    return tuple(np.frombuffer(out, dtype="<f8"))


@pytest.mark.parametrize("seed", range(24))
def test_extremes_exact(harness, seed):
    rng = np.random.default_rng(seed)
    np_ = int(rng.integers(1, 600))
    t = np.arange(np_) - np_ / 2
    kind = seed % 4
    speed = rng.uniform(0.05, 2.0)
    apc = np.zeros((np_, 3))
    apc[:, 0] = speed * t
    if kind >= 1:  # curved track with jitter
        apc[:, 1] = rng.uniform(0.1, 5) * np.sin(2 * np.pi * apc[:, 0] / rng.uniform(50, 500))
        apc[:, :] += rng.normal(0, 0.02, apc.shape)
    if kind >= 2:  # altitude
        apc[:, 2] = rng.uniform(100, 8000)
    r0 = rng.uniform(500, 20000)
    sq = rng.uniform(-0.5, 0.5)  # squint: grid centre ahead of or behind the aperture
    nx, ny = int(rng.integers(1, 5000)), int(rng.integers(1, 5000))
    sp = rng.uniform(0.05, 2.0)
    ux = np.array([0.0, sp, 0.0])
    uy = np.array([sp, 0.0, 0.0])
    if kind == 3:  # skewed, tilted axes
        uy = uy + rng.uniform(-0.3, 0.3) * ux + np.array([0, 0, rng.uniform(-0.05, 0.05)])
    origin = np.array([sq * r0 - 0.5 * ny * sp, r0 - 0.5 * nx * sp, rng.uniform(-50, 50)])
    want = brute(apc, origin, ux, uy, nx, ny)
    got = run(harness, apc, origin, ux, uy, nx, ny)
    assert got == want, (got, want)
