"""The split kernels' per-pixel FP32 arithmetic, emulated on the CPU.

numpy restates, operation by operation, what the split back-projection
kernels compute per pixel and pulse in FP32 (csrc/bp.cu: the series loop, the
linear-term loop, and the per-(tile, pulse) coefficients the producer writes
for each), and compares the differential range and the phase argument with
FP64 on tiles of the configured and of seeded random geometries.  Fused
multiply-adds are emulated as one FP64 evaluation rounded to FP32 (a product of
two FP32 values is exact in FP64, so only the final rounding is double, which
does not move these statistics).

Not emulated: the float-float per-(tile, pulse) reference (R_T, the carrier
phase, the per-step increments before their FP32 rounding: good to about
2^-44, taken here from FP64), and the sine / cosine of the rounded phase
argument (the GPU tests measure the images against the oracle).

Pinned:
  * the form the planner picks (tile, series terms, phase form, through the
    library's own planner) keeps the phase argument within -90 dB RMS (linear-
    term form) or -80 dB (series form) on every geometry, and the differential
    range within 2e-5 m;
  * on every geometry the planner gives the linear-term form, the series form
    would be at least 15 dB worse, and its error grows with the tile's extent
    while the linear-term form's does not: the reason for the planner's switch
    at 12 m of tile half-diagonal.
"""
import math

import numpy as np

from sar_cambrianaccelerationcard_gb300 import scenes
from test_gpu_random_geometry import random_scene
from test_planner_rules import planner  # noqa: F401  (fixture)

f32, f64 = np.float32, np.float64


def fma(a, b, c):
    return (np.asarray(a, f64) * np.asarray(b, f64) + np.asarray(c, f64)).astype(f32)


def mul(a, b):
    return (np.asarray(a, f32) * np.asarray(b, f32)).astype(f32)


def add(a, b):
    return (np.asarray(a, f32) + np.asarray(b, f32)).astype(f32)


def wrap(e):
    return np.remainder(e + math.pi, 2.0 * math.pi) - math.pi


def emulate(scene, tile=(32, 64), nterms=3, ntiles=6, npulses=48, seed=0):
    """RMS phase-argument error (rad) of both forms, their largest
    differential-range error (m), and the tile half-diagonal (m)."""
    tx, ty = tile
    g = scene.grid
    ux, uy, org = (np.asarray(v, f64) for v in (g.ux, g.uy, g.origin))
    kph = 4.0 * math.pi * scene.radar.fc / scene.radar.c  # phase per metre of range
    kh = f32(kph)
    g11, g12, g22 = ux @ ux, ux @ uy, uy @ uy
    gf11, gf12, gf22 = f32(g11), f32(g12), f32(g22)
    rng = np.random.default_rng(seed)
    # pixel offsets from the tile centre (half-integers) and |q|^2 per pixel
    XC, YC = np.meshgrid((np.arange(tx) - 0.5 * (tx - 1)).astype(f32), (np.arange(ty) - 0.5 * (ty - 1)).astype(f32))
    qq = fma(mul(YC, YC), gf22, fma(mul(mul(f32(2.0), XC), YC), gf12, mul(mul(XC, XC), gf11)))
    q = XC[..., None].astype(f64) * ux + YC[..., None].astype(f64) * uy
    err = {"series": [], "linear": []}
    derr = {"series": 0.0, "linear": 0.0}
    for _ in range(ntiles):
        xT = int(rng.integers(0, max(1, -(-g.nx // tx)))) * tx + 0.5 * (tx - 1)
        yT = int(rng.integers(0, max(1, -(-g.ny // ty)))) * ty + 0.5 * (ty - 1)
        PT = org + xT * ux + yT * uy
        for p in rng.choice(scene.np_, min(npulses, scene.np_), replace=False):
            apc = scene.apc[p]
            w = PT - apc
            RT = float(np.linalg.norm(w))
            dr_exact = np.linalg.norm(w + q, axis=-1) - RT
            phT = f32(rng.uniform(-math.pi, math.pi))  # the tile centre's carrier phase
            ph_exact = float(phT) + kph * dr_exact
            # producer: FP32 R_T and its reciprocal, the series coefficients, and
            # A = 2 u_x.w, B = 2 u_y.w from the pulse reference's FP32 hi parts
            r = f32(math.sqrt(float(f32(RT * RT))))
            iR = f32(f32(1.0) / r)
            i2 = mul(iR, iR)
            c1 = mul(f32(0.5), iR)
            wo = org - apc
            A = add(f32(2.0 * ux @ wo), mul(f32(2.0), fma(f32(xT), gf11, mul(f32(yT), gf12))))
            B = add(f32(2.0 * uy @ wo), mul(f32(2.0), fma(f32(xT), gf12, mul(f32(yT), gf22))))
            # series form: n = 2 q.w + |q|^2, dR = n (c1 + n (c2 + n (c3 [+ n c4])))
            c2 = mul(mul(f32(-0.125), iR), i2)
            c3 = mul(mul(mul(f32(0.0625), iR), i2), i2)
            c4 = mul(mul(mul(mul(f32(-0.0390625), iR), i2), i2), i2)
            n = fma(YC, B, add(mul(XC, A), qq))
            poly = fma(n, fma(n, c4, c3), c2) if nterms == 4 else fma(n, c3, c2)
            dR = mul(n, fma(n, poly, c1))
            err["series"].append(wrap(fma(dR, kh, phT).astype(f64) - ph_exact).ravel())
            derr["series"] = max(derr["series"], float(np.max(np.abs(dR - dr_exact))))
            # linear-term form: m = n / (2 R_T), dR = m + m^2 (d2 + m (d3 [+ m d4])),
            # phase = phT + 2 xc PX + 2 yc PY + kph (qq c1 + m^2 poly), PX and PY the
            # per-step increments (2 pi fc / c) u.w / R_T reduced modulo 2 pi
            d2, d3, d4 = mul(f32(-0.5), iR), mul(f32(0.5), i2), mul(mul(f32(-0.625), i2), iR)
            px = f32(math.remainder(0.5 * kph * (ux @ w) / RT, 2.0 * math.pi))
            py = f32(math.remainder(0.5 * kph * (uy @ w) / RT, 2.0 * math.pi))
            phx = fma(mul(f32(2.0), XC), px, phT)
            qc = mul(qq, c1)
            m = fma(YC, mul(B, c1), add(mul(XC, mul(A, c1)), qc))
            m2 = mul(m, m)
            poly = fma(m, fma(m, d4, d3), d2) if nterms == 4 else fma(m, d3, d2)
            dRl = fma(m2, poly, m)
            ph = fma(fma(m2, poly, qc), kh, fma(mul(f32(2.0), YC), py, phx))
            err["linear"].append(wrap(ph.astype(f64) - ph_exact).ravel())
            derr["linear"] = max(derr["linear"], float(np.max(np.abs(dRl - dr_exact))))
    hx, hy = 0.5 * (tx - 1), 0.5 * (ty - 1)
    half_diag = math.sqrt(hx * hx * g11 + 2.0 * hx * hy * abs(g12) + hy * hy * g22)
    rms = {k: float(np.sqrt(np.mean(np.concatenate(v) ** 2))) for k, v in err.items()}
    return rms, derr, half_diag


def db(x):
    return 20.0 * math.log10(x)


GEOMETRIES = [("config2", lambda: scenes.config2(np_=512, n_img=512)), ("config1", scenes.config1)] + [
    (f"random{k}", (lambda k=k: random_scene(k))) for k in range(16)]


def test_planned_form_accuracy(planner):  # noqa: F811
    rows = []
    for name, make in GEOMETRIES:
        s = make()
        p = planner(s)
        assert p["ok"], (name, p)
        rms, derr, hd = emulate(s, tile=p["tile"], nterms=p["nterms"])
        form = "linear" if p["lin"] else "series"
        rows.append((name, form, hd, db(rms["series"]), db(rms["linear"])))
        assert rms[form] <= 10 ** ((-90.0 if p["lin"] else -80.0) / 20.0), rows[-1]
        assert derr[form] <= 2e-5, (name, derr)
        if p["lin"]:
            assert db(rms["series"]) - db(rms["linear"]) >= 15.0, rows[-1]
    forms = {r[1] for r in rows}
    assert forms == {"linear", "series"}, rows  # both forms exercised


def test_error_against_tile_extent():
    # config-2 aperture and swath, 32 x 64 tiles, pixels scaled to each half-diagonal
    series = {}
    for half_diag in (3.0, 12.0, 24.0):
        s = scenes.config2(np_=512, n_img=512, spacing=half_diag / math.hypot(15.5, 31.5))
        rms, _, hd = emulate(s, nterms=4)
        assert abs(hd - half_diag) < 1e-9
        assert db(rms["linear"]) <= -100.0, (half_diag, rms)
        series[half_diag] = rms["series"]
    assert db(series[3.0]) <= -90.0 and db(series[12.0]) <= -80.0, series
    # past the planner's threshold the series form loses accuracy with the extent
    assert series[3.0] < series[12.0] < series[24.0] and series[24.0] >= 4.0 * series[3.0], series
