// bp.cu -- back-projection on sm_103a.
//
// Algorithm: code/SAR_BP/matlab/BPA_SAR.m:177-197 (per pixel and pulse: slant
// range, range bin, sample, phase compensation exp(+j 4 pi fc R / c), coherent
// sum), with linear interpolation on the upsampled bins instead of the script's
// nearest bin.  Kernel shape replaces backProjectionKernel
// (code/SAR_BP/CUDA/BPA_CUDA_kernels.cu:47-77: one thread per pixel, global
// loads, sqrtf + sincosf per pulse).
//
// Design (one CTA per TILE_X x TILE_Y pixel tile, optionally per pulse segment):
//  * Pulses are processed in chunks of CHUNK.  For each chunk every warp
//    computes, for two of its pulses, the tile-centre reference: range R_T
//    (FP32 square root refined by one FP64 Newton step), the FP64-wrapped
//    carrier phase, the bin of the tile centre and the window of bins the tile
//    can touch; it then issues one TMA bulk copy (cp.async.bulk, local HBM ->
//    shared memory, completion on an mbarrier) per pulse for that window.  A
//    three-stage ring of raw windows lets chunk c+1 load while chunk c computes.
//  * A conversion pass turns each raw window (complex64, or complex16 times the
//    per-pulse scale) into interpolation-ready pairs (mid, diff) with
//    mid_i = (s_i + s_{i+1})/2, diff_i = s_{i+1} - s_i, so one 16-byte shared load
//    and two FMAs interpolate.  Converted windows are double-buffered: one
//    block barrier per chunk.
//  * SPLIT arithmetic per pixel and pulse: with q the pixel offset from the tile
//    centre, n = 2 q.w + |q|^2 (w = tile centre - APC) and the differential
//    range dR = sqrt(R_T^2 + n) - R_T = n (c1 + n (c2 + n (c3 + n c4))) (series
//    of sqrt(1+e); the planner bounds the truncation error) -- all on the FMA
//    pipe; the phase fma(dR, k_hi, phi_T) + dR k_lo (compensated product); the
//    only MUFU work is one sin/cos pair.
//  * Staging windows are sized so every bin a pixel can need lies inside
//    [1, win-3]; the producer checks this per (tile, pulse) and, should a pulse
//    fail the check, neutralises it (no data, bin 1) and raises an error bit,
//    so shared-memory indices stay in bounds without a per-update clamp.  The
//    CHECKED variant keeps a clamp and reports whether it ever fired.
//  * FP32 and FP64 modes use the same staging with plain absolute-range
//    arithmetic (the comparators) and always clamp.
#include "sarbp_internal.h"

#include <math_constants.h>

#include "ffloat.cuh"
#include "tma.cuh"

#include <cstddef>

namespace sarbp {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kTileX = 32;  // pixels along x (columns); tile height is 8 * PIX rows
#ifndef SARBP_BP_CHUNK
#define SARBP_BP_CHUNK 16
#endif
#ifndef SARBP_BP_MINBLOCKS
#define SARBP_BP_MINBLOCKS 2
#endif
// Per-update phase: phi_T + dR k_hi (k_hi = float(4 pi fc / c)); the
// compensated form adds dR k_lo.  The omitted term is at most
// |dR| ulp(k)/2 (7e-5 rad at config 2's tile corners) and is of the size of the
// FP32 rounding of dR itself and of the sin/cos argument, so the image does
// not change measurably (-81.68 dB against FP64 either way) and the update is
// one packed FMA shorter.
#ifndef SARBP_BP_PHASE_COMPENSATED
#define SARBP_BP_PHASE_COMPENSATED 0
#endif
#ifndef SARBP_BP_PULSE_UNROLL
#define SARBP_BP_PULSE_UNROLL 2
#endif
constexpr int kPulseUnroll = SARBP_BP_PULSE_UNROLL;  // pulses per loop body (SPLIT)
constexpr int kChunk = SARBP_BP_CHUNK;  // pulses per staged chunk (a multiple of 8)
constexpr int kPerWarp = kChunk / kWarps;  // pulses each warp prepares
static_assert(kChunk % kWarps == 0 && kPerWarp <= 32, "chunk must split evenly over the warps");
constexpr int kStages = 3;  // raw-window ring depth
constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23: adding it rounds to an integer
constexpr unsigned kMagicBitsShift4 = 0x4B400000u << 4;

struct __align__(16) Prm {
    // SPLIT: each constant twice, so a 16-byte load yields two packed f32x2 operands
    float4 k0;     // SPLIT: c1, c1, c2, c2     FP32: apc x, y, z, bin offset
    float4 k1;     // SPLIT: c3, c3, c4, c4
    float4 k2;     // SPLIT: bin', bin', phT, phT
    float4 k3;     // SPLIT: A, A, B, B
    double ax, ay, az;  // FP64: APC position
    double dr, dph;     // FP64: per-pulse range (m) and phase (rad) corrections
    int ws;        // first bin of the window
    int lo, hi;    // copied part of the window [lo, hi) relative to ws
    float scale;   // FP16 storage scale
    int need;      // (M, d) pairs [0, need) any pixel of the tile reads (the rest are not converted)
};

// Linear-term split (LIN) kernels: the phase increments per pixel step,
// (PX, PX, PY, PY), in the 16 bytes of the FP64-only ax, ay (offset 64,
// 16-byte aligned), so the record keeps its size.
__device__ __forceinline__ float4 &prm_k4(Prm &q) { return *reinterpret_cast<float4 *>(&q.ax); }
__device__ __forceinline__ const float4 &prm_k4(const Prm &q) { return *reinterpret_cast<const float4 *>(&q.ax); }
static_assert(offsetof(Prm, ax) % 16 == 0 && offsetof(Prm, az) - offsetof(Prm, ax) == 16, "k4 slot");

__device__ __forceinline__ float4 lds128(unsigned addr) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(addr));
    return v;
}

// Packed FP32x2 arithmetic (sm_100+ f32x2 instructions): two IEEE FP32
// operations, each rounded to nearest, per issue slot.  A pair lives in a
// 64-bit register pair (lo, hi).
typedef unsigned long long f2;
__device__ __forceinline__ f2 pk2(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk2(f2 v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 ffma2(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2 fadd2(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 fmul2(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// 16-byte shared load as two packed pairs
__device__ __forceinline__ void lds2x2(const void *p, f2 &a, f2 &b) {
    asm volatile("ld.shared.v2.b64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "r"(smem_addr(p)));
}

struct Smem {
    float4 *staged;      // [2][chunk][win]
    unsigned char *raw;  // [kStages][chunk][win] stored elements (8 or 4 bytes)
    Prm *prm;            // [kStages][kChunk] (chunk <= kChunk pulses used per stage)
    uint64_t *bar;       // [kStages]
    float2 *red;         // [2][kWarps][kChunk] per-warp pulse sums (weighted projection)
};

// Bytes of one stored range bin in the raw ring: complex64 rows 8, complex16 4.
__host__ __device__ constexpr int raw_esize(int storage) { return storage == SARBP_STORE_C64 ? 8 : 4; }

template <int STORE>
__device__ __forceinline__ Smem carve(unsigned char *base, int win, int chunk) {
    Smem s;
    s.staged = reinterpret_cast<float4 *>(base);
    s.raw = base + (size_t)2 * chunk * win * 16;
    s.prm = reinterpret_cast<Prm *>(s.raw + (size_t)kStages * chunk * win * raw_esize(STORE));
    s.bar = reinterpret_cast<uint64_t *>(s.prm + kStages * kChunk);
    s.red = reinterpret_cast<float2 *>(s.bar + kStages);
    return s;
}

struct TileGeo {
    double pcx, pcy, pcz;   // tile centre
    float qq_max;           // max |q|^2 over the tile
    float xT, yT;           // tile centre in pixel units from the grid origin (exact)
    float qqh, qql;         // |xT ux + yT uy|^2 as a float pair
};

// Per-pulse reference (FP64), relative to the grid origin O:
//   a0 = |O - apc|^2, a1 = 2 ux.(O - apc), a2 = 2 uy.(O - apc)
// stored as float pairs: pref[2p] = (a0h, a0l, a1h, a1l), pref[2p+1] = (a2h, a2l, 0, 0).
// With (xT, yT) a tile centre in pixel units, R_T^2 = a0 + xT a1 + yT a2 + |q_T|^2.
// Per-pulse references for the SPLIT path.  The optional corrections enter
// as a bin offset db = drange * (2 bin_rate / c) and a phase offset
// dph = 2 pi frac(drange * 2 fc / c) + dphase (wrapped to [-pi, pi]), applied to
// the tile-centre bin and phase, so they cost nothing per update.
__global__ void pulse_ref_kernel(const double *__restrict__ apc, int np, BpGeom g, const double *__restrict__ drange,
                                 const double *__restrict__ dphase, double bins_per_m, double cyc_per_m,
                                 float4 *__restrict__ pref) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const double dr = drange ? drange[p] : 0.0;
    const double cyc = dr * cyc_per_m;
    double dph = 2.0 * CUDART_PI * (cyc - rint(cyc)) + (dphase ? dphase[p] : 0.0);
    dph -= 2.0 * CUDART_PI * rint(dph * (0.5 / CUDART_PI));
    const double wx = g.origin[0] - apc[3 * p], wy = g.origin[1] - apc[3 * p + 1], wz = g.origin[2] - apc[3 * p + 2];
    const double a0 = fma(wx, wx, fma(wy, wy, wz * wz));
    const double a1 = 2.0 * (g.ux[0] * wx + g.ux[1] * wy + g.ux[2] * wz);
    const double a2 = 2.0 * (g.uy[0] * wx + g.uy[1] * wy + g.uy[2] * wz);
    const float a0h = (float)a0, a1h = (float)a1, a2h = (float)a2;
    pref[2 * p] = make_float4(a0h, (float)(a0 - (double)a0h), a1h, (float)(a1 - (double)a1h));
    pref[2 * p + 1] = make_float4(a2h, (float)(a2 - (double)a2h), (float)(dr * bins_per_m), (float)dph);
}

// After the wait for chunk c ran out: raise the timeout bit and let the copies
// still in flight land before the CTA's shared memory is released.  Every warp
// has issued chunks c and (if it exists) c + 1 and waited for all before them,
// so those two phases are the outstanding ones: wait for each on its own
// parity (chunk k is phase k / kStages of ring stage k % kStages).  Out of line:
// inlined, this cold path moved the main loop's schedule (config 2: 54.1 ms
// against 53.1 ms per launch).
template <bool TESTF>
__device__ __noinline__ void drain_after_timeout(const BpPlan &P, uint64_t *bars, int c, int nchunks) {
    atomicOr(P.err, kErrWaitTimeout);
    for (int k = c; k <= c + 1 && k < nchunks; ++k) {
        const unsigned bar = smem_addr(&bars[k % kStages]);
        if (TESTF && k == P.fault_chunk) mbar_complete_tx(bar, kFaultBytes);
        const uint64_t lim = TESTF && P.wait_ns > kDrainWaitNs ? P.wait_ns : kDrainWaitNs;
        if (!mbar_wait_bounded(bar, (k / kStages) & 1, lim)) atomicOr(P.err, kErrDrainTimeout);
    }
}

// Per-(tile, pulse) geometry, window and TMA issue for this warp's pulses of
// one chunk.  Every warp arrives once on the stage's barrier.  `fault` (tests
// only) arms warp 0's arrival with kFaultBytes that no copy delivers, so the
// phase cannot complete and the consumers' bounded wait runs out.
template <int MODE, int STORE, int PIX, bool LIN = false>
__device__ __forceinline__ void produce(const BpPlan &P, const Smem &S, int stage, int p0, int count,
                                        const TileGeo &T, bool fault) {
    constexpr int kTileY = 8 * PIX;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int win = P.win;
    const int esize = STORE == SARBP_STORE_C64 ? 8 : 4;
    const int slot = warp * kPerWarp + lane;
    unsigned bytes = 0;
    const char *src = nullptr;
    unsigned dst = 0;
    if (lane < kPerWarp && slot < count) {
        const int p = p0 + slot;
        const float bpm = P.kb_h;  // bins per metre of range
        const float hx = 0.5f * (kTileX - 1), hy = 0.5f * (kTileY - 1);
        const int cen = win >> 1;  // staged index origin
        Prm &q = S.prm[stage * kChunk + slot];
        int ws;  // window start, clamped to +-1e9 bins: int arithmetic throughout
        int need = win;
        bool sane;
        if (MODE == SARBP_MODE_SPLIT || MODE == SARBP_MODE_FP16STORE) {
            // R_T^2 = a0 + xT a1 + yT a2 + |q_T|^2 in float-float
            const float4 r0v = __ldg(&P.pref[2 * p]);
            const float4 r1v = __ldg(&P.pref[2 * p + 1]);
            const ff a0 = {r0v.x, r0v.y}, a1 = {r0v.z, r0v.w}, a2 = {r1v.x, r1v.y};
            const ff S2 = ff_add(ff_add(a0, ff_mul_f(a1, T.xT)), ff_add(ff_mul_f(a2, T.yT), ff{T.qqh, T.qql}));
            const float r = sqrtf(S2.h);
            const float corr = (fmaf(-r, r, S2.h) + S2.l) * (0.5f / r);  // R_T = r + corr
            // bin of the tile centre: (2 R_T / c - t0) * bin_rate
            const float kbh = P.kb_h, kbl = P.kb_l;
            float ph_ = r * kbh;
            float pl_ = fmaf(r, kbh, -ph_) + fmaf(r, kbl, corr * kbh);
            const ff bT = ff_add(ff_add(quick_two_sum(ph_, pl_), ff{-P.tb_h, -P.tb_l}), ff{r1v.z, 0.f});
            // carrier phase 2 pi frac(R_T * 2 fc / c)
            const float kch = P.kc_h, kcl = P.kc_l;
            const float cy = r * kch;
            const float cy_e = fmaf(r, kch, -cy) + fmaf(r, kcl, corr * kch);
            const float fr = (cy - rintf(cy)) + cy_e;
            const float phT = fmaf(fr, 6.28318530717958647692f, r1v.w);
            const float iR = 1.0f / r;
            const float A = r0v.z + 2.f * (T.xT * P.gf11 + T.yT * P.gf12);
            const float B = r1v.x + 2.f * (T.xT * P.gf12 + T.yT * P.gf22);
            const float half = bpm * (fabsf(A) * hx + fabsf(B) * hy + T.qq_max) * 0.5f * iR * 1.03f + 2.f;
            ws = (int)floorf(fminf(fmaxf(bT.h - half, -1.0e9f), 1.0e9f));
            ws &= ~3;
            const int need_end = (int)ceilf(fminf(fmaxf(bT.h + half, -1.0e9f), 1.0e9f)) + 2;
            sane = isfinite(r) && r > 0.f && isfinite(half) && isfinite(phT) && need_end - ws <= win;
            // the tile's bins lie in [bT - half, bT + half]: pair indices up to
            // need_end - ws - 2, so pairs [0, need) cover every read (the checked
            // build flags any read past need - 2)
            if (sane) need = need_end - ws;
            const float i2 = iR * iR;
            if (sane) {
                const float c1 = 0.5f * iR, c2 = -0.125f * iR * i2, c3 = 0.0625f * iR * i2 * i2;
                const float c4 = -0.0390625f * iR * i2 * i2 * i2;
                const float bb = ((bT.h - (float)ws) + bT.l) - 0.5f - (float)cen;
                if constexpr (LIN) {
                    // the series in m = n / (2 R_T): dR = m + m^2 (d2 + m (d3 + m d4)), and
                    // the phase's linear part from the increments per pixel step, half of
                    // 4 pi / lambda (u.w) / R_T reduced modulo 2 pi (the pixel offsets are
                    // half-integers, 2 xc and 2 yc integers), in float-float:
                    // u.w = a1 / 2 + xT g11 + yT g12 (x), a2 / 2 + xT g12 + yT g22 (y),
                    // 1 / R_T from iR and one Newton correction
                    const float d2 = -0.5f * iR, d3 = 0.5f * i2, d4 = -0.625f * i2 * iR;
                    const ff g11 = {P.gf11, P.gf11l}, g12 = {P.gf12, P.gf12l}, g22 = {P.gf22, P.gf22l};
                    const ff uxw = ff_add(ff{0.5f * a1.h, 0.5f * a1.l}, ff_add(ff_mul_f(g11, T.xT), ff_mul_f(g12, T.yT)));
                    const ff uyw = ff_add(ff{0.5f * a2.h, 0.5f * a2.l}, ff_add(ff_mul_f(g12, T.xT), ff_mul_f(g22, T.yT)));
                    const ff invR = quick_two_sum(iR, iR * (fmaf(-r, iR, 1.f) - corr * iR));
                    const ff kh = {0.5f * P.kp_h, 0.5f * P.kp_l};  // 2 pi fc / c
                    const float pxr = ff_mod_2pi(ff_mul(ff_mul(kh, uxw), invR));
                    const float pyr = ff_mod_2pi(ff_mul(ff_mul(kh, uyw), invR));
                    q.k0 = make_float4(c1, c1, d2, d2);
                    q.k1 = make_float4(d3, d3, d4, d4);
                    q.k2 = make_float4(bb, bb, phT, phT);
                    q.k3 = make_float4(A * c1, A * c1, B * c1, B * c1);
                    prm_k4(q) = make_float4(pxr, pxr, pyr, pyr);
                } else {
                    q.k0 = make_float4(c1, c1, c2, c2);
                    q.k1 = make_float4(c3, c3, c4, c4);
                    q.k2 = make_float4(bb, bb, phT, phT);
                    q.k3 = make_float4(A, A, B, B);
                }
            } else {  // inert pulse: every pixel reads the centre bin of an all-zero window
                q.k0 = q.k1 = q.k2 = q.k3 = make_float4(0.f, 0.f, 0.f, 0.f);
                if constexpr (LIN) prm_k4(q) = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        } else {
            const double ax = __ldg(&P.apc[3 * p]), ay = __ldg(&P.apc[3 * p + 1]), az = __ldg(&P.apc[3 * p + 2]);
            const double wx = T.pcx - ax, wy = T.pcy - ay, wz = T.pcz - az;
            const double dr = P.drange ? __ldg(&P.drange[p]) : 0.0;
            const double dph = P.dphase ? __ldg(&P.dphase[p]) : 0.0;
            const double R = sqrt(fma(wx, wx, fma(wy, wy, wz * wz))) + dr;
            const float iR = (float)(1.0 / R);
            const float wxf = (float)wx, wyf = (float)wy, wzf = (float)wz;
            const float A = 2.f * ((float)P.g.ux[0] * wxf + (float)P.g.ux[1] * wyf + (float)P.g.ux[2] * wzf);
            const float B = 2.f * ((float)P.g.uy[0] * wxf + (float)P.g.uy[1] * wyf + (float)P.g.uy[2] * wzf);
            const double bT = fma(R, 2.0 / P.c * P.bin_rate, -P.t0_bins * P.bin_rate);
            const float half = bpm * (fabsf(A) * hx + fabsf(B) * hy + T.qq_max) * 0.5f * iR * 1.03f + 2.f;
            const float bTf = (float)bT;
            ws = (int)floorf(fminf(fmaxf(bTf - half, -1.0e9f), 1.0e9f));
            ws &= ~3;
            const int need_end = (int)ceilf(fminf(fmaxf(bTf + half, -1.0e9f), 1.0e9f)) + 2;
            sane = isfinite(R) && R > 0.0 && isfinite(half) && need_end - ws <= win;
            if (MODE == SARBP_MODE_FP32) {
                const double kph_d = 4.0 * CUDART_PI * P.fc / P.c;
                q.k0 = make_float4((float)ax, (float)ay, (float)az,
                                   (float)(dr * (2.0 / P.c * P.bin_rate) - P.t0_bins * P.bin_rate - (double)ws - 0.5 -
                                           (double)cen));
                q.k1 = make_float4((float)(kph_d * dr + dph), 0.f, 0.f, 0.f);
            }
            q.dr = dr;
            q.dph = dph;
            q.ax = ax;
            q.ay = ay;
            q.az = az;
        }
        if (!sane) atomicOr(P.err, kErrWindow);
        const int lo = ws < 0 ? 0 : ws;
        int hi = ws + win > P.nbins ? P.nbins : ws + win;
        if (hi < lo || !sane) hi = lo;
        q.ws = ws;
        q.lo = lo - ws;
        q.hi = hi - ws;
        q.need = need;
        q.scale = STORE == SARBP_STORE_C32H ? __ldg(&P.scale[p]) : 1.f;
        if (hi > lo) {
            bytes = (unsigned)((hi - lo) * esize);
            src = reinterpret_cast<const char *>(P.rc) + ((size_t)p * P.nbins + (size_t)lo) * esize;
            dst = smem_addr(S.raw + ((size_t)stage * P.chunk + (size_t)slot) * win * esize + (size_t)(lo - ws) * esize);
        }
    }
    unsigned total = bytes;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
    const unsigned bar = smem_addr(&S.bar[stage]);
    if (fault && warp == 0) total += kFaultBytes;
    if (lane == 0) mbar_expect_tx_arrive(bar, total);
    __syncwarp();
    if (bytes) tma_bulk_g2s(dst, src, bytes, bar);
}

// raw window -> (mid, diff) pairs; bins outside [lo, hi) read as zero.
// Flat over (pulse, bin), used for complex64 rows.
template <int MODE, int STORE, bool TRIM>
__device__ __forceinline__ void convert_flat(const Smem &S, int stage, int sbuf, int count, int win, unsigned win_magic,
                                        int chunk) {
    const int total = count * win;
    float4 *st = S.staged + (size_t)sbuf * chunk * win;
    for (int e = threadIdx.x; e < total; e += kThreads) {
        const int pl = (int)__umulhi((unsigned)e, win_magic);
        const int i = e - pl * win;
        const Prm &q = S.prm[stage * kChunk + pl];
        if (TRIM && i >= q.need) continue;  // no pixel of the tile reads it
        const int lo = q.lo, hi = q.hi;
        const unsigned char *rw = S.raw + ((size_t)stage * chunk + pl) * win * raw_esize(STORE);
        float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
        if (STORE == SARBP_STORE_C64) {
            const float2 *r = reinterpret_cast<const float2 *>(rw);
            if (i >= lo && i < hi) a = r[i];
            if (i + 1 >= lo && i + 1 < hi) b = r[i + 1];
        } else {
            const __half2 *r = reinterpret_cast<const __half2 *>(rw);
            const float sc = q.scale;
            if (i >= lo && i < hi) a = __half22float2(r[i]);
            if (i + 1 >= lo && i + 1 < hi) b = __half22float2(r[i + 1]);
            a.x *= sc; a.y *= sc; b.x *= sc; b.y *= sc;
        }
        const float dx = b.x - a.x, dy = b.y - a.y;
        // FP32 arithmetic: pairs centred on the window middle, so that s = M + b d
        // takes the centred position b directly; FP64 keeps (mid, diff).
        const float o = MODE == SARBP_MODE_FP64 ? 0.f : (float)(i - (win >> 1));
        st[e] = make_float4(fmaf(-o, dx, 0.5f * (a.x + b.x)), fmaf(-o, dy, 0.5f * (a.y + b.y)), dx, dy);
    }
}

// The same with one warp per pulse (pulse-uniform bounds and scale, lane =
// bin) and an unconditional path when the whole window was copied (every pulse
// but those at the swath edges), used for complex16 rows.
template <int MODE, int STORE, bool TRIM>
__device__ __forceinline__ void convert_warp(const Smem &S, int stage, int sbuf, int count, int win, int chunk) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cen = win >> 1;
    float4 *stb = S.staged + (size_t)sbuf * chunk * win;
    for (int pl = warp; pl < count; pl += kWarps) {
        const Prm &q = S.prm[stage * kChunk + pl];
        const int lo = q.lo, hi = q.hi;
        const float sc = STORE == SARBP_STORE_C32H ? q.scale : 1.f;
        const unsigned char *rw = S.raw + ((size_t)stage * chunk + pl) * win * raw_esize(STORE);
        float4 *st = stb + (size_t)pl * win;
        const bool whole = lo == 0 && hi == win;
        const int n = TRIM ? q.need : win;  // pairs any pixel of the tile reads
        for (int i = lane; i < n; i += 32) {
            float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
            const bool ina = whole || (i >= lo && i < hi);
            const bool inb = whole ? i + 1 < win : (i + 1 >= lo && i + 1 < hi);
            if (STORE == SARBP_STORE_C64) {
                const float2 *r = reinterpret_cast<const float2 *>(rw);
                if (ina) a = r[i];
                if (inb) b = r[i + 1];
            } else {
                const __half2 *r = reinterpret_cast<const __half2 *>(rw);
                if (ina) a = __half22float2(r[i]);
                if (inb) b = __half22float2(r[i + 1]);
                a.x *= sc; a.y *= sc; b.x *= sc; b.y *= sc;
            }
            const float dx = b.x - a.x, dy = b.y - a.y;
            // FP32 arithmetic: pairs centred on the window middle, so that s = M + b d
            // takes the centred position b directly; FP64 keeps (mid, diff).
            const float o = MODE == SARBP_MODE_FP64 ? 0.f : (float)(i - cen);
            st[i] = make_float4(fmaf(-o, dx, 0.5f * (a.x + b.x)), fmaf(-o, dy, 0.5f * (a.y + b.y)), dx, dy);
        }
    }
}

// Measured per storage on config 2 (Gupd/s, flat / warp-per-pulse): complex64
// 1275.7 / 1241.5, complex16 1231.5 / 1244.8.  The pass itself is ~6% of the
// kernel (3.1 ms of 53.9 without it), but its code shape moves the schedule
// of the main loop more than its own cost.
// TRIM: convert only the pairs [0, need) the tile reads (unchecked SPLIT /
// FP16STORE kernels); the checked build and the FP32 / FP64 comparators clamp
// reads anywhere in the window and convert all of it.
template <int MODE, int STORE, bool TRIM>
__device__ __forceinline__ void convert(const Smem &S, int stage, int sbuf, int count, int win, unsigned win_magic,
                                        int chunk) {
    if constexpr (STORE == SARBP_STORE_C32H)
        convert_warp<MODE, STORE, TRIM>(S, stage, sbuf, count, win, chunk);
    else
        convert_flat<MODE, STORE, TRIM>(S, stage, sbuf, count, win, win_magic, chunk);
}

// Sum of the warps' projections for the pulses of one chunk into
// proj[tile][pulse] (fixed order: deterministic).
__device__ __forceinline__ void flush_projection(const BpPlan &P, const Smem &S, int buf, int p0, int count) {
    const int t = threadIdx.x;
    if (t < count) {
        float sr = 0.f, si = 0.f;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const float2 v = S.red[(buf * kWarps + w) * kChunk + t];
            sr += v.x;
            si += v.y;
        }
        P.proj[(size_t)blockIdx.x * P.np + p0 + t] = make_float2(sr, si);
    }
}

// One chunk of the weighted projection: per pulse, this thread's sum over its
// pixels of conj(w) * term, then the warp's sum into red[2 pulse + {re, im}].
// conj(w) e^{i phi} = |w| e^{i (phi - arg w)}: the weight's phase joins the
// packed phase (half an op per pixel) and its magnitude scales cos / sin, so
// the weighted accumulate costs 6.5 FP32 ops instead of 8.
// Pulses go in pairs through one shared butterfly: the xor-16 step splits the
// pair's two pulses between the half-warps and the xor-8 step splits re / im,
// so a pair costs 6 shuffles instead of 20 for two separate 32-lane sums.
// LIN: the linear-term phase (as the back-projection's LIN loop), the weight's
// phase added to it the same way.
template <int NTERMS, int PIX, bool LIN>
__device__ __forceinline__ void project_chunk(const Smem &S, int stage, int count, int win, unsigned sbase, int cen,
                                              f2 XC2, const f2 (&YC2)[PIX / 2], const f2 (&QQ2)[PIX / 2], f2 BPM2,
                                              f2 KH2, f2 KL2, const f2 (&TH2)[PIX / 2], const float (&wm)[PIX],
                                              f2 X2C2, const f2 (&Y2C2)[LIN ? PIX / 2 : 1], float *red) {
    const int lane = threadIdx.x & 31;
    const bool hi16 = (lane & 16) != 0, hi8 = (lane & 8) != 0;
    f2 MP = pk2(kMagic + (float)cen, kMagic + (float)cen);
    const f2 WIN2 = pk2((float)win, (float)win);
#pragma unroll 1
    for (int pl = 0; pl < count; pl += 2) {
        float tr[2] = {0.f, 0.f}, ti[2] = {0.f, 0.f};
#pragma unroll
        for (int u2 = 0; u2 < 2; ++u2) {
            if (u2 == 1 && pl + 1 >= count) break;  // odd tail: pulse-uniform
            const Prm &q = S.prm[stage * kChunk + pl + u2];
            // k0..k3 (and k4 for LIN) as the producer wrote them: (C1, C2 | D2),
            // (C3 | D3, C4 | D4), (BT, PHT), (A | A c1, B | B c1), (PX, PY)
            f2 C1, C2, C3, C4, BT, PHT, AA, BB, PX, PY;
            lds2x2(&q.k0, C1, C2);
            lds2x2(&q.k1, C3, C4);
            lds2x2(&q.k2, BT, PHT);
            lds2x2(&q.k3, AA, BB);
            f2 PHX = PHT;
            if constexpr (LIN) {
                lds2x2(&prm_k4(q), PX, PY);
                PHX = ffma2(X2C2, PX, PHT);
            }
            const f2 XA = fmul2(XC2, AA);
#pragma unroll
            for (int h = 0; h < PIX / 2; ++h) {
                f2 b2, ph2;
                if constexpr (LIN) {
                    const f2 qc = fmul2(QQ2[h], C1);
                    const f2 m = ffma2(YC2[h], BB, fadd2(XA, qc));
                    const f2 m2 = fmul2(m, m);
                    const f2 poly = NTERMS == 4 ? ffma2(m, ffma2(m, C4, C3), C2) : ffma2(m, C3, C2);
                    b2 = ffma2(ffma2(m2, poly, m), BPM2, BT);
                    ph2 = fadd2(ffma2(ffma2(m2, poly, qc), KH2, ffma2(Y2C2[h], PY, PHX)), TH2[h]);
                } else {
                    const f2 n = ffma2(YC2[h], BB, fadd2(XA, QQ2[h]));
                    f2 poly = NTERMS == 4 ? ffma2(n, ffma2(n, C4, C3), C2) : ffma2(n, C3, C2);
                    poly = ffma2(n, poly, C1);
                    const f2 dR = fmul2(n, poly);
                    b2 = ffma2(dR, BPM2, BT);
#if SARBP_BP_PHASE_COMPENSATED
                    ph2 = fadd2(ffma2(dR, KL2, ffma2(dR, KH2, PHT)), TH2[h]);
#else
                    ph2 = fadd2(ffma2(dR, KH2, PHT), TH2[h]);
#endif
                }
                float bb[2], ph[2], tt[2];
                upk2(b2, bb[0], bb[1]);
                upk2(ph2, ph[0], ph[1]);
                upk2(fadd2(b2, MP), tt[0], tt[1]);
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int j = 2 * h + u;
                    const float4 v = lds128((__float_as_uint(tt[u]) << 4) + sbase);
                    const float sr = fmaf(bb[u], v.z, v.x);
                    const float si = fmaf(bb[u], v.w, v.y);
                    float sn, cs;
                    __sincosf(ph[u], &sn, &cs);
                    const float zr = wm[j] * cs, zi = wm[j] * sn;
                    tr[u2] = fmaf(sr, zr, fmaf(-si, zi, tr[u2]));
                    ti[u2] = fmaf(sr, zi, fmaf(si, zr, ti[u2]));
                }
            }
            MP = fadd2(MP, WIN2);
        }
        float k0 = hi16 ? tr[1] : tr[0], k1 = hi16 ? ti[1] : ti[0];
        k0 += __shfl_xor_sync(0xffffffffu, hi16 ? tr[0] : tr[1], 16);
        k1 += __shfl_xor_sync(0xffffffffu, hi16 ? ti[0] : ti[1], 16);
        float k = hi8 ? k1 : k0;
        k += __shfl_xor_sync(0xffffffffu, hi8 ? k0 : k1, 8);
        k += __shfl_xor_sync(0xffffffffu, k, 4);
        k += __shfl_xor_sync(0xffffffffu, k, 2);
        k += __shfl_xor_sync(0xffffffffu, k, 1);
        const int pp = pl + (hi16 ? 1 : 0);
        if ((lane & 7) == 0 && pp < count) red[2 * pp + (hi8 ? 1 : 0)] = k;
    }
}

// ADJ: weighted projection (the adjoint) instead of back-projection: every
// pixel's term of pulse p is multiplied by conj(weight[pixel]) and summed over
// the tile into proj[tile][p] (SPLIT / FP16STORE arithmetic).
// CHUNK: pulses per staged chunk fixed at compile time (the hot unchecked
// SPLIT / FP16STORE case at 16), or 0 to take the planner's P.chunk.
// TESTF: the waits take their limit from P.wait_ns and P.fault_chunk arms one
// chunk's barrier so that its wait runs out (tests of the timeout path, through
// sarbp_debug_set); production variants wait 2 s and carry no injector.
template <int MODE, int STORE, int NTERMS, bool CHECKED, int PIX, bool ADJ = false, int CHUNK = 0, bool TESTF = false,
          bool LIN = false>
__global__ void __launch_bounds__(kThreads, SARBP_BP_MINBLOCKS)
    bp_kernel(const __grid_constant__ BpPlan P, int tiles_y, int pulses_per_seg, float qq_max) {
    static_assert(!ADJ || MODE == SARBP_MODE_SPLIT || MODE == SARBP_MODE_FP16STORE, "projection: split arithmetic");
    static_assert(!LIN || MODE == SARBP_MODE_SPLIT || MODE == SARBP_MODE_FP16STORE,
                  "linear-term phase: split arithmetic only");
    constexpr int kPix = PIX;  // pixels per thread, all in one column
    constexpr int kTileY = 8 * PIX;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int win = P.win;
    const int chunk = CHUNK ? CHUNK : P.chunk;  // pulses per staged chunk: 16, 8 or 4 (two CTAs per SM)
    const Smem S = carve<STORE>(smem_raw, win, chunk);
    const unsigned win_magic = (unsigned)((0xFFFFFFFFull + (unsigned long long)win) / (unsigned long long)win);

    const int tile = blockIdx.x;
    const int ty = tile % tiles_y;  // tiles sharing a range strip run together (L2 reuse)
    const int tx = tile / tiles_y;
    const int seg = blockIdx.y;
    const int p_begin = seg * pulses_per_seg;
    const int p_end = min(P.np, p_begin + pulses_per_seg);
    const int nchunks = p_end > p_begin ? (p_end - p_begin + chunk - 1) / chunk : 0;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int lx = lane >> 2, ly = lane & 3;
    const int xl = (warp & 3) * 8 + lx;
    const float xc = (float)xl - 0.5f * (kTileX - 1);
    float yc[kPix], qq[kPix];
    const float g11 = P.gf11, g12 = P.gf12, g22 = P.gf22;
#pragma unroll
    for (int j = 0; j < kPix; ++j) {
        const int yl = ((warp >> 2) + 2 * j) * 4 + ly;
        yc[j] = (float)yl - 0.5f * (kTileY - 1);
        qq[j] = xc * xc * g11 + 2.f * xc * yc[j] * g12 + yc[j] * yc[j] * g22;
    }
    TileGeo T;
    {
        const double pcx_i = tx * kTileX + 0.5 * (kTileX - 1), pcy_i = ty * kTileY + 0.5 * (kTileY - 1);
        T.pcx = P.g.origin[0] + pcx_i * P.g.ux[0] + pcy_i * P.g.uy[0];
        T.pcy = P.g.origin[1] + pcx_i * P.g.ux[1] + pcy_i * P.g.uy[1];
        T.pcz = P.g.origin[2] + pcx_i * P.g.ux[2] + pcy_i * P.g.uy[2];
        T.qq_max = qq_max;
        T.xT = (float)pcx_i;
        T.yT = (float)pcy_i;
        T.qqh = T.qql = 0.f;
        if (lane < kPerWarp) {  // producer lanes only: FP64 once per CTA
            const double qq = pcx_i * pcx_i * P.g.g11 + 2.0 * pcx_i * pcy_i * P.g.g12 + pcy_i * pcy_i * P.g.g22;
            T.qqh = (float)qq;
            T.qql = (float)(qq - (double)T.qqh);
        }
    }
    const int cen = win >> 1;
    const float cenf = (float)cen;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(smem_addr(&S.bar[s]), kWarps);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();

    float acc_r[kPix], acc_i[kPix];
    double dacc_r[MODE == SARBP_MODE_FP64 ? kPix : 1], dacc_i[MODE == SARBP_MODE_FP64 ? kPix : 1];
#pragma unroll
    for (int j = 0; j < kPix; ++j) { acc_r[j] = 0.f; acc_i[j] = 0.f; }
#pragma unroll
    for (int j = 0; j < (MODE == SARBP_MODE_FP64 ? kPix : 1); ++j) { dacc_r[j] = 0.0; dacc_i[j] = 0.0; }

    const float bpm = P.kb_h;
    const float kph_hi = P.kp_h, kph_lo = P.kp_l;  // 4 pi fc / c as a float pair
    const float wmax = (float)(win - 2);

    // weighted projection: |weight| and -arg(weight) of this thread's pixels
    // (zero outside the grid)
    float wm[ADJ ? kPix : 1], wth[ADJ ? kPix : 1];
    if constexpr (ADJ) {
#pragma unroll
        for (int j = 0; j < kPix; ++j) {
            const int x = tx * kTileX + xl, y = ty * kTileY + ((warp >> 2) + 2 * j) * 4 + ly;
            float2 w = make_float2(0.f, 0.f);
            if (x < P.g.nx && y < P.g.ny) w = __ldg(&P.weight[(size_t)y * P.g.nx + x]);
            wm[j] = hypotf(w.x, w.y);
            wth[j] = -atan2f(w.y, w.x);
        }
    }

    float fpy[kPix], fpz[kPix], fpxx[kPix];
    if (MODE == SARBP_MODE_FP32) {
#pragma unroll
        for (int j = 0; j < kPix; ++j) {
            const double xi = tx * kTileX + xl, yi = ty * kTileY + ((warp >> 2) + 2 * j) * 4 + ly;
            fpxx[j] = (float)(P.g.origin[0] + xi * P.g.ux[0] + yi * P.g.uy[0]);
            fpy[j] = (float)(P.g.origin[1] + xi * P.g.ux[1] + yi * P.g.uy[1]);
            fpz[j] = (float)(P.g.origin[2] + xi * P.g.ux[2] + yi * P.g.uy[2]);
        }
    }

    const f2 XC2 = pk2(xc, xc);
    const f2 BPM2 = pk2(bpm, bpm), KH2 = pk2(kph_hi, kph_hi), KL2 = pk2(kph_lo, kph_lo);
    f2 YC2[kPix / 2], QQ2[kPix / 2], TH2[ADJ ? kPix / 2 : 1], Y2C2[LIN ? kPix / 2 : 1];
#pragma unroll
    for (int h = 0; h < kPix / 2; ++h) {
        YC2[h] = pk2(yc[2 * h], yc[2 * h + 1]);
        QQ2[h] = pk2(qq[2 * h], qq[2 * h + 1]);
        if constexpr (ADJ) TH2[h] = pk2(wth[2 * h], wth[2 * h + 1]);
        if constexpr (LIN) Y2C2[h] = pk2(2.f * yc[2 * h], 2.f * yc[2 * h + 1]);
    }
    const f2 X2C2 = pk2(2.f * xc, 2.f * xc);

    if (nchunks > 0)
        produce<MODE, STORE, PIX, LIN>(P, S, 0, p_begin, min(chunk, p_end - p_begin), T, TESTF && P.fault_chunk == 0);

    bool failed = false;
    bool clamped = false;
    int c = 0;  // after a failed wait, the chunk it was for
#pragma unroll 1
    for (; c < nchunks; ++c) {
        const int stage = c % kStages;
        const int sbuf = c & 1;
        const int pc0 = p_begin + c * chunk;
        const int count = min(chunk, p_end - pc0);
        if (c + 1 < nchunks) {
            const int pn = pc0 + chunk;
            produce<MODE, STORE, PIX, LIN>(P, S, (c + 1) % kStages, pn, min(chunk, p_end - pn), T,
                                      TESTF && P.fault_chunk == c + 1);
        }
        const bool ok =
            mbar_wait_bounded(smem_addr(&S.bar[stage]), (c / kStages) & 1, TESTF ? P.wait_ns : kDefaultWaitNs);
        if (!ok) { failed = true; }
        // One block barrier per chunk, after the conversion: each thread has seen
        // its own wait complete, the chunk's parameters were published by the
        // previous chunk's barrier, and a thread whose wait ran out converts
        // in-bounds shared memory only before the barrier's vote ends the loop
        // (config 2 53.04 -> 52.64 ms against a barrier on each side, same bits).
        // trimmed to the pairs the tile reads for complex16 rows (warp per pulse:
        // config 5 892 -> 864 ms); the flat complex64 pass measured slower with
        // the per-element test (config 2 1296 -> 1283 Gupd/s), and complex64 rows
        // through the trimmed warp-per-pulse pass tied with it (1300.2 vs
        // 1301-1303), so complex64 converts the whole window
        convert<MODE, STORE,
                !CHECKED && STORE == SARBP_STORE_C32H && (MODE == SARBP_MODE_SPLIT || MODE == SARBP_MODE_FP16STORE)>(
            S, stage, sbuf, count, win, win_magic, chunk);
        if (__syncthreads_or(failed)) { failed = true; break; }
        if constexpr (ADJ) {  // every warp has finished chunk c-1: combine its pulse sums
            if (c > 0) flush_projection(P, S, (c - 1) & 1, pc0 - chunk, chunk);
        }

        const float4 *stg = S.staged + (size_t)sbuf * chunk * win;
        const unsigned sbase = smem_addr(stg) - kMagicBitsShift4;
        if constexpr (ADJ) {
            project_chunk<NTERMS, kPix, LIN>(S, stage, count, win, sbase, cen, XC2, YC2, QQ2, BPM2, KH2, KL2, TH2, wm,
                                             X2C2, Y2C2, reinterpret_cast<float *>(S.red + ((c & 1) * kWarps + warp) * kChunk));
        } else if (LIN && (MODE == SARBP_MODE_SPLIT || MODE == SARBP_MODE_FP16STORE)) {
            // linear-term form (large tiles): m = n / (2 R_T) centred offset, bin from
            // dR = m + m^2 poly(m), phase from the increments per pixel step (reduced
            // modulo 2 pi per pulse) plus 4 pi / lambda times the nonlinear remainder
            // qq c1 + m^2 poly(m), so no FP32 quantity of the size of the tile's
            // extent enters the phase
            f2 MP = pk2(kMagic + (float)cen, kMagic + (float)cen);
            const f2 WIN2 = pk2((float)win, (float)win);
#pragma unroll kPulseUnroll
            for (int pl = 0; pl < count; ++pl) {
                const Prm &q = S.prm[stage * kChunk + pl];
                f2 C1, D2, D3, D4, BT, PHT, AP, BP, PX, PY;
                lds2x2(&q.k0, C1, D2);
                lds2x2(&q.k1, D3, D4);
                lds2x2(&q.k2, BT, PHT);
                lds2x2(&q.k3, AP, BP);
                lds2x2(&prm_k4(q), PX, PY);
                const f2 XAP = fmul2(XC2, AP);
                const f2 PHX = ffma2(X2C2, PX, PHT);
#pragma unroll
                for (int h = 0; h < kPix / 2; ++h) {
                    const f2 qc = fmul2(QQ2[h], C1);
                    const f2 m = ffma2(YC2[h], BP, fadd2(XAP, qc));
                    const f2 m2 = fmul2(m, m);
                    const f2 poly = NTERMS == 4 ? ffma2(m, ffma2(m, D4, D3), D2) : ffma2(m, D3, D2);
                    const f2 dR = ffma2(m2, poly, m);
                    f2 b2 = ffma2(dR, BPM2, BT);  // bin positions relative to the window middle
                    const f2 nl = ffma2(m2, poly, qc);
                    const f2 ph2 = ffma2(nl, KH2, ffma2(Y2C2[h], PY, PHX));
                    float bb[2], ph[2];
                    upk2(b2, bb[0], bb[1]);
                    upk2(ph2, ph[0], ph[1]);
                    if (CHECKED) {
                        const float needf = (float)(q.need - 2) - cenf;
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            const float bc = fminf(fmaxf(bb[u], -cenf), wmax - cenf);
                            clamped |= !(bc == bb[u]) || bb[u] > needf;
                            bb[u] = bc;
                        }
                        b2 = pk2(bb[0], bb[1]);
                    }
                    const f2 t2 = fadd2(b2, MP);
                    float tt[2];
                    upk2(t2, tt[0], tt[1]);
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const int j = 2 * h + u;
                        const float4 v = lds128((__float_as_uint(tt[u]) << 4) + sbase);
                        const float sr = fmaf(bb[u], v.z, v.x);
                        const float si = fmaf(bb[u], v.w, v.y);
                        float sn, cs;
                        __sincosf(ph[u], &sn, &cs);
                        acc_r[j] = fmaf(sr, cs, fmaf(-si, sn, acc_r[j]));
                        acc_i[j] = fmaf(sr, sn, fmaf(si, cs, acc_i[j]));
                    }
                }
                MP = fadd2(MP, WIN2);
            }
        } else if (MODE == SARBP_MODE_SPLIT || MODE == SARBP_MODE_FP16STORE) {
            // geometry, bin and phase for pixel pairs (2j, 2j+1) in packed FP32x2;
            // interpolation and the complex accumulate per pixel
            f2 MP = pk2(kMagic + (float)cen, kMagic + (float)cen);
            const f2 WIN2 = pk2((float)win, (float)win);
#pragma unroll kPulseUnroll
            for (int pl = 0; pl < count; ++pl) {
                const Prm &q = S.prm[stage * kChunk + pl];
                f2 C1, C2, C3, C4, BT, PHT, AA, BB;
                lds2x2(&q.k0, C1, C2);
                lds2x2(&q.k1, C3, C4);
                lds2x2(&q.k2, BT, PHT);
                lds2x2(&q.k3, AA, BB);
                const f2 XA = fmul2(XC2, AA);
#pragma unroll
                for (int h = 0; h < kPix / 2; ++h) {
                    const f2 n = ffma2(YC2[h], BB, fadd2(XA, QQ2[h]));
                    f2 poly = NTERMS == 4 ? ffma2(n, ffma2(n, C4, C3), C2) : ffma2(n, C3, C2);
                    poly = ffma2(n, poly, C1);
                    const f2 dR = fmul2(n, poly);
                    f2 b2 = ffma2(dR, BPM2, BT);  // bin positions relative to the window middle
#if SARBP_BP_PHASE_COMPENSATED
                    const f2 ph2 = ffma2(dR, KL2, ffma2(dR, KH2, PHT));
#else
                    const f2 ph2 = ffma2(dR, KH2, PHT);
#endif
                    float bb[2], ph[2];
                    upk2(b2, bb[0], bb[1]);
                    upk2(ph2, ph[0], ph[1]);
                    if (CHECKED) {
                        // past the window, or past the pairs an unchecked kernel converts
                        const float needf = (float)(q.need - 2) - cenf;
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            const float bc = fminf(fmaxf(bb[u], -cenf), wmax - cenf);
                            clamped |= !(bc == bb[u]) || bb[u] > needf;
                            bb[u] = bc;
                        }
                        b2 = pk2(bb[0], bb[1]);
                    }
                    const f2 t2 = fadd2(b2, MP);
                    float tt[2];
                    upk2(t2, tt[0], tt[1]);
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const int j = 2 * h + u;
                        const float4 v = lds128((__float_as_uint(tt[u]) << 4) + sbase);
                        const float sr = fmaf(bb[u], v.z, v.x);
                        const float si = fmaf(bb[u], v.w, v.y);
                        float sn, cs;
                        __sincosf(ph[u], &sn, &cs);
                        acc_r[j] = fmaf(sr, cs, fmaf(-si, sn, acc_r[j]));
                        acc_i[j] = fmaf(sr, sn, fmaf(si, cs, acc_i[j]));
                    }
                }
                MP = fadd2(MP, WIN2);
            }
        } else if (MODE == SARBP_MODE_FP32) {
#pragma unroll 1
            for (int pl = 0; pl < count; ++pl) {
                const Prm &q = S.prm[stage * kChunk + pl];
                const float4 k0 = q.k0;
                const float phc = q.k1.x;  // per-pulse phase correction
                const float mp = kMagic + (float)(pl * win + cen);
                const float kph = kph_hi;
#pragma unroll
                for (int j = 0; j < kPix; ++j) {
                    const float dx = k0.x - fpxx[j], dy = k0.y - fpy[j], dz = k0.z - fpz[j];
                    const float R = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
                    float b = fmaf(R, bpm, k0.w);
                    b = fminf(fmaxf(b, -cenf), wmax - cenf);
                    const float t = b + mp;
                    const float4 v = lds128((__float_as_uint(t) << 4) + sbase);
                    const float sr = fmaf(b, v.z, v.x);
                    const float si = fmaf(b, v.w, v.y);
                    float sn, cs;
                    sincosf(fmaf(kph, R, phc), &sn, &cs);
                    acc_r[j] = fmaf(sr, cs, fmaf(-si, sn, acc_r[j]));
                    acc_i[j] = fmaf(sr, sn, fmaf(si, cs, acc_i[j]));
                }
            }
        } else {  // FP64
            const double cyc_per_m = 2.0 * P.fc / P.c;
#pragma unroll 1
            for (int pl = 0; pl < count; ++pl) {
                const Prm &q = S.prm[stage * kChunk + pl];
                const double ax = q.ax, ay = q.ay, az = q.az, dr = q.dr, dph_pi = q.dph / CUDART_PI;
                const double boff = -P.t0_bins * P.bin_rate - (double)q.ws;
                const float4 *st = stg + pl * win;
#pragma unroll
                for (int j = 0; j < kPix; ++j) {
                    const double xi = tx * kTileX + xl, yi = ty * kTileY + ((warp >> 2) + 2 * j) * 4 + ly;
                    const double px = P.g.origin[0] + xi * P.g.ux[0] + yi * P.g.uy[0];
                    const double py = P.g.origin[1] + xi * P.g.ux[1] + yi * P.g.uy[1];
                    const double pz = P.g.origin[2] + xi * P.g.ux[2] + yi * P.g.uy[2];
                    const double dx = ax - px, dy = ay - py, dz = az - pz;
                    const double R = sqrt(dx * dx + dy * dy + dz * dz) + dr;
                    double b = fma(R, 2.0 / P.c * P.bin_rate, boff) - 0.5;
                    b = fmin(fmax(b, 0.0), (double)(win - 2));
                    const double r0 = rint(b);
                    const double f = b - r0;
                    const float4 v = st[(int)r0];
                    const double sr = fma(f, (double)v.z, (double)v.x);
                    const double si = fma(f, (double)v.w, (double)v.y);
                    const double cyc = cyc_per_m * R;
                    double sn, cs;
                    sincospi(2.0 * (cyc - rint(cyc)) + dph_pi, &sn, &cs);
                    dacc_r[j] = fma(sr, cs, fma(-si, sn, dacc_r[j]));
                    dacc_i[j] = fma(sr, sn, fma(si, cs, dacc_i[j]));
                }
            }
        }
    }

    if (CHECKED && clamped) atomicOr(P.err, kErrIndexClamp);
    if (failed) {
        if (threadIdx.x == 0) drain_after_timeout<TESTF>(P, S.bar, c, nchunks);
        __syncthreads();
        return;
    }

    if constexpr (ADJ) {
        if (nchunks > 0) {
            __syncthreads();
            const int last = nchunks - 1;
            flush_projection(P, S, last & 1, p_begin + last * chunk, min(chunk, p_end - p_begin - last * chunk));
        }
        return;
    }

    // write the tile
    float2 *dst = P.segments > 1 ? P.partial + (size_t)seg * P.g.nx * P.g.ny : P.image;
    const bool acc_mode = P.segments == 1 && P.accumulate;
    const int x = tx * kTileX + xl;
#pragma unroll
    for (int j = 0; j < kPix; ++j) {
        const int y = ty * kTileY + ((warp >> 2) + 2 * j) * 4 + ly;
        if (x < P.g.nx && y < P.g.ny) {
            float2 v = MODE == SARBP_MODE_FP64 ? make_float2((float)dacc_r[j], (float)dacc_i[j])
                                               : make_float2(acc_r[j], acc_i[j]);
            const size_t idx = (size_t)y * P.g.nx + x;
            if (acc_mode) {
                const float2 o = dst[idx];
                v.x += o.x;
                v.y += o.y;
            }
            dst[idx] = v;
        }
    }
}

// image (=|+=) sum over segments of the partial images, fixed order.
__global__ void reduce_segments_kernel(const float2 *__restrict__ partial, int segments, size_t count,
                                       float2 *__restrict__ image, int accumulate) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count;
         i += (size_t)gridDim.x * blockDim.x) {
        float2 s = accumulate ? image[i] : make_float2(0.f, 0.f);
        for (int k = 0; k < segments; ++k) {
            const float2 v = __ldg(&partial[(size_t)k * count + i]);
            s.x += v.x;
            s.y += v.y;
        }
        image[i] = s;
    }
}

// When set (bp_occupancy), the dispatch below reports the chosen variant's
// resident CTAs per SM there instead of launching it.
thread_local int *t_occupancy = nullptr;

template <int MODE, int STORE, int NTERMS, bool CHECKED, int PIX, bool ADJ = false, int CHUNK = 0, bool TESTF = false,
          bool LIN = false>
cudaError_t launch_variant(const BpPlan &p, cudaStream_t s, int tiles, int tiles_y, int pps, float qq_max) {
    if (CHUNK && p.chunk != CHUNK) return cudaErrorInvalidValue;
    auto k = bp_kernel<MODE, STORE, NTERMS, CHECKED, PIX, ADJ, CHUNK, TESTF, LIN>;
    const size_t smem = bp_smem_bytes(STORE, p.win, p.chunk);
    cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void *>(k));
    if (e != cudaSuccess) return e;
    if (t_occupancy) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(t_occupancy, k, kThreads, smem);
    dim3 grid(tiles, p.segments);
    k<<<grid, kThreads, smem, s>>>(p, tiles_y, pps, qq_max);
    return cudaGetLastError();
}

template <int MODE, int STORE, int PIX>
cudaError_t launch_split(const BpPlan &p, cudaStream_t s, int tiles, int tiles_y, int pps, float qq_max) {
    if (p.lin) {  // large tiles: the linear-term phase
        if (p.checked)
            return p.nterms == 3 ? launch_variant<MODE, STORE, 3, true, PIX, false, 0, false, true>(p, s, tiles, tiles_y, pps, qq_max)
                                 : launch_variant<MODE, STORE, 4, true, PIX, false, 0, false, true>(p, s, tiles, tiles_y, pps, qq_max);
        if (p.chunk == kChunk)
            return p.nterms == 3 ? launch_variant<MODE, STORE, 3, false, PIX, false, kChunk, false, true>(p, s, tiles, tiles_y, pps, qq_max)
                                 : launch_variant<MODE, STORE, 4, false, PIX, false, kChunk, false, true>(p, s, tiles, tiles_y, pps, qq_max);
        return p.nterms == 3 ? launch_variant<MODE, STORE, 3, false, PIX, false, 0, false, true>(p, s, tiles, tiles_y, pps, qq_max)
                             : launch_variant<MODE, STORE, 4, false, PIX, false, 0, false, true>(p, s, tiles, tiles_y, pps, qq_max);
    }
    if (p.checked)
        return p.nterms == 3 ? launch_variant<MODE, STORE, 3, true, PIX>(p, s, tiles, tiles_y, pps, qq_max)
                             : launch_variant<MODE, STORE, 4, true, PIX>(p, s, tiles, tiles_y, pps, qq_max);
    if (p.chunk == kChunk)
        return p.nterms == 3 ? launch_variant<MODE, STORE, 3, false, PIX, false, kChunk>(p, s, tiles, tiles_y, pps, qq_max)
                             : launch_variant<MODE, STORE, 4, false, PIX, false, kChunk>(p, s, tiles, tiles_y, pps, qq_max);
    return p.nterms == 3 ? launch_variant<MODE, STORE, 3, false, PIX>(p, s, tiles, tiles_y, pps, qq_max)
                         : launch_variant<MODE, STORE, 4, false, PIX>(p, s, tiles, tiles_y, pps, qq_max);
}

// A plan asks for the test variants when it carries a fault or a wait limit
// other than the default (sarbp_debug_set); they exist for 8-pixel columns.
bool bp_testing(const BpPlan &p) { return p.fault_chunk >= 0 || p.wait_ns != kDefaultWaitNs; }

template <int MODE, int STORE, bool ADJ>
cudaError_t launch_testf_mode(const BpPlan &p, cudaStream_t s, int tiles, int tiles_y, int pps, float qq_max) {
    if constexpr (MODE == SARBP_MODE_SPLIT || MODE == SARBP_MODE_FP16STORE)
        return p.nterms == 3 ? launch_variant<MODE, STORE, 3, false, 8, ADJ, 0, true>(p, s, tiles, tiles_y, pps, qq_max)
                             : launch_variant<MODE, STORE, 4, false, 8, ADJ, 0, true>(p, s, tiles, tiles_y, pps, qq_max);
    else
        return launch_variant<MODE, STORE, 4, false, 8, false, 0, true>(p, s, tiles, tiles_y, pps, qq_max);
}

template <bool ADJ>
cudaError_t launch_testf(const BpPlan &p, cudaStream_t s, int tiles, int tiles_y, int pps, float qq_max) {
    if (p.pix != 8) return cudaErrorNotSupported;
    const bool fp16 = p.storage == SARBP_STORE_C32H;
    if constexpr (ADJ)
        return fp16 ? launch_testf_mode<SARBP_MODE_SPLIT, SARBP_STORE_C32H, true>(p, s, tiles, tiles_y, pps, qq_max)
                    : launch_testf_mode<SARBP_MODE_SPLIT, SARBP_STORE_C64, true>(p, s, tiles, tiles_y, pps, qq_max);
    switch (p.mode) {
        case SARBP_MODE_FP64:
            return fp16 ? launch_testf_mode<SARBP_MODE_FP64, SARBP_STORE_C32H, false>(p, s, tiles, tiles_y, pps, qq_max)
                        : launch_testf_mode<SARBP_MODE_FP64, SARBP_STORE_C64, false>(p, s, tiles, tiles_y, pps, qq_max);
        case SARBP_MODE_FP32:
            return fp16 ? launch_testf_mode<SARBP_MODE_FP32, SARBP_STORE_C32H, false>(p, s, tiles, tiles_y, pps, qq_max)
                        : launch_testf_mode<SARBP_MODE_FP32, SARBP_STORE_C64, false>(p, s, tiles, tiles_y, pps, qq_max);
        default:
            return fp16 ? launch_testf_mode<SARBP_MODE_SPLIT, SARBP_STORE_C32H, false>(p, s, tiles, tiles_y, pps, qq_max)
                        : launch_testf_mode<SARBP_MODE_SPLIT, SARBP_STORE_C64, false>(p, s, tiles, tiles_y, pps, qq_max);
    }
}

template <int PIX>
cudaError_t launch_pix(const BpPlan &p, cudaStream_t s, int tiles, int tiles_y, int pps, float qq_max) {
    const bool fp16 = p.storage == SARBP_STORE_C32H;
    switch (p.mode) {
        case SARBP_MODE_FP64:
            return fp16 ? launch_variant<SARBP_MODE_FP64, SARBP_STORE_C32H, 4, false, PIX>(p, s, tiles, tiles_y, pps, qq_max)
                        : launch_variant<SARBP_MODE_FP64, SARBP_STORE_C64, 4, false, PIX>(p, s, tiles, tiles_y, pps, qq_max);
        case SARBP_MODE_FP32:
            return fp16 ? launch_variant<SARBP_MODE_FP32, SARBP_STORE_C32H, 4, false, PIX>(p, s, tiles, tiles_y, pps, qq_max)
                        : launch_variant<SARBP_MODE_FP32, SARBP_STORE_C64, 4, false, PIX>(p, s, tiles, tiles_y, pps, qq_max);
        default:
            return fp16 ? launch_split<SARBP_MODE_SPLIT, SARBP_STORE_C32H, PIX>(p, s, tiles, tiles_y, pps, qq_max)
                        : launch_split<SARBP_MODE_SPLIT, SARBP_STORE_C64, PIX>(p, s, tiles, tiles_y, pps, qq_max);
    }
}

// out[p] = sum over tiles of proj[tile][p] in FP64.  A CTA takes 32 pulses
// (one per lane, coalesced rows); its 16 warps take tiles w, w + 16, ... and
// their partial sums combine in warp order, so the order is fixed and the
// result deterministic.  (One thread per pulse walking every tile kept only
// np / 128 CTAs busy: 0.15 ms for 512 tiles x 4096 pulses.)
constexpr int kProjWarps = 16;
__global__ void __launch_bounds__(32 * kProjWarps)
    proj_reduce_kernel(const float2 *__restrict__ proj, int tiles, int np, double2 *__restrict__ out) {
    __shared__ double2 part[kProjWarps][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int p = blockIdx.x * 32 + lane;
    double sr = 0.0, si = 0.0;
    if (p < np) {
        for (int t = warp; t < tiles; t += kProjWarps) {
            const float2 v = __ldg(&proj[(size_t)t * np + p]);
            sr += v.x;
            si += v.y;
        }
    }
    part[warp][lane] = make_double2(sr, si);
    __syncthreads();
    if (warp == 0 && p < np) {
        double r = 0.0, i = 0.0;
#pragma unroll
        for (int w = 0; w < kProjWarps; ++w) {
            r += part[w][lane].x;
            i += part[w][lane].y;
        }
        out[p] = make_double2(r, i);
    }
}

template <int STORE, int PIX>
cudaError_t launch_proj_pix(const BpPlan &p, cudaStream_t s, int tiles, int tiles_y, int pps, float qq_max) {
    if (p.lin) {  // large tiles: the linear-term phase
        if constexpr (PIX == 8) {
            if (p.chunk == kChunk)
                return p.nterms == 3
                           ? launch_variant<SARBP_MODE_SPLIT, STORE, 3, false, PIX, true, kChunk, false, true>(p, s, tiles, tiles_y, pps, qq_max)
                           : launch_variant<SARBP_MODE_SPLIT, STORE, 4, false, PIX, true, kChunk, false, true>(p, s, tiles, tiles_y, pps, qq_max);
        }
        return p.nterms == 3 ? launch_variant<SARBP_MODE_SPLIT, STORE, 3, false, PIX, true, 0, false, true>(p, s, tiles, tiles_y, pps, qq_max)
                             : launch_variant<SARBP_MODE_SPLIT, STORE, 4, false, PIX, true, 0, false, true>(p, s, tiles, tiles_y, pps, qq_max);
    }
    if constexpr (PIX == 8) {  // the usual tile: pulse chunk fixed at compile time
        if (p.chunk == kChunk)
            return p.nterms == 3
                       ? launch_variant<SARBP_MODE_SPLIT, STORE, 3, false, PIX, true, kChunk>(p, s, tiles, tiles_y, pps, qq_max)
                       : launch_variant<SARBP_MODE_SPLIT, STORE, 4, false, PIX, true, kChunk>(p, s, tiles, tiles_y, pps, qq_max);
    }
    return p.nterms == 3 ? launch_variant<SARBP_MODE_SPLIT, STORE, 3, false, PIX, true>(p, s, tiles, tiles_y, pps, qq_max)
                         : launch_variant<SARBP_MODE_SPLIT, STORE, 4, false, PIX, true>(p, s, tiles, tiles_y, pps, qq_max);
}

void launch_geometry(const BpPlan &p, int *tiles, int *tiles_y, int *pps, float *qq_max) {
    const int tile_y = 8 * p.pix;
    const int tiles_x = (p.g.nx + kTileX - 1) / kTileX;
    *tiles_y = (p.g.ny + tile_y - 1) / tile_y;
    *tiles = tiles_x * *tiles_y;
    int n = (p.np + p.segments - 1) / p.segments;
    *pps = (n + kChunk - 1) / kChunk * kChunk;
    // |q|^2 bound over a tile (pixel offsets from the tile centre)
    const double hx = 0.5 * (kTileX - 1), hy = 0.5 * (tile_y - 1);
    *qq_max = (float)(hx * hx * p.g.g11 + 2.0 * hx * hy * fabs(p.g.g12) + hy * hy * p.g.g22);
}

cudaError_t launch_pulse_refs(const BpPlan &p, cudaStream_t s) {
    pulse_ref_kernel<<<(p.np + 127) / 128, 128, 0, s>>>(p.apc, p.np, p.g, p.drange, p.dphase,
                                                         2.0 / p.c * p.bin_rate, 2.0 * p.fc / p.c, p.pref);
    return cudaGetLastError();
}

}  // namespace

size_t bp_tiles(const BpPlan &p) {
    int tiles, tiles_y, pps;
    float qq;
    launch_geometry(p, &tiles, &tiles_y, &pps, &qq);
    return (size_t)tiles;
}

cudaError_t launch_project(const BpPlan &p, double2 *out, cudaStream_t s, int *launches) {
    if (p.np <= 0) return cudaSuccess;
    if (p.mode != SARBP_MODE_SPLIT && p.mode != SARBP_MODE_FP16STORE) return cudaErrorInvalidValue;
    if (p.pix != 8 && p.pix != 4 && p.pix != 2) return cudaErrorInvalidValue;
    if (!p.weight || !p.proj || !out) return cudaErrorInvalidValue;
    if (p.g.nx <= 0 || p.g.ny <= 0) return cudaMemsetAsync(out, 0, sizeof(double2) * p.np, s);
    int tiles, tiles_y, pps;
    float qq_max;
    launch_geometry(p, &tiles, &tiles_y, &pps, &qq_max);
    cudaError_t e = launch_pulse_refs(p, s);
    if (e != cudaSuccess) return e;
    if (launches) ++*launches;
    const bool fp16 = p.storage == SARBP_STORE_C32H;
    if (bp_testing(p)) e = launch_testf<true>(p, s, tiles, tiles_y, pps, qq_max);
    else if (p.pix == 8) e = fp16 ? launch_proj_pix<SARBP_STORE_C32H, 8>(p, s, tiles, tiles_y, pps, qq_max)
                             : launch_proj_pix<SARBP_STORE_C64, 8>(p, s, tiles, tiles_y, pps, qq_max);
    else if (p.pix == 4) e = fp16 ? launch_proj_pix<SARBP_STORE_C32H, 4>(p, s, tiles, tiles_y, pps, qq_max)
                                  : launch_proj_pix<SARBP_STORE_C64, 4>(p, s, tiles, tiles_y, pps, qq_max);
    else e = fp16 ? launch_proj_pix<SARBP_STORE_C32H, 2>(p, s, tiles, tiles_y, pps, qq_max)
                  : launch_proj_pix<SARBP_STORE_C64, 2>(p, s, tiles, tiles_y, pps, qq_max);
    if (e != cudaSuccess) return e;
    if (launches) ++*launches;
    proj_reduce_kernel<<<(p.np + 31) / 32, 32 * kProjWarps, 0, s>>>(p.proj, tiles, p.np, out);
    e = cudaGetLastError();
    if (launches) ++*launches;
    return e;
}

cudaError_t bp_occupancy(const BpPlan &p, int *ctas_per_sm) {
    *ctas_per_sm = 0;
    if (p.pix != 8 && p.pix != 4 && p.pix != 2) return cudaErrorInvalidValue;
    int tiles, tiles_y, pps;
    float qq_max;
    launch_geometry(p, &tiles, &tiles_y, &pps, &qq_max);
    t_occupancy = ctas_per_sm;
    cudaError_t e = p.pix == 8 ? launch_pix<8>(p, nullptr, tiles, tiles_y, pps, qq_max)
                  : p.pix == 4 ? launch_pix<4>(p, nullptr, tiles, tiles_y, pps, qq_max)
                               : launch_pix<2>(p, nullptr, tiles, tiles_y, pps, qq_max);
    t_occupancy = nullptr;
    return e;
}

void bp_tile_dims(int pix, int *tile_x, int *tile_y) {
    *tile_x = kTileX;
    *tile_y = 8 * pix;
}

int bp_max_chunk() { return kChunk; }

size_t bp_smem_bytes(int storage, int win, int chunk) {
    return (size_t)2 * chunk * win * 16 + (size_t)kStages * chunk * win * raw_esize(storage) +
           kStages * kChunk * sizeof(Prm) +
           kStages * sizeof(uint64_t) + 2 * kWarps * kChunk * sizeof(float2);
}

// ---------------------------------------------------------------- planning extremes
// One thread per (pulse, lattice point); warp min / max, then one atomic per
// warp on the FP64 bit patterns (all four quantities are >= 0, where the
// unsigned order of the bits is the numeric order).
__global__ void bp_extremes_init_kernel(unsigned long long *out) {
    if (threadIdx.x == 0) {
        out[0] = (unsigned long long)__double_as_longlong(1e300);
        out[1] = out[2] = out[3] = 0ull;
        out[4] = 0ull;
    }
}

__global__ void __launch_bounds__(256) bp_extremes_kernel(const double *apc, int np, const sarbp_grid g, double lux,
                                                          double luy, unsigned long long *out) {
    constexpr int kPts = kLattice * kLattice;
    __shared__ double P[kPts][3];
    for (int k = threadIdx.x; k < kPts; k += blockDim.x) ext_lattice(g, k / kLattice, k % kLattice, P[k]);
    __syncthreads();
    // one thread per (pulse, lattice row): nine points
    ExtAcc acc;
    ext_acc_init(acc);
    bool bad = false;
    const long long total = (long long)np * kLattice;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int p = (int)(i / kLattice), u = (int)(i - (long long)p * kLattice);
        const double a[3] = {apc[3 * (size_t)p], apc[3 * (size_t)p + 1], apc[3 * (size_t)p + 2]};
        if (!isfinite(a[0]) || !isfinite(a[1]) || !isfinite(a[2])) {
            bad = true;
            continue;
        }
#pragma unroll 1
        for (int v = 0; v < kLattice; ++v) ext_acc_point(acc, g, lux, luy, P[u * kLattice + v], a);
    }
    double r2min = acc.r2min, r2max = acc.r2max, cx = acc.cx.best, sy = acc.sy.best;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        r2min = fmin(r2min, __shfl_xor_sync(0xffffffffu, r2min, o));
        r2max = fmax(r2max, __shfl_xor_sync(0xffffffffu, r2max, o));
        cx = fmax(cx, __shfl_xor_sync(0xffffffffu, cx, o));
        sy = fmax(sy, __shfl_xor_sync(0xffffffffu, sy, o));
    }
    // the block's warps combine in shared memory, then one thread per block
    // updates the result (order-free min / max: the same bits as the host's)
    __shared__ double red[4][8];
    __shared__ int red_bad;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) red_bad = 0;
    __syncthreads();
    const bool any_bad = __any_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0) {
        red[0][warp] = r2min;
        red[1][warp] = r2max;
        red[2][warp] = cx;
        red[3][warp] = sy;
        if (any_bad) red_bad = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // holds warp 0's values already
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            r2min = fmin(r2min, red[0][w]);
            r2max = fmax(r2max, red[1][w]);
            cx = fmax(cx, red[2][w]);
            sy = fmax(sy, red[3][w]);
        }
        atomicMin(&out[0], (unsigned long long)__double_as_longlong(r2min));
        atomicMax(&out[1], (unsigned long long)__double_as_longlong(r2max));
        atomicMax(&out[2], (unsigned long long)__double_as_longlong(cx));
        atomicMax(&out[3], (unsigned long long)__double_as_longlong(sy));
        if (red_bad) atomicOr(&out[4], 1ull);
    }
}

cudaError_t launch_bp_extremes(const double *apc, int np, const sarbp_grid &g, unsigned long long *out,
                               cudaStream_t s) {
    bp_extremes_init_kernel<<<1, 32, 0, s>>>(out);
    if (np <= 0) return cudaGetLastError();
    double lux, luy;
    ext_axes(g, &lux, &luy);
    const long long total = (long long)np * kLattice;  // threads: (pulse, lattice row)
    const int blocks = (int)std::min<long long>((total + 255) / 256, 512);
    bp_extremes_kernel<<<blocks, 256, 0, s>>>(apc, np, g, lux, luy, out);
    return cudaGetLastError();
}

cudaError_t launch_bp(const BpPlan &p, cudaStream_t s, int *launches) {
    if (p.np <= 0 || p.g.nx <= 0 || p.g.ny <= 0) return cudaSuccess;
    if (p.pix != 8 && p.pix != 4 && p.pix != 2) return cudaErrorInvalidValue;
    int tiles, tiles_y, pps;
    float qq_max;
    launch_geometry(p, &tiles, &tiles_y, &pps, &qq_max);
    cudaError_t e;
    if (p.mode == SARBP_MODE_SPLIT || p.mode == SARBP_MODE_FP16STORE) {
        e = launch_pulse_refs(p, s);
        if (e != cudaSuccess) return e;
        if (launches) ++*launches;
    }
    if (bp_testing(p)) e = launch_testf<false>(p, s, tiles, tiles_y, pps, qq_max);
    else if (p.pix == 8) e = launch_pix<8>(p, s, tiles, tiles_y, pps, qq_max);
    else if (p.pix == 4) e = launch_pix<4>(p, s, tiles, tiles_y, pps, qq_max);
    else e = launch_pix<2>(p, s, tiles, tiles_y, pps, qq_max);
    if (e != cudaSuccess) return e;
    if (launches) ++*launches;
    if (p.segments > 1) {
        const size_t count = (size_t)p.g.nx * p.g.ny;
        const int blocks = (int)std::min<size_t>((count + 255) / 256, (size_t)current_sms() * 8);
        reduce_segments_kernel<<<blocks, 256, 0, s>>>(p.partial, p.segments, count, p.image, p.accumulate);
        e = cudaGetLastError();
        if (launches) ++*launches;
    }
    return e;
}

}  // namespace sarbp
