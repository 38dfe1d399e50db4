// fft_smem.cuh -- shared-memory Stockham FFT used by range compression
// (rc.cu) and the omega-K imager (wk.cu).
//
// Stockham autosort transform with radix-32, radix-16 and radix-8 stages (one
// radix-4 or radix-2 stage for the remaining factor), in place in shared memory
// (XOR-swizzled so every stage's accesses are free of bank conflicts) with a
// barrier between each stage's loads and stores.  Twiddles come from two-level
// tables held in shared memory (see Etab / load_etab).
#pragma once

#include <type_traits>

#include "sarbp_internal.h"

namespace sarbp {
namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// Complex add / subtract as one packed FP32x2 instruction (sm_100+ f32x2:
// each half rounded to nearest, the same results as two scalar operations):
// a float2 already lives in a register pair, so the butterflies' add network
// takes half the issue slots.  Measured against scalar adds: omega-K image
// 1.067 vs 1.080 ms, config-2 range compression 3.07 vs 3.09 ms (complex64) and
// 3.14 vs 3.08 ms (FP16): the transforms are bound by shared-memory bursts and
// barriers, not by FP32 issue.
#ifndef SARBP_FFT_PACKED
#define SARBP_FFT_PACKED 1
#endif
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
#if SARBP_FFT_PACKED
    float2 r;
    asm("{\n\t.reg .b64 x, y, d;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
        "add.rn.f32x2 d, x, y;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
#else
    return make_float2(a.x + b.x, a.y + b.y);
#endif
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
#if SARBP_FFT_PACKED
    float2 r;
    asm("{\n\t.reg .b64 x, y, d;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 y, {%4, %5};\n\t"
        "sub.rn.f32x2 d, x, y;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
#else
    return make_float2(a.x - b.x, a.y - b.y);
#endif
}
// multiply by -j (forward kernel) or +j (inverse kernel)
template <bool INV>
__device__ __forceinline__ float2 mulj(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// Shared-memory layout of the transform points: point x lives in slot sw(x),
// an XOR swizzle inside each run of 16 float2 (128 bytes):
// x ^ (t ^ ((t & 4) << 1)) with t = (x >> 4) & 15.  A half-warp of 64-bit
// accesses then touches 16 distinct bank pairs for every access pattern of the
// transform: contiguous runs (loads of every stage, stores of the later
// stages), the stride-8 / stride-64 stores of the first two radix-8 stages and
// the stride-16 stores of the first radix-16 stage.  The swizzle only changes
// bits 0..3 and depends on bits 4..7, so sw(x + c) = sw(x) + c for any
// multiple c of 256.
__host__ __device__ constexpr int sw(int x) { return x ^ (((x >> 4) & 15) ^ ((x >> 3) & 8)); }

// table slot of entry i: one spare slot per 8 entries, so strided gathers
// spread over the banks
__device__ __forceinline__ int tslot(int i) { return i + (i >> 3); }

constexpr int kWlo = 128;  // low level of the transform twiddle table

// Shared-memory tables.  E^m = e^{+j 2 pi m / (L N)} (upsampling ramp, split
// combine) from E^m = T_hi[m >> 8] * T_lo[m & 255]; the transform twiddles
// W^m = e^{+j 2 pi m / N} = E^{L m} from W^m = W_hi[m >> 7] * W_lo[m & 127].
struct Etab {
    const float2 *lo;   // E^i, i < 256 (or L N entries when L N < 256), slot tslot(i)
    const float2 *hi;   // E^{256 i}, i < max(1, L N / 256), slot tslot(i)
    const float2 *wlo;  // W^i, i < min(N, 128)
    const float2 *whi;  // W^{128 i}, i < max(1, N / 128)
    __device__ __forceinline__ float2 operator()(int m) const {
        return cmul(hi[tslot(m >> 8)], lo[tslot(m & 255)]);
    }
    __device__ __forceinline__ float2 w(int m) const { return cmul(whi[m >> 7], wlo[m & (kWlo - 1)]); }
};

template <int R, bool INV>
struct Dft;

template <bool INV>
struct Dft<2, INV> {
    __device__ __forceinline__ static void run(float2 *v) {
        float2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

template <bool INV>
struct Dft<4, INV> {
    __device__ __forceinline__ static void run(float2 *v) {
        float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
        float2 t2 = cadd(v[1], v[3]), t3 = mulj<INV>(csub(v[1], v[3]));
        v[0] = cadd(t0, t2);
        v[2] = csub(t0, t2);
        v[1] = cadd(t1, t3);
        v[3] = csub(t1, t3);
    }
};

template <bool INV>
struct Dft<8, INV> {
    __device__ __forceinline__ static void run(float2 *v) {
        float2 e[4] = {v[0], v[2], v[4], v[6]};
        float2 o[4] = {v[1], v[3], v[5], v[7]};
        Dft<4, INV>::run(e);
        Dft<4, INV>::run(o);
        const float h = 0.70710678118654752440f;
        // W8^1, W8^2, W8^3 for the chosen direction
        float2 o1 = INV ? make_float2(h * (o[1].x - o[1].y), h * (o[1].x + o[1].y))
                        : make_float2(h * (o[1].x + o[1].y), h * (o[1].y - o[1].x));
        float2 o2 = mulj<INV>(o[2]);
        float2 o3 = INV ? make_float2(-h * (o[3].x + o[3].y), h * (o[3].x - o[3].y))
                        : make_float2(h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y));
        v[0] = cadd(e[0], o[0]);
        v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], o1);
        v[5] = csub(e[1], o1);
        v[2] = cadd(e[2], o2);
        v[6] = csub(e[2], o2);
        v[3] = cadd(e[3], o3);
        v[7] = csub(e[3], o3);
    }
};

// x W16^e for the chosen direction (forward e^{-j 2 pi e/16}, inverse
// e^{+j 2 pi e/16}), e a compile-time constant.
template <int E, bool INV>
__device__ __forceinline__ float2 tw16(float2 x) {
    constexpr float kC[16] = {1.f, 0.92387953251128675613f, 0.70710678118654752440f, 0.38268343236508977173f,
                              0.f, -0.38268343236508977173f, -0.70710678118654752440f, -0.92387953251128675613f,
                              -1.f, -0.92387953251128675613f, -0.70710678118654752440f, -0.38268343236508977173f,
                              0.f, 0.38268343236508977173f, 0.70710678118654752440f, 0.92387953251128675613f};
    constexpr int e = E & 15;
    if constexpr (e == 0) {
        return x;
    } else if constexpr (e == 4) {
        return mulj<INV>(x);
    } else if constexpr (e == 8) {
        return make_float2(-x.x, -x.y);
    } else if constexpr (e == 12) {
        return mulj<!INV>(x);
    } else {
        const float c = kC[e], sn = kC[(e + 12) & 15];  // sin(2 pi e / 16) = cos(2 pi (e - 4) / 16)
        const float si = INV ? sn : -sn;
        return make_float2(fmaf(x.x, c, -x.y * si), fmaf(x.x, si, x.y * c));
    }
}

// Radix-16 DFT as 4 x 4: DFT-4 over v[n2 + 4 n1], twiddles W16^{n2 k1},
// DFT-4 over n2; X[k1 + 4 k2].
template <bool INV>
struct Dft<16, INV> {
    __device__ __forceinline__ static void run(float2 *v) {
        float2 a[4][4];
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) {
            a[n2][0] = v[n2];
            a[n2][1] = v[n2 + 4];
            a[n2][2] = v[n2 + 8];
            a[n2][3] = v[n2 + 12];
            Dft<4, INV>::run(a[n2]);
        }
        a[1][1] = tw16<1, INV>(a[1][1]);
        a[1][2] = tw16<2, INV>(a[1][2]);
        a[1][3] = tw16<3, INV>(a[1][3]);
        a[2][1] = tw16<2, INV>(a[2][1]);
        a[2][2] = tw16<4, INV>(a[2][2]);
        a[2][3] = tw16<6, INV>(a[2][3]);
        a[3][1] = tw16<3, INV>(a[3][1]);
        a[3][2] = tw16<6, INV>(a[3][2]);
        a[3][3] = tw16<9, INV>(a[3][3]);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            float2 b[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
            Dft<4, INV>::run(b);
            v[k1] = b[0];
            v[k1 + 4] = b[1];
            v[k1 + 8] = b[2];
            v[k1 + 12] = b[3];
        }
    }
};

// x W32^e for the chosen direction, e a compile-time constant (odd e; the even
// ones are W16 powers).
template <int E, bool INV>
__device__ __forceinline__ float2 tw32(float2 x) {
    constexpr int e = E & 31;
    if constexpr ((e & 1) == 0) {
        return tw16<e / 2, INV>(x);
    } else {
        // cos and sin of 2 pi e / 32 for the odd e (first quadrant values, then signs)
        constexpr float kC[8] = {0.98078528040323044913f, 0.83146961230254523708f, 0.55557023301960222474f,
                                 0.19509032201612826785f, -0.19509032201612826785f, -0.55557023301960222474f,
                                 -0.83146961230254523708f, -0.98078528040323044913f};
        // e = 2 i + 1: cos(2 pi e/32) = kC[i] for e < 16; e >= 16: cos(2 pi e/32) = -cos(2 pi (e-16)/32)
        constexpr int i = (e & 15) >> 1;
        constexpr float c0 = kC[i];
        // sin(2 pi e/32) = cos(2 pi (e - 8)/32): e - 8 is odd and in [-7, 7] for e < 16
        constexpr int es = (e & 15) - 8;  // odd, -7..7
        constexpr float s0 = es >= 0 ? kC[es >> 1] : kC[(-es) >> 1];  // cos is even
        constexpr float c = e >= 16 ? -c0 : c0, sn = e >= 16 ? -s0 : s0;
        const float si = INV ? sn : -sn;
        return make_float2(fmaf(x.x, c, -x.y * si), fmaf(x.x, si, x.y * c));
    }
}

template <int... K>
struct Seq {};

// Radix-32 DFT as 2 x 16 (decimation in time): X[k] = E[k] + W32^k O[k],
// X[k + 16] = E[k] - W32^k O[k], E and O the 16-point DFTs of the even and
// odd points.
template <bool INV>
struct Dft<32, INV> {
    template <int K>
    __device__ __forceinline__ static void out(float2 *v, const float2 *e, const float2 *o) {
        const float2 t = tw32<K, INV>(o[K]);
        v[K] = cadd(e[K], t);
        v[K + 16] = csub(e[K], t);
    }
    template <int... K>
    __device__ __forceinline__ static void outs(float2 *v, const float2 *e, const float2 *o, Seq<K...>) {
        (out<K>(v, e, o), ...);
    }
    __device__ __forceinline__ static void run(float2 *v) {
        float2 e[16], o[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            e[i] = v[2 * i];
            o[i] = v[2 * i + 1];
        }
        Dft<16, INV>::run(e);
        Dft<16, INV>::run(o);
        outs(v, e, o, Seq<0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15>{});
    }
};

// Radix-16 stage twiddles W^{m r}, r = 1..15, applied to v[1..15] as products
// of the four table powers w, w^2, w^4, w^8 (at most four factors), so only
// the powers and four partial products are live.
struct Tw16 {
    float2 b1, b2, b4, b8;
};
template <bool INV, bool HOISTED_LO>
__device__ __forceinline__ Tw16 tw16_bases(const Etab &E, int m, const float2 *lo) {
    Tw16 t;
    t.b1 = HOISTED_LO ? cmul(E.whi[m >> 7], lo[0]) : E.w(m);
    t.b2 = HOISTED_LO ? cmul(E.whi[(2 * m) >> 7], lo[1]) : E.w(2 * m);
    t.b4 = HOISTED_LO ? cmul(E.whi[(4 * m) >> 7], lo[2]) : E.w(4 * m);
    t.b8 = HOISTED_LO ? cmul(E.whi[(8 * m) >> 7], lo[3]) : E.w(8 * m);
    if (!INV) {
        t.b1.y = -t.b1.y;
        t.b2.y = -t.b2.y;
        t.b4.y = -t.b4.y;
        t.b8.y = -t.b8.y;
    }
    return t;
}
__device__ __forceinline__ void tw16_apply(float2 *v, const Tw16 &t) {
    const float2 w3 = cmul(t.b1, t.b2), w5 = cmul(t.b1, t.b4), w6 = cmul(t.b2, t.b4);
    const float2 w7 = cmul(w3, t.b4);
    v[1] = cmul(v[1], t.b1);
    v[2] = cmul(v[2], t.b2);
    v[3] = cmul(v[3], w3);
    v[4] = cmul(v[4], t.b4);
    v[5] = cmul(v[5], w5);
    v[6] = cmul(v[6], w6);
    v[7] = cmul(v[7], w7);
    v[8] = cmul(v[8], t.b8);
    v[9] = cmul(v[9], cmul(t.b1, t.b8));
    v[10] = cmul(v[10], cmul(t.b2, t.b8));
    v[11] = cmul(v[11], cmul(w3, t.b8));
    v[12] = cmul(v[12], cmul(t.b4, t.b8));
    v[13] = cmul(v[13], cmul(w5, t.b8));
    v[14] = cmul(v[14], cmul(w6, t.b8));
    v[15] = cmul(v[15], cmul(w7, t.b8));
}

// Radix-32 stage twiddles: v[r] W^{m r}, r = 1..31, as v[16 + r] times w^16
// and then the radix-16 pattern on both halves.
struct Tw32 {
    Tw16 t16;
    float2 b16;
};
template <bool INV, bool HOISTED_LO>
__device__ __forceinline__ Tw32 tw32_bases(const Etab &E, int m, const float2 *lo) {
    Tw32 t;
    t.t16 = tw16_bases<INV, HOISTED_LO>(E, m, lo);
    t.b16 = HOISTED_LO ? cmul(E.whi[(16 * m) >> 7], lo[4]) : E.w(16 * m);
    if (!INV) t.b16.y = -t.b16.y;
    return t;
}
__device__ __forceinline__ void tw32_apply(float2 *v, const Tw32 &t) {
#pragma unroll
    for (int r = 16; r < 32; ++r) v[r] = cmul(v[r], t.b16);
    tw16_apply(v, t.t16);
    tw16_apply(v + 16, t.t16);
}

// Twiddles W^{m r}, r = 1..R-1 (forward: conjugated) for a butterfly whose
// base exponent is m: w, w^2, w^4 from the table, the others as products.
// lo1/lo2/lo4 are the low-level table entries when the caller hoisted them.
template <int R, bool INV, bool HOISTED_LO>
__device__ __forceinline__ void twiddles(const Etab &E, int m, float2 lo1, float2 lo2, float2 lo4, float2 *w) {
    w[1] = HOISTED_LO ? cmul(E.whi[m >> 7], lo1) : E.w(m);
    if (!INV) w[1].y = -w[1].y;
    if (R >= 4) {
        w[2] = HOISTED_LO ? cmul(E.whi[(2 * m) >> 7], lo2) : E.w(2 * m);
        if (!INV) w[2].y = -w[2].y;
        w[3] = cmul(w[1], w[2]);
    }
    if (R >= 8) {
        w[4] = HOISTED_LO ? cmul(E.whi[(4 * m) >> 7], lo4) : E.w(4 * m);
        if (!INV) w[4].y = -w[4].y;
        w[5] = cmul(w[1], w[4]);
        w[6] = cmul(w[2], w[4]);
        w[7] = cmul(w[3], w[4]);
    }
}

// One Stockham stage: butterfly j reads s[j + r*N/R], applies twiddles
// W_N^{k r N/(Ns R)} (k = j mod Ns), runs a radix-R DFT and writes
// s[(j - k) R + k + r Ns] (slots through sw()).  Ns is a compile-time
// constant: offsets that are multiples of 256 points pass through sw()
// unchanged and become immediates.  When T is a multiple of Ns every
// butterfly of a thread has the same k and the twiddles are computed once.
// Destination of a stage's outputs: back to shared memory (every stage but
// the last of an I/O-fused transform), or a caller's functor sink(x, value)
// receiving output point x in natural order.
struct SmemSink {};

// BATCH > 1: the stage runs over BATCH independent N-point arrays CS points
// apart (s + c CS), their butterflies spread over the threads and sharing the
// stage's barriers.
template <int N, int R, int T, bool INV, int Ns, class Sink = SmemSink, int BATCH = 1, int CS = N>
__device__ __forceinline__ void stage(float2 *s, const Etab &E, Sink sink = Sink{}) {
    constexpr bool kToSmem = std::is_same<Sink, SmemSink>::value;
    constexpr int NB = N / R;
    constexpr int NBT = NB * BATCH;
    constexpr int PER = (NBT + T - 1) / T;
    constexpr int C = N / (Ns * R);  // k -> twiddle exponent step
    static_assert(BATCH == 1 || kToSmem, "batched stages write shared memory");
    float2 v[PER][R];
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int jj = threadIdx.x + b * T;
        if (PER * T == NBT || jj < NBT) {
            const int col = BATCH == 1 ? 0 : jj / NB;
            const int j = jj - col * NB;
            const float2 *sc = s + col * CS;
            if constexpr (NB % 256 == 0) {
                const float2 *src = sc + sw(j);
#pragma unroll
                for (int r = 0; r < R; ++r) v[b][r] = src[r * NB];
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) v[b][r] = sc[sw(j + r * NB)];
            }
        }
    }
    if constexpr (kToSmem) __syncthreads();  // loads done before the in-place stores
    float2 w[R <= 8 ? R : 1];
    Tw16 t16;
    Tw32 t32;
    constexpr bool kSameK = Ns > 1 && T % Ns == 0;
    // k = j when Ns >= NB (last stage); the low table level is then fixed per thread
    // (batched: also across the wrap from one array to the next)
    constexpr bool kHoistLo = Ns > 1 && !kSameK && Ns >= NB && N >= kWlo && (C * T) % kWlo == 0 &&
                              (BATCH == 1 || (C * NB) % kWlo == 0);
    float2 lo1 = make_float2(1.f, 0.f), lo2 = lo1, lo4 = lo1;
    float2 lo[5] = {lo1, lo1, lo1, lo1, lo1};
    if constexpr (kSameK) {
        if constexpr (R == 32)
            t32 = tw32_bases<INV, false>(E, C * (int)(threadIdx.x & (Ns - 1)), lo);
        else if constexpr (R == 16)
            t16 = tw16_bases<INV, false>(E, C * (int)(threadIdx.x & (Ns - 1)), lo);
        else
            twiddles<R, INV, false>(E, C * (int)(threadIdx.x & (Ns - 1)), lo1, lo2, lo4, w);
    } else if constexpr (kHoistLo) {
        const int m = C * (int)threadIdx.x;
        lo1 = E.wlo[m & (kWlo - 1)];
        if (R >= 4) lo2 = E.wlo[(2 * m) & (kWlo - 1)];
        if (R >= 8) lo4 = E.wlo[(4 * m) & (kWlo - 1)];
        if constexpr (R >= 16) {
            lo[0] = lo1;
            lo[1] = lo2;
            lo[2] = lo4;
            lo[3] = E.wlo[(8 * m) & (kWlo - 1)];
        }
        if constexpr (R == 32) lo[4] = E.wlo[(16 * m) & (kWlo - 1)];
    }
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int jj = threadIdx.x + b * T;
        if (PER * T == NBT || jj < NBT) {
            const int col = BATCH == 1 ? 0 : jj / NB;
            const int j = jj - col * NB;
            float2 *sc = s + col * CS;
            const int k = j & (Ns - 1);
            if constexpr (Ns > 1) {
                if constexpr (R == 32) {
                    if constexpr (!kSameK) t32 = tw32_bases<INV, kHoistLo>(E, C * k, lo);
                    tw32_apply(v[b], t32);
                } else if constexpr (R == 16) {
                    if constexpr (!kSameK) t16 = tw16_bases<INV, kHoistLo>(E, C * k, lo);
                    tw16_apply(v[b], t16);
                } else {
                    if constexpr (!kSameK) twiddles<R, INV, kHoistLo>(E, C * k, lo1, lo2, lo4, w);
#pragma unroll
                    for (int r = 1; r < R; ++r) v[b][r] = cmul(v[b][r], w[r]);
                }
            }
            Dft<R, INV>::run(v[b]);
            const int x0 = (j - k) * R + k;
            if constexpr (!kToSmem) {
#pragma unroll
                for (int r = 0; r < R; ++r) sink(x0 + r * Ns, v[b][r]);
            } else if constexpr (Ns % 256 == 0) {
                float2 *dst = sc + sw(x0);
#pragma unroll
                for (int r = 0; r < R; ++r) dst[r * Ns] = v[b][r];
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) sc[sw(x0 + r * Ns)] = v[b][r];
            }
        }
    }
    if constexpr (kToSmem) __syncthreads();
}

#ifndef SARBP_FFT_RADIX16
#define SARBP_FFT_RADIX16 1
#endif
// radix-32 stages where every thread holds at least one 32-point butterfly
// (N / 32 >= T: transforms with at least 32 points per thread): two
// shared-memory passes instead of three for 16384 points at 512 threads
// (32-32-16) and 8192 at 256 (32-32-8).  Range compression on GB300, 4096
// pulses: 16384 points 3.077 -> 2.986 ms, 8192 points 1.295 -> 1.123 ms; 32768
// (2048 pulses) 4.289 -> 4.170 ms.  Shapes with fewer points per thread (the
// omega-K transforms) keep their radix-16/8 stages.
#ifndef SARBP_FFT_RADIX32
#define SARBP_FFT_RADIX32 1
#endif
// radix-16 stages while 16 * Ns <= N and the stage keeps all T threads busy
// (N / 16 >= T), then radix-8 stages while 8 * Ns <= N, then one radix-4 or
// radix-2 stage
template <int N, int T, bool INV, int Ns>
struct Stages {
    __device__ __forceinline__ static void run(float2 *s, const Etab &E) {
        if constexpr (SARBP_FFT_RADIX32 && Ns * 32 <= N && N / 32 >= T) {
            stage<N, 32, T, INV, Ns>(s, E);
            Stages<N, T, INV, Ns * 32>::run(s, E);
        } else if constexpr (SARBP_FFT_RADIX16 && Ns * 16 <= N && N / 16 >= T) {
            stage<N, 16, T, INV, Ns>(s, E);
            Stages<N, T, INV, Ns * 16>::run(s, E);
        } else if constexpr (Ns * 8 <= N) {
            stage<N, 8, T, INV, Ns>(s, E);
            Stages<N, T, INV, Ns * 8>::run(s, E);
        } else if constexpr (Ns * 4 == N) {
            stage<N, 4, T, INV, Ns>(s, E);
        } else if constexpr (Ns * 2 == N) {
            stage<N, 2, T, INV, Ns>(s, E);
        }
    }
};

// Unnormalised in-place FFT of N points held (swizzled) in shared memory.
// Caller must have synchronised after filling s; returns synchronised.
template <int N, int T, bool INV>
__device__ void fft_smem(float2 *s, const Etab &E) {
    Stages<N, T, INV, 1>::run(s, E);
}

// BATCH transforms of N points, array c at s + c CS, sharing each stage's
// barriers (same radix sequence as Stages).
template <int N, int T, bool INV, int Ns, int BATCH, int CS>
struct StagesBatched {
    __device__ __forceinline__ static void run(float2 *s, const Etab &E) {
        if constexpr (SARBP_FFT_RADIX32 && Ns * 32 <= N && N / 32 >= T) {
            stage<N, 32, T, INV, Ns, SmemSink, BATCH, CS>(s, E);
            StagesBatched<N, T, INV, Ns * 32, BATCH, CS>::run(s, E);
        } else if constexpr (SARBP_FFT_RADIX16 && Ns * 16 <= N && N / 16 >= T) {
            stage<N, 16, T, INV, Ns, SmemSink, BATCH, CS>(s, E);
            StagesBatched<N, T, INV, Ns * 16, BATCH, CS>::run(s, E);
        } else if constexpr (Ns * 8 <= N) {
            stage<N, 8, T, INV, Ns, SmemSink, BATCH, CS>(s, E);
            StagesBatched<N, T, INV, Ns * 8, BATCH, CS>::run(s, E);
        } else if constexpr (Ns * 4 == N) {
            stage<N, 4, T, INV, Ns, SmemSink, BATCH, CS>(s, E);
        } else if constexpr (Ns * 2 == N) {
            stage<N, 2, T, INV, Ns, SmemSink, BATCH, CS>(s, E);
        }
    }
};

// Radix of the stage with stride Ns (the same sequence as Stages).
template <int N, int T, int Ns>
__host__ __device__ constexpr int stage_radix() {
    return (SARBP_FFT_RADIX32 && Ns * 32 <= N && N / 32 >= T)   ? 32
           : (SARBP_FFT_RADIX16 && Ns * 16 <= N && N / 16 >= T) ? 16
           : (Ns * 8 <= N ? 8 : N / Ns);
}

// I/O-fused transform.  The first stage (stride 1) takes its inputs from
// registers: butterfly j = threadIdx.x + b T (j < N / R) holds points
// j + r N / R, r < R, in v[b][r] (FirstIn<N, T> gives R, the butterfly count
// and the per-thread array shape), so the caller loads them straight from
// global memory and shared memory is never filled in a pass of its own.  The
// last stage hands its outputs to sink(x, value) instead of writing shared
// memory back.  Two shared-memory passes and two barriers fewer than filling
// s, fft_smem and reading s out.  s must not be in use by other threads'
// reads when called (the first stage writes it without a barrier first).
template <int N, int T>
struct FirstIn {
    static constexpr int R = stage_radix<N, T, 1>();
    static constexpr int NB = N / R;
    static constexpr int PER = (NB + T - 1) / T;
    static_assert(R < N, "I/O-fused transforms need at least two stages");
    __device__ __forceinline__ static bool live(int b) { return PER * T == NB || (int)threadIdx.x + b * T < NB; }
    __device__ __forceinline__ static int point(int b, int r) { return (int)threadIdx.x + b * T + r * NB; }
};

template <int N, int T, bool INV, int Ns, class Sink>
struct StagesTo {
    __device__ __forceinline__ static void run(float2 *s, const Etab &E, Sink sink) {
        constexpr int R = stage_radix<N, T, Ns>();
        if constexpr (Ns * R == N) {
            stage<N, R, T, INV, Ns, Sink>(s, E, sink);
        } else {
            stage<N, R, T, INV, Ns>(s, E);
            StagesTo<N, T, INV, Ns * R, Sink>::run(s, E, sink);
        }
    }
};

template <int N, int T, bool INV, class Sink>
__device__ __forceinline__ void fft_io(float2 *s, const Etab &E, float2 (&v)[FirstIn<N, T>::PER][FirstIn<N, T>::R], Sink sink) {
    using F = FirstIn<N, T>;
    constexpr int R = F::R;
#pragma unroll
    for (int b = 0; b < F::PER; ++b) {
        if (F::live(b)) {
            const int j = (int)threadIdx.x + b * T;
            Dft<R, INV>::run(v[b]);
#pragma unroll
            for (int r = 0; r < R; ++r) s[sw(j * R + r)] = v[b][r];  // stride 1: x0 = j R
        }
    }
    __syncthreads();
    StagesTo<N, T, INV, R, Sink>::run(s, E, sink);
}

// Shared memory after the N points: E low/high levels (slots through
// tslot), W low/high levels, and the per-CTA ramp table of the inverse.
constexpr int kEloSlots = 288, kEhiSlots = 1152, kWhiMax = 128, kRampMax = 64;
constexpr size_t kTabSmem = sizeof(float2) * (kEloSlots + kEhiSlots + kWlo + kWhiMax + kRampMax);
template <int N>
__device__ __forceinline__ float2 *ramp_slots(float2 *sm) {
    return sm + N + kEloSlots + kEhiSlots + kWlo + kWhiMax;
}

// Fills the E tables from global memory, then derives the W tables
// (W^m = E^{L m}).  Contains one block barrier; the caller synchronises again
// before the W tables are read.
template <int N, int T>
__device__ __forceinline__ Etab load_etab_at(float2 *tables, const float2 *__restrict__ etab, int L) {
    static_assert(N / kWlo <= kWhiMax, "W table too small");
    const int LN = L * N;
    const int nlo = LN < 256 ? LN : 256;
    const int nhi = LN < 256 ? 1 : LN / 256;
    float2 *lo = tables;
    float2 *hi = lo + kEloSlots;
    float2 *wlo = hi + kEhiSlots;
    float2 *whi = wlo + kWlo;
    for (int i = threadIdx.x; i < nlo; i += T) lo[tslot(i)] = __ldg(&etab[i]);
    for (int i = threadIdx.x; i < nhi; i += T) hi[tslot(i)] = __ldg(&etab[256 + i]);
    __syncthreads();
    const Etab E{lo, hi, wlo, whi};
    constexpr int nwlo = N < kWlo ? N : kWlo;
    constexpr int nwhi = N < kWlo ? 1 : N / kWlo;
    for (int i = threadIdx.x; i < nwlo + nwhi; i += T) {
        if (i < nwlo)
            wlo[i] = E(L * i);
        else
            whi[i - nwlo] = E((L * kWlo * (i - nwlo)) & (LN - 1));
    }
    return E;
}
// Tables right after the N points of a single transform at sm.
template <int N, int T>
__device__ __forceinline__ Etab load_etab(float2 *sm, const float2 *__restrict__ etab, int L) {
    return load_etab_at<N, T>(sm + N, etab, L);
}

// CTAs per SM that a T-thread kernel holding an N-point transform (plus the
// tables) aims its register allocation at: two when both fit twice (8192
// points at 512 threads: 64 registers per thread), else one.
template <int N, int T>
constexpr int fft_min_blocks() {
    return (T * 64 <= 32768 && (size_t)N * 8 + kTabSmem <= (size_t)110 * 1024) ? 2 : 1;
}

}  // namespace
}  // namespace sarbp
