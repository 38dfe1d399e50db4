// rc.cu -- range compression and range upsampling on sm_103a.
//
// Implements code/SAR_BP/matlab/BPA_SAR.m:93-111 (matched filter
// ifft(fft(s).*conj(fft(h))) followed by 8x upsampling through mid-spectrum
// zero insertion) as two kernels:
//
//   rc_forward  (one CTA per pulse): zero-padded echo row -> shared memory ->
//               forward FFT -> multiply by the filter spectrum
//               G[k] = conj(H[k]) e^{-j2pi k D/N} / N -> spectrum scratch.
//               Also emits the per-pulse bound sum_k |Y[k]| (>= max |output|)
//               from which the FP16 storage scale is derived.
//   rc_inverse  (one CTA per pulse and upsampling phase r): the L*N-point
//               inverse of the zero-inserted spectrum evaluated at bins
//               b = L*i + r equals the N-point inverse of Y[k]*e^{+j2pi kappa r/(LN)}
//               (kappa = signed frequency), so each CTA runs one N-point
//               inverse FFT and writes every L-th output bin.
//
// The FFT is a Stockham autosort transform with radix-8 stages (one radix-4
// or radix-2 stage when log2 N is not a multiple of 3), in place in shared
// memory (XOR-swizzled so every stage's accesses are free of bank conflicts)
// with a barrier between each stage's loads and stores.  The upsampling ramp
// is a power of E = e^{j 2 pi / (L N)}, read from a two-level table in shared
// memory, E^m = T_hi[m >> 8] * T_lo[m & 255] (computed in double precision on
// the host); the transform twiddles are powers of W = E^L from a second
// two-level table derived from it at kernel start, so no FFT stage touches
// global memory.
//
// N = 32768 (shared memory holds 16384 points) is split by one radix-2 stage:
// the forward runs two CTAs per pulse on the half-size inputs x[n] + x[n+M] and
// (x[n] - x[n+M]) W_N^n, giving the even and odd spectral bins; the inverse
// runs a 2-CTA cluster per (pulse, phase) on the even and odd bins and forms
// y[i] = A[i] + W_N^{-i} B[i], y[i+M] = A[i] - W_N^{-i} B[i] with the partner's
// half read through distributed shared memory.
#include <cooperative_groups.h>

#include "sarbp_internal.h"

namespace sarbp {
namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// multiply by -j (forward kernel) or +j (inverse kernel)
template <bool INV>
__device__ __forceinline__ float2 mulj(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// Shared-memory layout of the transform points: point x lives in slot sw(x),
// an XOR swizzle inside each run of 16 float2 (128 bytes).  A half-warp of
// 64-bit accesses then touches 16 distinct bank pairs for every access pattern
// of the transform: contiguous runs (loads of every stage, stores of the later
// stages) and the stride-8 / stride-64 stores of the first two radix-8 stages.
// The swizzle only changes bits 0..3 and depends on bits 4..6, so
// sw(x + c) = sw(x) + c for any multiple c of 128.
__host__ __device__ constexpr int sw(int x) { return x ^ (((x >> 4) & 7) | ((x >> 3) & 8)); }

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
// constant: offsets that are multiples of 128 points pass through sw()
// unchanged and become immediates.  When T is a multiple of Ns every
// butterfly of a thread has the same k and the twiddles are computed once.
template <int N, int R, int T, bool INV, int Ns>
__device__ __forceinline__ void stage(float2 *s, const Etab &E) {
    constexpr int NB = N / R;
    constexpr int PER = (NB + T - 1) / T;
    constexpr int C = N / (Ns * R);  // k -> twiddle exponent step
    float2 v[PER][R];
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int j = threadIdx.x + b * T;
        if (PER * T == NB || j < NB) {
            if constexpr (NB % 128 == 0) {
                const float2 *src = s + sw(j);
#pragma unroll
                for (int r = 0; r < R; ++r) v[b][r] = src[r * NB];
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) v[b][r] = s[sw(j + r * NB)];
            }
        }
    }
    __syncthreads();
    float2 w[R];
    constexpr bool kSameK = Ns > 1 && T % Ns == 0;
    // k = j when Ns >= NB (last stage); the low table level is then fixed per thread
    constexpr bool kHoistLo = Ns > 1 && !kSameK && Ns >= NB && N >= kWlo && (C * T) % kWlo == 0;
    float2 lo1 = make_float2(1.f, 0.f), lo2 = lo1, lo4 = lo1;
    if constexpr (kSameK) {
        twiddles<R, INV, false>(E, C * (int)(threadIdx.x & (Ns - 1)), lo1, lo2, lo4, w);
    } else if constexpr (kHoistLo) {
        const int m = C * (int)threadIdx.x;
        lo1 = E.wlo[m & (kWlo - 1)];
        if (R >= 4) lo2 = E.wlo[(2 * m) & (kWlo - 1)];
        if (R >= 8) lo4 = E.wlo[(4 * m) & (kWlo - 1)];
    }
#pragma unroll
    for (int b = 0; b < PER; ++b) {
        const int j = threadIdx.x + b * T;
        if (PER * T == NB || j < NB) {
            const int k = j & (Ns - 1);
            if constexpr (Ns > 1) {
                if constexpr (!kSameK) twiddles<R, INV, kHoistLo>(E, C * k, lo1, lo2, lo4, w);
#pragma unroll
                for (int r = 1; r < R; ++r) v[b][r] = cmul(v[b][r], w[r]);
            }
            Dft<R, INV>::run(v[b]);
            const int x0 = (j - k) * R + k;
            if constexpr (Ns % 128 == 0) {
                float2 *dst = s + sw(x0);
#pragma unroll
                for (int r = 0; r < R; ++r) dst[r * Ns] = v[b][r];
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) s[sw(x0 + r * Ns)] = v[b][r];
            }
        }
    }
    __syncthreads();
}

// radix-8 stages while 8 * Ns <= N, then one radix-4 or radix-2 stage
template <int N, int T, bool INV, int Ns>
struct Stages {
    __device__ __forceinline__ static void run(float2 *s, const Etab &E) {
        if constexpr (Ns * 8 <= N) {
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
__device__ __forceinline__ Etab load_etab(float2 *sm, const float2 *__restrict__ etab, int L) {
    static_assert(N / kWlo <= kWhiMax, "W table too small");
    const int LN = L * N;
    const int nlo = LN < 256 ? LN : 256;
    const int nhi = LN < 256 ? 1 : LN / 256;
    float2 *lo = sm + N;
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

template <int T>
__device__ __forceinline__ float block_sum(float v, float *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    float t = 0.f;
    if (threadIdx.x < 32) {
        t = (l < T / 32) ? red[l] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;  // valid in thread 0
}

template <int N, int T>
__global__ void __launch_bounds__(T) rc_forward_kernel(int ns, int L, const float2 *__restrict__ echo,
                                                       const float2 *__restrict__ filt,
                                                       const float2 *__restrict__ etab,
                                                       float2 *__restrict__ spec,
                                                       float *__restrict__ scale) {
    extern __shared__ float2 sm[];
    __shared__ float red[32];
    const int p = blockIdx.x;
    const Etab E = load_etab<N, T>(sm, etab, L);
    const float2 *row = echo + (size_t)p * ns;
    for (int i = threadIdx.x; i < N; i += T) sm[sw(i)] = i < ns ? __ldg(&row[i]) : make_float2(0.f, 0.f);
    __syncthreads();
    fft_smem<N, T, false>(sm, E);
    float2 *out = spec + (size_t)p * N;
    float acc = 0.f;
    for (int k = threadIdx.x; k < N; k += T) {
        float2 y = cmul(sm[sw(k)], __ldg(&filt[k]));
        out[k] = y;
        acc += sqrtf(fmaf(y.x, y.x, y.y * y.y));
    }
    const float bound = block_sum<T>(acc, red);
    if (threadIdx.x == 0 && scale) {
        // power-of-two scale so that stored FP16 magnitudes stay <= 2^14
        float sc = 1.f;
        if (bound > 0.f && isfinite(bound)) sc = exp2f(ceilf(log2f(bound) - 14.f));
        scale[p] = sc;
    }
}

template <int N, int T, int STORE>
__global__ void __launch_bounds__(T) rc_inverse_kernel(int ns, int L, int nbins,
                                                       const float2 *__restrict__ spec,
                                                       const float2 *__restrict__ etab,
                                                       const float *__restrict__ scale,
                                                       void *__restrict__ out) {
    extern __shared__ float2 sm[];
    const int p = blockIdx.x / L;
    const int r = blockIdx.x - p * L;
    const float2 *in = spec + (size_t)p * N;
    const int LN = L * N;
    const Etab E = load_etab<N, T>(sm, etab, L);
    // Ramp E^{kappa r}, kappa the signed frequency (MATLAB split floor((N+1)/2)
    // = N/2 for even N).  With k = tid + T i and N/2 a multiple of T it factors
    // into a per-thread E^{tid r} and a per-CTA table over i that also carries
    // the E^{-N r} of the negative half (one broadcast read per point).
    constexpr bool kTwoLevel = (N / 2) % T == 0 && N / T <= kRampMax;
    float2 *rt = ramp_slots<N>(sm);
    float2 base = make_float2(1.f, 0.f);
    if (kTwoLevel && r != 0) {
        if (threadIdx.x < N / T) {
            const int i = threadIdx.x;
            float2 v = E((T * i * r) & (LN - 1));
            if (T * i >= N / 2) v = cmul(v, E((LN - N * r) & (LN - 1)));
            rt[i] = v;
        }
        base = E((int)(threadIdx.x * r) & (LN - 1));
    }
    __syncthreads();
    for (int k = threadIdx.x, i = 0; k < N; k += T, ++i) {
        float2 y = __ldg(&in[k]);
        if (r != 0) {
            if (kTwoLevel) {
                y = cmul(cmul(y, base), rt[i]);
            } else {
                const int kap = k < N / 2 ? k : k - N;
                y = cmul(y, E((kap * r) & (LN - 1)));  // LN is a power of two
            }
        }
        sm[sw(k)] = y;
    }
    __syncthreads();
    fft_smem<N, T, true>(sm, E);
    if (STORE == SARBP_STORE_C64) {
        float2 *o = reinterpret_cast<float2 *>(out) + (size_t)p * nbins + r;
        for (int i = threadIdx.x; i < ns; i += T) o[(size_t)L * i] = sm[sw(i)];
    } else {
        const float inv = 1.f / __ldg(&scale[p]);  // exact: scale is a power of two
        __half2 *o = reinterpret_cast<__half2 *>(out) + (size_t)p * nbins + r;
        for (int i = threadIdx.x; i < ns; i += T) {
            float2 v = sm[sw(i)];
            o[(size_t)L * i] = __floats2half2_rn(v.x * inv, v.y * inv);
        }
    }
}

namespace cg = cooperative_groups;

// N = 2M forward: CTA pair (h = 0, 1) per pulse; h = 0 yields X[2k], h = 1 X[2k+1].
// bound2[2p + h] receives the CTA's part of sum_k |Y[k]|.
template <int M, int T>
__global__ void __launch_bounds__(T) rc_forward2_kernel(int ns, int L, const float2 *__restrict__ echo,
                                                        const float2 *__restrict__ filt,
                                                        const float2 *__restrict__ etab,
                                                        float2 *__restrict__ spec, float *__restrict__ bound2) {
    extern __shared__ float2 sm[];
    __shared__ float red[32];
    const int h = blockIdx.x & 1, p = blockIdx.x >> 1;
    const Etab E = load_etab<M, T>(sm, etab, 2 * L);
    const float2 *row = echo + (size_t)p * ns;
    for (int i = threadIdx.x; i < M; i += T) {
        const float2 a = i < ns ? __ldg(&row[i]) : make_float2(0.f, 0.f);
        const float2 b = i + M < ns ? __ldg(&row[i + M]) : make_float2(0.f, 0.f);
        float2 v;
        if (h == 0) {
            v = cadd(a, b);
        } else {
            float2 w = E(L * i);  // W_N^i = conj(E^{L i})
            w.y = -w.y;
            v = cmul(csub(a, b), w);
        }
        sm[sw(i)] = v;
    }
    __syncthreads();
    fft_smem<M, T, false>(sm, E);
    float2 *out = spec + (size_t)p * (2 * M);
    float acc = 0.f;
    for (int k = threadIdx.x; k < M; k += T) {
        const int idx = 2 * k + h;
        const float2 y = cmul(sm[sw(k)], __ldg(&filt[idx]));
        out[idx] = y;
        acc += sqrtf(fmaf(y.x, y.x, y.y * y.y));
    }
    const float bound = block_sum<T>(acc, red);
    if (threadIdx.x == 0) bound2[2 * p + h] = bound;
}

// N = 2M inverse: cluster of two CTAs per (pulse, phase r).  CTA h transforms
// the bins 2k + h, then each CTA writes half of the outputs using both halves.
template <int M, int T, int STORE>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(T)
    rc_inverse2_kernel(int ns, int L, int nbins, const float2 *__restrict__ spec, const float2 *__restrict__ etab,
                       const float *__restrict__ bound2, float *__restrict__ scale, void *__restrict__ out) {
    extern __shared__ float2 sm[];
    cg::cluster_group cluster = cg::this_cluster();
    const int h = (int)cluster.block_rank();
    const int pr = blockIdx.x >> 1;
    const int p = pr / L, r = pr - p * L;
    constexpr int N = 2 * M;
    const int LN = L * N;
    const Etab E = load_etab<M, T>(sm, etab, 2 * L);
    const float2 *in = spec + (size_t)p * N;
    for (int k = threadIdx.x; k < M; k += T) {
        const int idx = 2 * k + h;
        float2 y = __ldg(&in[idx]);
        if (r != 0) {
            const int kap = idx < N / 2 ? idx : idx - N;
            y = cmul(y, E((kap * r) & (LN - 1)));  // LN is a power of two
        }
        sm[sw(k)] = y;
    }
    __syncthreads();
    fft_smem<M, T, true>(sm, E);
    cluster.sync();  // both halves transformed
    const float2 *A = cluster.map_shared_rank(sm, 0);
    const float2 *B = cluster.map_shared_rank(sm, 1);
    float inv = 1.f;
    if (STORE == SARBP_STORE_C32H) {
        const float bound = __ldg(&bound2[2 * p]) + __ldg(&bound2[2 * p + 1]);
        float sc = 1.f;
        if (bound > 0.f && isfinite(bound)) sc = exp2f(ceilf(log2f(bound) - 14.f));
        inv = 1.f / sc;
        if (r == 0 && h == 0 && threadIdx.x == 0) scale[p] = sc;
    }
    const int i0 = h * (M / 2), i1 = i0 + M / 2;
    for (int i = i0 + threadIdx.x; i < i1; i += T) {
        const float2 a = A[sw(i)];
        const float2 t = cmul(E(L * i), B[sw(i)]);  // W_N^{-i} B[i]
        const float2 y0 = cadd(a, t), y1 = csub(a, t);
        if (STORE == SARBP_STORE_C64) {
            float2 *o = reinterpret_cast<float2 *>(out) + (size_t)p * nbins + r;
            if (i < ns) o[(size_t)L * i] = y0;
            if (i + M < ns) o[(size_t)L * (i + M)] = y1;
        } else {
            __half2 *o = reinterpret_cast<__half2 *>(out) + (size_t)p * nbins + r;
            if (i < ns) o[(size_t)L * i] = __floats2half2_rn(y0.x * inv, y0.y * inv);
            if (i + M < ns) o[(size_t)L * (i + M)] = __floats2half2_rn(y1.x * inv, y1.y * inv);
        }
    }
    cluster.sync();  // the partner has finished reading this CTA's shared memory
}

// FFT sizes from this one up run as two half-size CTAs (forward) or 2-CTA
// clusters (inverse); 32768 always does (its data exceed one CTA's shared memory).
#ifndef SARBP_RC_SPLIT_MIN
#define SARBP_RC_SPLIT_MIN 32768
#endif
#ifndef SARBP_RC_BIG_THREADS
#define SARBP_RC_BIG_THREADS 1024
#endif
template <int N>
constexpr int threads_for() {
    return N >= 8192 ? SARBP_RC_BIG_THREADS : (N >= 4096 ? 512 : (N >= 512 ? N / 8 : 64));
}


template <int N>
cudaError_t fwd_n(const RcPlan &p, const float2 *echo, const float2 *filt, const float2 *etab,
                  float2 *spec, float *scale, cudaStream_t s) {
    constexpr int T = threads_for<N>();
    const size_t smem = sizeof(float2) * N + kTabSmem;
    auto k = rc_forward_kernel<N, T>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<p.np, T, smem, s>>>(p.ns, p.L, echo, filt, etab, spec, scale);
    return cudaGetLastError();
}

template <int N>
cudaError_t inv_n(const RcPlan &p, const float2 *spec, const float2 *etab, const float *scale, void *out,
                  cudaStream_t s) {
    constexpr int T = threads_for<N>();
    const size_t smem = sizeof(float2) * N + kTabSmem;
    cudaError_t e;
    if (p.storage == SARBP_STORE_C64) {
        auto k = rc_inverse_kernel<N, T, SARBP_STORE_C64>;
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<p.np * p.L, T, smem, s>>>(p.ns, p.L, p.nbins, spec, etab, scale, out);
    } else {
        auto k = rc_inverse_kernel<N, T, SARBP_STORE_C32H>;
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<p.np * p.L, T, smem, s>>>(p.ns, p.L, p.nbins, spec, etab, scale, out);
    }
    return cudaGetLastError();
}

template <int M>
cudaError_t fwd2(const RcPlan &p, const float2 *echo, const float2 *filt, const float2 *etab, float2 *spec,
                 float *bound2, cudaStream_t s) {
    constexpr int T = threads_for<M>();
    const size_t smem = sizeof(float2) * M + kTabSmem;
    auto k = rc_forward2_kernel<M, T>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<2 * p.np, T, smem, s>>>(p.ns, p.L, echo, filt, etab, spec, bound2);
    return cudaGetLastError();
}

template <int M>
cudaError_t inv2(const RcPlan &p, const float2 *spec, const float2 *etab, const float *bound2, float *scale,
                 void *out, cudaStream_t s) {
    constexpr int T = threads_for<M>();
    const size_t smem = sizeof(float2) * M + kTabSmem;
    cudaError_t e;
    if (p.storage == SARBP_STORE_C64) {
        auto k = rc_inverse2_kernel<M, T, SARBP_STORE_C64>;
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<2 * p.np * p.L, T, smem, s>>>(p.ns, p.L, p.nbins, spec, etab, bound2, scale, out);
    } else {
        auto k = rc_inverse2_kernel<M, T, SARBP_STORE_C32H>;
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<2 * p.np * p.L, T, smem, s>>>(p.ns, p.L, p.nbins, spec, etab, bound2, scale, out);
    }
    return cudaGetLastError();
}

}  // namespace

bool rc_size_supported(int nfft) {
    return nfft >= 64 && nfft <= 32768 && (nfft & (nfft - 1)) == 0;
}

#define SARBP_RC_SWITCH(N_, CALL)      \
    switch (N_) {                      \
        case 64: return CALL(64);      \
        case 128: return CALL(128);    \
        case 256: return CALL(256);    \
        case 512: return CALL(512);    \
        case 1024: return CALL(1024);  \
        case 2048: return CALL(2048);  \
        case 4096: return CALL(4096);  \
        case 8192: return CALL(8192);  \
        case 16384: return CALL(16384); \
        default: return cudaErrorInvalidValue; \
    }

cudaError_t launch_rc_forward(const RcPlan &p, const float2 *echo, const float2 *filt,
                              const float2 *etab, float2 *spec, float *scale, cudaStream_t s) {
    if (p.np <= 0) return cudaSuccess;
    if (p.L < 1 || p.L > 16) return cudaErrorInvalidValue;
    if (p.nfft >= SARBP_RC_SPLIT_MIN && p.nfft >= 8192) {
        if (!p.bound2) return cudaErrorInvalidValue;
        if (p.nfft == 32768) return fwd2<16384>(p, echo, filt, etab, spec, p.bound2, s);
        if (p.nfft == 16384) return fwd2<8192>(p, echo, filt, etab, spec, p.bound2, s);
        if (p.nfft == 8192) return fwd2<4096>(p, echo, filt, etab, spec, p.bound2, s);
    }
#define SARBP_FWD(N) fwd_n<N>(p, echo, filt, etab, spec, scale, s)
    SARBP_RC_SWITCH(p.nfft, SARBP_FWD)
#undef SARBP_FWD
}

cudaError_t launch_rc_inverse(const RcPlan &p, const float2 *spec, const float2 *etab,
                              const float *scale, void *out, cudaStream_t s) {
    if (p.np <= 0) return cudaSuccess;
    if (p.L < 1 || p.L > 16) return cudaErrorInvalidValue;
    if (p.nfft >= SARBP_RC_SPLIT_MIN && p.nfft >= 8192) {
        if (!p.bound2) return cudaErrorInvalidValue;
        float *sc = const_cast<float *>(scale);
        if (p.nfft == 32768) return inv2<16384>(p, spec, etab, p.bound2, sc, out, s);
        if (p.nfft == 16384) return inv2<8192>(p, spec, etab, p.bound2, sc, out, s);
        if (p.nfft == 8192) return inv2<4096>(p, spec, etab, p.bound2, sc, out, s);
    }
#define SARBP_INV(N) inv_n<N>(p, spec, etab, scale, out, s)
    SARBP_RC_SWITCH(p.nfft, SARBP_INV)
#undef SARBP_INV
}

}  // namespace sarbp
