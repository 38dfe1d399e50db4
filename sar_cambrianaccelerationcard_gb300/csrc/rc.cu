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
// The FFT is a Stockham autosort transform with radix-32/16/8 stages (one
// radix-4 or radix-2 stage for the remaining factor), in place in shared
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

#include "fft_smem.cuh"

namespace sarbp {
namespace {

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

// SCALE: also the per-pulse bound sum_k |Y[k]| and the FP16 storage scale
// from it (complex16 rows only).
template <int N, int T, bool SCALE>
__global__ void __launch_bounds__(T, (fft_min_blocks<N, T>())) rc_forward_kernel(int ns, int L, const float2 *__restrict__ echo,
                                                       const float2 *__restrict__ filt,
                                                       const float2 *__restrict__ etab,
                                                       float2 *__restrict__ spec,
                                                       float *__restrict__ scale) {
    extern __shared__ float2 sm[];
    __shared__ float red[32];
    const int p = blockIdx.x;
    // first-stage inputs straight from the echo row (zero padding past ns),
    // issued before the table loads so both latencies overlap
    using F = FirstIn<N, T>;
    float2 v[F::PER][F::R];
    const float2 *row = echo + (size_t)p * ns;
#pragma unroll
    for (int b = 0; b < F::PER; ++b)
#pragma unroll
        for (int r = 0; r < F::R; ++r) {
            const int i = F::point(b, r);
            v[b][r] = (F::live(b) && i < ns) ? __ldg(&row[i]) : make_float2(0.f, 0.f);
        }
    const Etab E = load_etab<N, T>(sm, etab, L);  // the first stage's barrier publishes the W tables
    float2 *out = spec + (size_t)p * N;
    float acc = 0.f;
    fft_io<N, T, false>(sm, E, v, [&](int k, float2 x) {
        const float2 y = cmul(x, __ldg(&filt[k]));
        out[k] = y;
        if constexpr (SCALE) acc += sqrtf(fmaf(y.x, y.x, y.y * y.y));
    });
    if constexpr (!SCALE) return;
    const float bound = block_sum<T>(acc, red);
    if (threadIdx.x == 0) {
        // power-of-two scale so that stored FP16 magnitudes stay <= 2^14
        float sc = 1.f;
        if (bound > 0.f && isfinite(bound)) sc = exp2f(ceilf(log2f(bound) - 14.f));
        scale[p] = sc;
    }
}

template <int N, int T, int STORE>
__global__ void __launch_bounds__(T, (fft_min_blocks<N, T>())) rc_inverse_kernel(int ns, int L, int nbins,
                                                       const float2 *__restrict__ spec,
                                                       const float2 *__restrict__ etab,
                                                       const float *__restrict__ scale,
                                                       void *__restrict__ out) {
    extern __shared__ float2 sm[];
    const int p = blockIdx.x / L;
    const int r = blockIdx.x - p * L;
    const float2 *in = spec + (size_t)p * N;
    const int LN = L * N;
    // first-stage inputs straight from the spectrum, issued before the tables
    using F = FirstIn<N, T>;
    float2 v[F::PER][F::R];
#pragma unroll
    for (int b = 0; b < F::PER; ++b)
#pragma unroll
        for (int q = 0; q < F::R; ++q)
            v[b][q] = F::live(b) ? __ldg(&in[F::point(b, q)]) : make_float2(0.f, 0.f);
    const Etab E = load_etab<N, T>(sm, etab, L);
    // Ramp E^{kappa r}, kappa the signed frequency (MATLAB split floor((N+1)/2)
    // = N/2 for even N).  With k = tid + T i (every first-stage point of a
    // thread is congruent to tid mod T when N / R is a multiple of T) and N/2 a
    // multiple of T it factors into a per-thread E^{tid r} and a per-CTA table
    // over i that also carries the E^{-N r} of the negative half.
    constexpr bool kTwoLevel = (N / 2) % T == 0 && N / T <= kRampMax && F::NB % T == 0;
    float2 *rt = ramp_slots<N>(sm);
    float2 base = make_float2(1.f, 0.f);
    if (kTwoLevel && r != 0) {
        if (threadIdx.x < N / T) {
            const int i = threadIdx.x;
            float2 w = E((T * i * r) & (LN - 1));
            if (T * i >= N / 2) w = cmul(w, E((LN - N * r) & (LN - 1)));
            rt[i] = w;
        }
        base = E((int)(threadIdx.x * r) & (LN - 1));
    }
    __syncthreads();
    if (r != 0) {
#pragma unroll
        for (int b = 0; b < F::PER; ++b)
#pragma unroll
            for (int q = 0; q < F::R; ++q) {
                const int k = F::point(b, q);
                if (kTwoLevel) {
                    v[b][q] = cmul(cmul(v[b][q], base), rt[k / T]);
                } else {
                    const int kap = k < N / 2 ? k : k - N;
                    v[b][q] = cmul(v[b][q], E((kap * r) & (LN - 1)));  // LN is a power of two
                }
            }
    }
    if (STORE == SARBP_STORE_C64) {
        float2 *o = reinterpret_cast<float2 *>(out) + (size_t)p * nbins + r;
        fft_io<N, T, true>(sm, E, v, [&](int i, float2 x) {
            if (i < ns) o[(size_t)L * i] = x;
        });
    } else {
        const float inv = 1.f / __ldg(&scale[p]);  // exact: scale is a power of two
        __half2 *o = reinterpret_cast<__half2 *>(out) + (size_t)p * nbins + r;
        fft_io<N, T, true>(sm, E, v, [&](int i, float2 x) {
            if (i < ns) o[(size_t)L * i] = __floats2half2_rn(x.x * inv, x.y * inv);
        });
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
    const Etab E = load_etab<M, T>(sm, etab, 2 * L);  // E tables published by its barrier
    const float2 *row = echo + (size_t)p * ns;
    using F = FirstIn<M, T>;
    float2 v[F::PER][F::R];
#pragma unroll
    for (int b = 0; b < F::PER; ++b)
#pragma unroll
        for (int q = 0; q < F::R; ++q) {
            const int i = F::point(b, q);
            const float2 x0 = (F::live(b) && i < ns) ? __ldg(&row[i]) : make_float2(0.f, 0.f);
            const float2 x1 = (F::live(b) && i + M < ns) ? __ldg(&row[i + M]) : make_float2(0.f, 0.f);
            if (h == 0) {
                v[b][q] = cadd(x0, x1);
            } else {
                float2 w = E(L * i);  // W_N^i = conj(E^{L i})
                w.y = -w.y;
                v[b][q] = cmul(csub(x0, x1), w);
            }
        }
    float2 *out = spec + (size_t)p * (2 * M);
    float acc = 0.f;
    fft_io<M, T, false>(sm, E, v, [&](int k, float2 x) {
        const int idx = 2 * k + h;
        const float2 y = cmul(x, __ldg(&filt[idx]));
        out[idx] = y;
        acc += sqrtf(fmaf(y.x, y.x, y.y * y.y));
    });
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
    const float2 *in = spec + (size_t)p * N;
    // first-stage inputs (bins 2k + h) straight into registers, issued before
    // the table loads; the ramp needs the tables
    using F = FirstIn<M, T>;
    float2 v[F::PER][F::R];
#pragma unroll
    for (int b = 0; b < F::PER; ++b)
#pragma unroll
        for (int q = 0; q < F::R; ++q)
            v[b][q] = F::live(b) ? __ldg(&in[2 * F::point(b, q) + h]) : make_float2(0.f, 0.f);
    const Etab E = load_etab<M, T>(sm, etab, 2 * L);
    if (r != 0) {  // the ramp reads only the E tables, published by load_etab's barrier
#pragma unroll
        for (int b = 0; b < F::PER; ++b)
#pragma unroll
            for (int q = 0; q < F::R; ++q) {
                const int idx = 2 * F::point(b, q) + h;
                const int kap = idx < N / 2 ? idx : idx - N;
                v[b][q] = cmul(v[b][q], E((kap * r) & (LN - 1)));  // LN is a power of two
            }
    }
    fft_io<M, T, true>(sm, E, v, SmemSink{});  // the partner reads the result from shared memory
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
// CTA sizes (threads) per transform length, measured on GB300 (ms for 4096
// pulses, forward + eight inverse transforms each).  8192 points: 1.886 at
// 1024 threads (one CTA per SM: its barriers are overlapped by nothing), 1.295
// at 512 (two CTAs per SM), 1.123 at 256 (two per SM, 32 points per thread:
// radix-32 stages 32-32-8).  16384 points (128 KB, one CTA per SM whatever the
// size): 3.077 at 1024 (16-16-16-4), 2.986 at 512 (32-32-16).  The 16384-point
// halves of the 32768-point split path: 4.35 at 1024, 4.29 at 512 (radix-16),
// 4.17 at 512 with radix-32 stages (2048 pulses).
#ifndef SARBP_RC_8K_THREADS
#define SARBP_RC_8K_THREADS 256
#endif
#ifndef SARBP_RC_BIG_THREADS
#define SARBP_RC_BIG_THREADS 512
#endif
#ifndef SARBP_RC_HALF_THREADS
#define SARBP_RC_HALF_THREADS 512
#endif
template <int N>
constexpr int threads_for() {
    return N >= 16384 ? SARBP_RC_BIG_THREADS : (N >= 8192 ? SARBP_RC_8K_THREADS : (N >= 4096 ? 512 : (N >= 512 ? N / 8 : 64)));
}
// the half-size transforms of the split path (two CTAs / a 2-CTA cluster per transform)
template <int M>
constexpr int threads_for_half() {
    return M >= 16384 ? SARBP_RC_HALF_THREADS : threads_for<M>();
}

// With t_prepare set the launchers below configure their kernel and return
// without launching it (prepare_rc_kernels).
thread_local bool t_prepare = false;

template <int N>
cudaError_t fwd_n(const RcPlan &p, const float2 *echo, const float2 *filt, const float2 *etab,
                  float2 *spec, float *scale, cudaStream_t s) {
    constexpr int T = threads_for<N>();
    const size_t smem = sizeof(float2) * N + kTabSmem;
    // the FP16 scale only for complex16 rows (a scale array is ignored otherwise)
    auto k = p.storage == SARBP_STORE_C32H ? rc_forward_kernel<N, T, true> : rc_forward_kernel<N, T, false>;
    cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void *>(k));
    if (e != cudaSuccess || t_prepare) return e;
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
        e = allow_dynamic_smem(reinterpret_cast<const void *>(k));
        if (e != cudaSuccess || t_prepare) return e;
        k<<<p.np * p.L, T, smem, s>>>(p.ns, p.L, p.nbins, spec, etab, scale, out);
    } else {
        auto k = rc_inverse_kernel<N, T, SARBP_STORE_C32H>;
        e = allow_dynamic_smem(reinterpret_cast<const void *>(k));
        if (e != cudaSuccess || t_prepare) return e;
        k<<<p.np * p.L, T, smem, s>>>(p.ns, p.L, p.nbins, spec, etab, scale, out);
    }
    return cudaGetLastError();
}

template <int M>
cudaError_t fwd2(const RcPlan &p, const float2 *echo, const float2 *filt, const float2 *etab, float2 *spec,
                 float *bound2, cudaStream_t s) {
    constexpr int T = threads_for_half<M>();
    const size_t smem = sizeof(float2) * M + kTabSmem;
    auto k = rc_forward2_kernel<M, T>;
    cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void *>(k));
    if (e != cudaSuccess || t_prepare) return e;
    k<<<2 * p.np, T, smem, s>>>(p.ns, p.L, echo, filt, etab, spec, bound2);
    return cudaGetLastError();
}

template <int M>
cudaError_t inv2(const RcPlan &p, const float2 *spec, const float2 *etab, const float *bound2, float *scale,
                 void *out, cudaStream_t s) {
    constexpr int T = threads_for_half<M>();
    const size_t smem = sizeof(float2) * M + kTabSmem;
    cudaError_t e;
    if (p.storage == SARBP_STORE_C64) {
        auto k = rc_inverse2_kernel<M, T, SARBP_STORE_C64>;
        e = allow_dynamic_smem(reinterpret_cast<const void *>(k));
        if (e != cudaSuccess || t_prepare) return e;
        k<<<2 * p.np * p.L, T, smem, s>>>(p.ns, p.L, p.nbins, spec, etab, bound2, scale, out);
    } else {
        auto k = rc_inverse2_kernel<M, T, SARBP_STORE_C32H>;
        e = allow_dynamic_smem(reinterpret_cast<const void *>(k));
        if (e != cudaSuccess || t_prepare) return e;
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
        if (!p.bound2 && !t_prepare) return cudaErrorInvalidValue;
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
        if (!p.bound2 && !t_prepare) return cudaErrorInvalidValue;
        float *sc = const_cast<float *>(scale);
        if (p.nfft == 32768) return inv2<16384>(p, spec, etab, p.bound2, sc, out, s);
        if (p.nfft == 16384) return inv2<8192>(p, spec, etab, p.bound2, sc, out, s);
        if (p.nfft == 8192) return inv2<4096>(p, spec, etab, p.bound2, sc, out, s);
    }
#define SARBP_INV(N) inv_n<N>(p, spec, etab, scale, out, s)
    SARBP_RC_SWITCH(p.nfft, SARBP_INV)
#undef SARBP_INV
}

cudaError_t prepare_rc_kernels(const RcPlan &p) {
    if (p.L < 1 || p.L > 16) return cudaErrorInvalidValue;
    RcPlan q = p;
    q.np = 1;  // the launchers return early for empty plans
    t_prepare = true;
    cudaError_t e = launch_rc_forward(q, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (e == cudaSuccess) e = launch_rc_inverse(q, nullptr, nullptr, nullptr, nullptr, nullptr);
    t_prepare = false;
    return e;
}

}  // namespace sarbp
