// wk.cu -- omega-K (Stolt) imager on sm_103a.
//
// Implements the reference's omega-K path (code/SAR_WK/wk_v5.2.3/wk.cc:43-343,
// specified by code/SAR_WK/matlab/mian_wka_sinc.m): zero padding and azimuth
// down-conversion (task/preprocess.cc:17-167), 2-D FFT (task/fft.cc:18+),
// reference-function multiply (task/compression.cc:17-73), Stolt mapping with
// a P-tap sinc kernel (task/stolt.cc:324+) and 2-D IFFT.
//
// GPU design (data [Na][Nr] complex64 in HBM, ping-pong between two buffers):
//   * 1-D DFTs along the rows, one CTA per row, in shared memory: the
//     Stockham FFT of fft_smem.cuh for power-of-two lengths (<= 16384), and
//     Bluestein's chirp-z form for other lengths n <= 8192: the row times the
//     chirp conj(w), w_j = e^{j pi j^2 / n}, is convolved with w through one
//     forward and one inverse power-of-two FFT of M >= 2n - 1 points held in
//     the same shared memory, with the convolution kernel's spectrum
//     precomputed in FP64 on the host.  The first range transform takes its
//     input straight from the echo (zero padding and azimuth down-conversion
//     fused into its load).
//   * Azimuth transforms of power-of-two lengths 512..4096 run down the
//     columns (dft_cols_kernel: 4 adjacent columns per CTA, whole 32-byte row
//     segments, the columns' butterflies batched per stage); other lengths go
//     through 32 x 32-tile transposes and the row transforms.
//   * The reference-function multiply and the Stolt interpolation are one
//     kernel per azimuth-frequency row.  With P = f0 + fr, q = c^2 fa^2 /
//     (4 Vr^2) and eps = q / P^2 <= 1e-2 (wk_stolt_ff_kernel), the phase
//     theta = 4 pi R0 / c sqrt(P^2 - q) + pi fr^2 / kr is a per-column table
//     reduced modulo 2 pi in FP64 on the host, minus a float-float term
//     (ffloat.cuh) and an FP32 remainder, so no sample needs FP64; larger eps
//     (wk_stolt_kernel) takes an FP64 square root per sample.  The Stolt shift
//     is delta = (sqrt(P^2 - q) - P) Nr / Fr; the multiplied row is staged in
//     shared memory and each output sums P taps at clip(floor(n - delta + k -
//     P/2), 0, Nr - 1) weighted by sin(pi u) / (pi u), u = (n - delta) - tap, as
//     the reference's gather / sinc / reduce chain does.  One sin per output:
//     away from the row edges the taps' sines differ only in sign.
#include <algorithm>

#include "fft_smem.cuh"
#include "ffloat.cuh"

namespace sarbp {
namespace {

// ------------------------------------------------------------------ DFT rows

#ifndef SARBP_DFT_T8192
#define SARBP_DFT_T8192 512
#endif
#ifndef SARBP_DFT_T4096
#define SARBP_DFT_T4096 512
#endif
template <int N>
constexpr int dft_threads() {
    return N >= 16384 ? 1024 : (N >= 8192 ? SARBP_DFT_T8192 : (N >= 4096 ? SARBP_DFT_T4096 : (N >= 512 ? N / 8 : 64)));
}

// Element i of the transformed row b: the row itself, or (fused padding and
// azimuth down-conversion) src[b][i - col0] * rowmul[b] inside the source
// columns and 0 outside.
__device__ __forceinline__ float2 dft_input(const DftIo &io, const float2 *row, int b, int i) {
    if (!io.src) return row[i];
    const int c = i - io.col0;
    if (c < 0 || c >= io.src_cols) return make_float2(0.f, 0.f);
    return cmul(__ldg(&io.src[(size_t)b * io.src_cols + c]), __ldg(&io.rowmul[b]));
}

// Power-of-two row transform: row r of data (stride ld) in place, times scale.
template <int N, int T, bool INV>
__global__ void __launch_bounds__(T, (fft_min_blocks<N, T>())) dft_pow2_kernel(float2 *__restrict__ data, long long ld, float scale,
                                                     const float2 *__restrict__ etab, DftIo io) {
    extern __shared__ float2 sm[];
    float2 *row = data + (size_t)blockIdx.x * ld;
    if constexpr (stage_radix<N, T, 1>() == N) {  // one stage: through shared memory
        const Etab E = load_etab<N, T>(sm, etab, 1);
        for (int i = threadIdx.x; i < N; i += T) sm[sw(i)] = dft_input(io, row, blockIdx.x, i);
        __syncthreads();
        fft_smem<N, T, INV>(sm, E);
        for (int i = threadIdx.x; i < N; i += T) {
            const float2 v = sm[sw(i)];
            row[i] = make_float2(v.x * scale, v.y * scale);
        }
        return;
    } else {
    // first-stage inputs straight from the row (read before any output is
    // written: the last stage runs after every thread's loads)
    using F = FirstIn<N, T>;
    float2 v[F::PER][F::R];
#pragma unroll
    for (int b = 0; b < F::PER; ++b)
#pragma unroll
        for (int r = 0; r < F::R; ++r)
            v[b][r] = F::live(b) ? dft_input(io, row, blockIdx.x, F::point(b, r)) : make_float2(0.f, 0.f);
    const Etab E = load_etab<N, T>(sm, etab, 1);
    fft_io<N, T, INV>(sm, E, v, [&](int i, float2 x) { row[i] = make_float2(x.x * scale, x.y * scale); });
    }
}

// Bluestein row transform of length n through M-point FFTs.
//   forward: X[k] = conj(w_k) sum_j (x_j conj(w_j)) w_{k-j}
//   inverse: X[k] = w_k sum_j (x_j w_j) conj(w_{k-j})
// chirp[j] = w_j (j < n); kspec = FFT_M of the circular kernel (w or conj(w)),
// divided by M (the inverse FFT's normalisation).
template <int M, int T, bool INV>
__global__ void __launch_bounds__(T, (fft_min_blocks<M, T>())) dft_bluestein_kernel(float2 *__restrict__ data, long long ld, int n,
                                                          float scale, const float2 *__restrict__ etab,
                                                          const float2 *__restrict__ chirp,
                                                          const float2 *__restrict__ kspec, DftIo io) {
    extern __shared__ float2 sm[];
    float2 *row = data + (size_t)blockIdx.x * ld;
    if constexpr (stage_radix<M, T, 1>() == M) {  // one stage: through shared memory
        const Etab E = load_etab<M, T>(sm, etab, 1);
        for (int i = threadIdx.x; i < M; i += T) {
            float2 x = make_float2(0.f, 0.f);
            if (i < n) {
                float2 w = __ldg(&chirp[i]);
                if (!INV) w.y = -w.y;
                x = cmul(dft_input(io, row, blockIdx.x, i), w);
            }
            sm[sw(i)] = x;
        }
        __syncthreads();
        fft_smem<M, T, false>(sm, E);
        for (int i = threadIdx.x; i < M; i += T) sm[sw(i)] = cmul(sm[sw(i)], __ldg(&kspec[i]));
        __syncthreads();
        fft_smem<M, T, true>(sm, E);
        for (int i = threadIdx.x; i < n; i += T) {
            float2 w = __ldg(&chirp[i]);
            if (!INV) w.y = -w.y;
            const float2 y = cmul(sm[sw(i)], w);
            row[i] = make_float2(y.x * scale, y.y * scale);
        }
        return;
    } else {
    using F = FirstIn<M, T>;
    // tables first: with the chirped inputs live through the table loads the
    // two-CTA register budget (64) spills
    const Etab E = load_etab<M, T>(sm, etab, 1);
    float2 v[F::PER][F::R];
    // forward transform of the chirped row: inputs straight into registers
#pragma unroll
    for (int b = 0; b < F::PER; ++b)
#pragma unroll
        for (int r = 0; r < F::R; ++r) {
            const int i = F::point(b, r);
            float2 x = make_float2(0.f, 0.f);
            if (F::live(b) && i < n) {
                float2 w = __ldg(&chirp[i]);
                if (!INV) w.y = -w.y;
                x = cmul(dft_input(io, row, blockIdx.x, i), w);
            }
            v[b][r] = x;
        }
    fft_io<M, T, false>(sm, E, v, SmemSink{});
    // times the kernel spectrum on the way into the inverse's first stage.
    // At the two-CTA budget of 64 registers this keeps about 120 bytes per
    // thread in (L1-resident) local memory; still faster than a separate
    // multiply pass through shared memory: 1.080 vs 1.129 ms per omega-K image.
#pragma unroll
    for (int b = 0; b < F::PER; ++b)
#pragma unroll
        for (int r = 0; r < F::R; ++r) {
            const int i = F::point(b, r);
            v[b][r] = F::live(b) ? cmul(sm[sw(i)], __ldg(&kspec[i])) : make_float2(0.f, 0.f);
        }
    __syncthreads();  // every point read before the first stage overwrites it
    fft_io<M, T, true>(sm, E, v, [&](int i, float2 x) {
        if (i < n) {
            float2 w = __ldg(&chirp[i]);
            if (!INV) w.y = -w.y;
            const float2 y = cmul(x, w);
            row[i] = make_float2(y.x * scale, y.y * scale);
        }
    });
    }
}

// Power-of-two transforms down C adjacent columns of a row-major [N][ncols]
// array, times scale, written to out (out == in: in place).  Rows of C x 8
// bytes are read and written whole (one 32-byte sector at C = 4), the C
// columns are transformed together in shared memory (sharing each stage's
// barriers; each column padded by 4 points so the columns start in different
// banks).  Replaces transpose + row transform + transpose.
#ifndef SARBP_WK_COLS
#define SARBP_WK_COLS 4
#endif
#ifndef SARBP_WK_COL_THREADS
#define SARBP_WK_COL_THREADS 512
#endif
#ifndef SARBP_WK_COL_UNROLL
#define SARBP_WK_COL_UNROLL 8
#endif
constexpr int kColUnroll = SARBP_WK_COL_UNROLL;
constexpr int kColPad = 4;
template <int N, int T, bool INV, int C>
__global__ void __launch_bounds__(T, (C <= 2 ? 2 : 1)) dft_cols_kernel(const float2 *in, float2 *out, int ncols, float scale,
                                                     const float2 *__restrict__ etab) {
    extern __shared__ float2 sm[];
    constexpr int CS = N + kColPad;
    const Etab E = load_etab_at<N, T>(sm + C * CS, etab, 1);
    const int c0 = blockIdx.x * C;
    // fill: kColUnroll loads in flight per thread (one CTA per SM: no other
    // CTA hides a load's latency)
    static_assert((N * C) % T == 0, "whole fill iterations");
#pragma unroll kColUnroll
    for (int it = 0; it < N * C / T; ++it) {
        const int e = threadIdx.x + it * T;
        const int c = e % C, i = e / C, col = c0 + c;
        sm[c * CS + sw(i)] = col < ncols ? in[(size_t)i * ncols + col] : make_float2(0.f, 0.f);
    }
    __syncthreads();  // also publishes the W tables
    StagesBatched<N, T, INV, 1, C, CS>::run(sm, E);
    for (int e = threadIdx.x; e < N * C; e += T) {
        const int c = e % C, i = e / C, col = c0 + c;
        if (col < ncols) {
            const float2 v = sm[c * CS + sw(i)];
            out[(size_t)i * ncols + col] = make_float2(v.x * scale, v.y * scale);
        }
    }
}

template <int N, bool INV>
cudaError_t cols_n(const DftPlan &p, const float2 *in, float2 *out, int ncols, float scale, cudaStream_t s) {
    constexpr int C = SARBP_WK_COLS, T = SARBP_WK_COL_THREADS;
    const size_t smem = sizeof(float2) * (size_t)C * (N + kColPad) + kTabSmem;
    auto k = dft_cols_kernel<N, T, INV, C>;
    cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void *>(k));
    if (e != cudaSuccess) return e;
    k<<<(ncols + C - 1) / C, T, smem, s>>>(in, out, ncols, scale, p.etab);
    return cudaGetLastError();
}

template <int N, bool INV>
cudaError_t pow2_n(const DftPlan &p, float2 *data, int rows, long long ld, float scale, const DftIo &io,
                   cudaStream_t s) {
    constexpr int T = dft_threads<N>();
    const size_t smem = sizeof(float2) * N + kTabSmem;
    auto k = dft_pow2_kernel<N, T, INV>;
    cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void *>(k));
    if (e != cudaSuccess) return e;
    k<<<rows, T, smem, s>>>(data, ld, scale, p.etab, io);
    return cudaGetLastError();
}

template <int M, bool INV>
cudaError_t blue_m(const DftPlan &p, float2 *data, int rows, long long ld, float scale, const DftIo &io,
                   cudaStream_t s) {
    constexpr int T = dft_threads<M>();
    const size_t smem = sizeof(float2) * M + kTabSmem;
    auto k = dft_bluestein_kernel<M, T, INV>;
    cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void *>(k));
    if (e != cudaSuccess) return e;
    k<<<rows, T, smem, s>>>(data, ld, p.n, scale, p.etab, p.chirp, INV ? p.kinv : p.kfwd, io);
    return cudaGetLastError();
}

template <bool INV>
cudaError_t dft_dispatch(const DftPlan &p, float2 *data, int rows, long long ld, float scale, const DftIo &io,
                         cudaStream_t s) {
#define SARBP_DFT_CASE(F, V) \
    case V: return F<V, INV>(p, data, rows, ld, scale, io, s);
    if (p.m == 0) {
        switch (p.n) {
            SARBP_DFT_CASE(pow2_n, 2) SARBP_DFT_CASE(pow2_n, 4) SARBP_DFT_CASE(pow2_n, 8)
            SARBP_DFT_CASE(pow2_n, 16) SARBP_DFT_CASE(pow2_n, 32) SARBP_DFT_CASE(pow2_n, 64)
            SARBP_DFT_CASE(pow2_n, 128) SARBP_DFT_CASE(pow2_n, 256) SARBP_DFT_CASE(pow2_n, 512)
            SARBP_DFT_CASE(pow2_n, 1024) SARBP_DFT_CASE(pow2_n, 2048) SARBP_DFT_CASE(pow2_n, 4096)
            SARBP_DFT_CASE(pow2_n, 8192) SARBP_DFT_CASE(pow2_n, 16384)
            default: return cudaErrorInvalidValue;
        }
    }
    switch (p.m) {
        SARBP_DFT_CASE(blue_m, 4) SARBP_DFT_CASE(blue_m, 8) SARBP_DFT_CASE(blue_m, 16)
        SARBP_DFT_CASE(blue_m, 32) SARBP_DFT_CASE(blue_m, 64) SARBP_DFT_CASE(blue_m, 128)
        SARBP_DFT_CASE(blue_m, 256) SARBP_DFT_CASE(blue_m, 512) SARBP_DFT_CASE(blue_m, 1024)
        SARBP_DFT_CASE(blue_m, 2048) SARBP_DFT_CASE(blue_m, 4096) SARBP_DFT_CASE(blue_m, 8192)
        SARBP_DFT_CASE(blue_m, 16384)
        default: return cudaErrorInvalidValue;
    }
#undef SARBP_DFT_CASE
}

// ------------------------------------------------------------------ transpose

constexpr int kTile = 32;

// out[c][r] = in[r][c] for a dense rows x cols matrix.
__global__ void __launch_bounds__(kTile * 8) transpose_kernel(const float2 *__restrict__ in, float2 *__restrict__ out,
                                                               int rows, int cols) {
    __shared__ float2 t[kTile][kTile + 1];
    const int c0 = blockIdx.x * kTile, r0 = blockIdx.y * kTile;
    for (int i = threadIdx.y; i < kTile; i += 8) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) t[i][threadIdx.x] = in[(size_t)r * cols + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < kTile; i += 8) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (c < cols && r < rows) out[(size_t)c * rows + r] = t[threadIdx.x][i];
    }
}

// ------------------------------------------------------------------ RFM + Stolt

constexpr int kStoltThreads = 512;

// Stolt taps of one row: out[n] = sum over k of w_k sm[idx_k],
// idx_k = clip(floor(n - delta[n] + k - taps/2), 0, NR - 1),
// w_k = sin(pi u) / (pi u), u = n - delta[n] - idx_k.
__device__ __forceinline__ void stolt_taps(const float2 *sm, const float *sdelta, float2 *dst, int NR, int taps) {
    const float half = 0.5f * (float)taps;
    for (int n = threadIdx.x; n < NR; n += kStoltThreads) {
        // centre c = n - delta = fl + f, f in [0, 1)
        const float nd = -sdelta[n];
        const float fnd = floorf(nd);
        const float f = nd - fnd;
        const int fl = n + (int)fnd;
        const float s0 = sinpif(f);  // sin(pi (f + o)) = (-1)^o s0 for integer o
        float2 acc = make_float2(0.f, 0.f);
        for (int k = 0; k < taps; ++k) {
            // tap floor(c + k - taps/2), clipped to the row (stolt.cc: arange, floor, clip)
            const int t = fl + (int)floorf(f + ((float)k - half));
            const int idx = min(max(t, 0), NR - 1);
            const float u = f + (float)(fl - idx);  // c - idx
            float w;
            if (u == 0.f) {
                w = 1.f;
            } else {
                const float s = (idx == t) ? (((fl - idx) & 1) ? -s0 : s0) : sinpif(u);
                // |pi u| is in [1e-7, 10): the reciprocal-based quotient (<= 2 ulp)
                // is far inside the stage's FP32 error
                w = __fdividef(s, 3.14159265358979323846f * u);
            }
            const float2 v = sm[idx];
            acc.x = fmaf(w, v.x, acc.x);
            acc.y = fmaf(w, v.y, acc.y);
        }
        dst[n] = acc;
    }
}

// One CTA per azimuth-frequency row m of in/out ([NA][NR]).
//   col_f2[n]  = (f0 + fr_n)^2,  col_ph[n] = pi fr_n^2 / kr,  col_fr[n] = fr_n
//   row_q[m]   = c^2 fa_m^2 / (4 Vr^2)
__global__ void __launch_bounds__(kStoltThreads) wk_stolt_kernel(const float2 *__restrict__ in,
                                                                  float2 *__restrict__ out, int NR,
                                                                  const double *__restrict__ col_f2,
                                                                  const double *__restrict__ col_ph,
                                                                  const double *__restrict__ col_fr,
                                                                  const double *__restrict__ row_q, double a4r,
                                                                  double f0, double inv_gap, int taps) {
    extern __shared__ float2 sm[];
    float *sdelta = reinterpret_cast<float *>(sm + NR);
    const int m = blockIdx.x;
    const double q = row_q[m];
    const float2 *src = in + (size_t)m * NR;
    constexpr double kTwoPi = 6.283185307179586476925;
    for (int n = threadIdx.x; n < NR; n += kStoltThreads) {
        const double root = sqrt(fmax(col_f2[n] - q, 0.0));
        double th = fma(a4r, root, col_ph[n]);
        th -= kTwoPi * rint(th * (1.0 / kTwoPi));
        float sn, cs;
        sincosf((float)th, &sn, &cs);
        sm[n] = cmul(__ldg(&src[n]), make_float2(cs, sn));
        sdelta[n] = (float)((root - f0 - col_fr[n]) * inv_gap);
    }
    __syncthreads();
    stolt_taps(sm, sdelta, out + (size_t)m * NR, NR, taps);
}

// The same stage without FP64 arithmetic per sample.  With P = f0 + fr_n,
// eps = q_m / P^2 and s = sqrt(1 - eps):
//   root = P - u h,  u = q_m / P,  h = 1 / (1 + s) = 1/2 + eps / (2 (1 + s)^2)
//   theta = [A P + pi fr^2 / kr] - A u / 2 - A u (h - 1/2)
// The bracket is a per-column table reduced modulo 2 pi in FP64 on the host;
// A u / 2 (~1e5 rad) is formed and reduced in float-float; the last term
// (A u eps / 8, tens of radians when eps <= 1e-2) is FP32.
//   col_c[n] = (A P + pi fr^2 / kr) mod 2 pi,  col_ip[n] = 1 / P (float pair)
//   row_q[m] = q_m (float pair),  a2 = A / 2 (float pair)
__global__ void __launch_bounds__(kStoltThreads) wk_stolt_ff_kernel(const float2 *__restrict__ in,
                                                                     float2 *__restrict__ out, int NR,
                                                                     const float *__restrict__ col_c,
                                                                     const float2 *__restrict__ col_ip,
                                                                     const float2 *__restrict__ row_q, float a2h,
                                                                     float a2l, float a, float nr_over_fr,
                                                                     int taps) {
    extern __shared__ float2 sm[];
    float *sdelta = reinterpret_cast<float *>(sm + NR);
    const int m = blockIdx.x;
    const float2 qv = __ldg(&row_q[m]);
    const ff q{qv.x, qv.y};
    const ff a2{a2h, a2l};
    const ff two_pi{6.28318548202514648438f, -1.74845553e-07f};
    const float2 *src = in + (size_t)m * NR;
    for (int n = threadIdx.x; n < NR; n += kStoltThreads) {
        const float2 ipv = __ldg(&col_ip[n]);
        const ff u = ff_mul(q, ff{ipv.x, ipv.y});
        const float eps = u.h * ipv.x;
        const float sq = sqrtf(1.f - eps);
        const float op = 1.f + sq;
        const float h = 1.f / op;
        const float hm = eps * (0.5f * h * h);  // h - 1/2
        const ff d = ff_mul(u, a2);             // A u / 2
        const float k = rintf(d.h * 0.159154943091895335769f);
        const ff dr = ff_add(d, ff_mul_f(two_pi, -k));
        float th = __ldg(&col_c[n]) - (dr.h + dr.l) - a * u.h * hm;
        th -= 6.28318530717958647692f * rintf(th * 0.159154943091895335769f);
        float sn, cs;
        __sincosf(th, &sn, &cs);
        sm[n] = cmul(__ldg(&src[n]), make_float2(cs, sn));
        sdelta[n] = -u.h * h * nr_over_fr;  // (root - P) Nr / Fr
    }
    __syncthreads();
    stolt_taps(sm, sdelta, out + (size_t)m * NR, NR, taps);
}

}  // namespace

bool dft_size_supported(int n) {
    if (n < 2 || n > 16384) return false;
    if ((n & (n - 1)) == 0) return true;
    return n <= 8192;
}

int dft_bluestein_size(int n) {
    if ((n & (n - 1)) == 0) return 0;
    int m = 4;
    while (m < 2 * n - 1) m <<= 1;
    return m;
}

cudaError_t launch_dft_rows(const DftPlan &p, float2 *data, int rows, long long ld, bool inverse, float scale,
                            cudaStream_t s, const DftIo &io) {
    if (rows <= 0) return cudaSuccess;
    return inverse ? dft_dispatch<true>(p, data, rows, ld, scale, io, s)
                   : dft_dispatch<false>(p, data, rows, ld, scale, io, s);
}

// Zero padding and azimuth down-conversion into [NA][NR]: echo row m - pa at
// columns pr.., times rowmul[m] (task/preprocess.cc:17-167); HBM-bound.
__global__ void __launch_bounds__(256) wk_pad_kernel(const float2 *__restrict__ echo, int na, int nr,
                                                     const float2 *__restrict__ rowmul, int pa, int pr, int NA, int NR,
                                                     float2 *__restrict__ out) {
    const long long total = (long long)NA * NR;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total; k += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(k / NR), n = (int)(k - (long long)m * NR);
        const int a = m - pa, c = n - pr;
        float2 v = make_float2(0.f, 0.f);
        if (a >= 0 && a < na && c >= 0 && c < nr) v = cmul(__ldg(&echo[(size_t)a * nr + c]), __ldg(&rowmul[m]));
        out[k] = v;
    }
}

cudaError_t launch_wk_pad(const float2 *echo, int na, int nr, const float2 *rowmul, int pa, int pr, int NA, int NR,
                          float2 *out, cudaStream_t s) {
    const long long total = (long long)NA * NR;
    const int blocks = (int)std::min<long long>((total + 255) / 256, (long long)current_sms() * 16);
    wk_pad_kernel<<<blocks, 256, 0, s>>>(echo, na, nr, rowmul, pa, pr, NA, NR, out);
    return cudaGetLastError();
}

bool dft_cols_supported(const DftPlan &p) { return p.m == 0 && p.n >= 512 && p.n <= 4096; }

cudaError_t launch_dft_cols(const DftPlan &p, const float2 *in, float2 *out, int ncols, bool inverse, float scale,
                            cudaStream_t s) {
    if (ncols <= 0) return cudaSuccess;
    if (!dft_cols_supported(p)) return cudaErrorInvalidValue;
    switch (p.n) {
        case 512: return inverse ? cols_n<512, true>(p, in, out, ncols, scale, s) : cols_n<512, false>(p, in, out, ncols, scale, s);
        case 1024: return inverse ? cols_n<1024, true>(p, in, out, ncols, scale, s) : cols_n<1024, false>(p, in, out, ncols, scale, s);
        case 2048: return inverse ? cols_n<2048, true>(p, in, out, ncols, scale, s) : cols_n<2048, false>(p, in, out, ncols, scale, s);
        case 4096: return inverse ? cols_n<4096, true>(p, in, out, ncols, scale, s) : cols_n<4096, false>(p, in, out, ncols, scale, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_transpose(const float2 *in, float2 *out, int rows, int cols, cudaStream_t s) {
    dim3 grid((cols + kTile - 1) / kTile, (rows + kTile - 1) / kTile);
    transpose_kernel<<<grid, dim3(kTile, 8), 0, s>>>(in, out, rows, cols);
    return cudaGetLastError();
}

size_t wk_stolt_smem(int NR) { return (size_t)NR * (sizeof(float2) + sizeof(float)); }

cudaError_t launch_wk_stolt_ff(const float2 *in, float2 *out, int NA, int NR, const float *col_c,
                               const float2 *col_ip, const float2 *row_q, double a4r, double nr_over_fr, int taps,
                               cudaStream_t s) {
    const size_t smem = wk_stolt_smem(NR);
    cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void *>(wk_stolt_ff_kernel));
    if (e != cudaSuccess) return e;
    const double a2 = 0.5 * a4r;
    const float a2h = (float)a2, a2l = (float)(a2 - (double)a2h);
    wk_stolt_ff_kernel<<<NA, kStoltThreads, smem, s>>>(in, out, NR, col_c, col_ip, row_q, a2h, a2l, (float)a4r,
                                                       (float)nr_over_fr, taps);
    return cudaGetLastError();
}

cudaError_t launch_wk_stolt(const float2 *in, float2 *out, int NA, int NR, const double *col_f2, const double *col_ph,
                            const double *col_fr, const double *row_q, double a4r, double f0, double inv_gap, int taps,
                            cudaStream_t s) {
    const size_t smem = wk_stolt_smem(NR);
    cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void *>(wk_stolt_kernel));
    if (e != cudaSuccess) return e;
    wk_stolt_kernel<<<NA, kStoltThreads, smem, s>>>(in, out, NR, col_f2, col_ph, col_fr, row_q, a4r, f0, inv_gap, taps);
    return cudaGetLastError();
}

}  // namespace sarbp
