// synth.cu -- point-target echo synthesis on the GPU (FP64 phase).
//
// Formula of code/SAR_BP/matlab/BPA_SAR.m:80-89 and generateEchoKernel
// (code/SAR_BP/CUDA/BPA_CUDA_kernels.cu:3-45):
//   s[p][n] = sum_k amp_k * gate(u) * exp(j (pi kr (u - tc)^2 - 2 pi fc tau_pk)),
//   u = t_rec0 + n/fs - tau_pk,  tau_pk = 2 |apc_p - tgt_k| / c,  gate = [0, tp).
// One CTA per pulse: the per-(pulse, target) delay and carrier phase are
// computed once into shared memory, then each thread owns output samples and
// visits only the targets whose gate covers it.
//
// Noise: counter-based complex Gaussian (splitmix64 hash of (seed, element
// index) -> two uniforms -> Box-Muller), sigma from the mean noiseless power.
#include "sarbp_internal.h"

#include <math_constants.h>

namespace sarbp {
namespace {

constexpr int kSynthThreads = 256;
constexpr int kMaxTargets = 4096;

struct TgtPre {
    double tau;  // two-way delay
    double car;  // -2 frac(fc tau): carrier phase in units of pi
    double amp;
    int lo, hi;  // samples whose gate can be open
};

__global__ void __launch_bounds__(kSynthThreads)
    echo_synth_kernel(const double *__restrict__ apc, int ns, const sarbp_target *__restrict__ tg, int nt,
                      double t_rec0, double fs, double kr, double tp, double tc, double fc, double c,
                      float2 *__restrict__ echo, double *__restrict__ power_acc) {
    extern __shared__ TgtPre s_t[];
    __shared__ double s_red[kSynthThreads / 32];
    const int p = blockIdx.x;
    const double ax = apc[3 * p], ay = apc[3 * p + 1], az = apc[3 * p + 2];
    for (int k = threadIdx.x; k < nt; k += kSynthThreads) {
        const sarbp_target T = tg[k];
        const double dx = ax - T.x, dy = ay - T.y, dz = az - T.z;
        const double tau = 2.0 * sqrt(dx * dx + dy * dy + dz * dz) / c;
        const double cyc = fc * tau;
        TgtPre q;
        q.tau = tau;
        q.car = -2.0 * (cyc - floor(cyc));
        q.amp = T.amp;
        q.lo = (int)fmax(0.0, floor((tau - t_rec0) * fs) - 1.0);
        q.hi = (int)fmin((double)(ns - 1), ceil((tau + tp - t_rec0) * fs) + 1.0);
        s_t[k] = q;
    }
    __syncthreads();
    float2 *row = echo + (size_t)p * ns;
    double pw = 0.0;
    for (int n = threadIdx.x; n < ns; n += kSynthThreads) {
        double re = 0.0, im = 0.0;
        const double tn = t_rec0 + (double)n / fs;
        for (int k = 0; k < nt; ++k) {
            const TgtPre &q = s_t[k];
            if (n < q.lo || n > q.hi) continue;
            const double u = tn - q.tau;
            if (!(u >= 0.0 && u < tp)) continue;
            const double ph = kr * (u - tc) * (u - tc) + q.car;  // units of pi
            double sn, cs;
            sincospi(ph, &sn, &cs);
            re += q.amp * cs;
            im += q.amp * sn;
        }
        row[n] = make_float2((float)re, (float)im);
        pw += re * re + im * im;
    }
    if (power_acc) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) pw += __shfl_xor_sync(0xffffffffu, pw, o);
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = pw;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < kSynthThreads / 32; ++w) t += s_red[w];
            atomicAdd(power_acc, t);
        }
    }
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__global__ void echo_noise_kernel(float2 *__restrict__ echo, int64_t count,
                                  const double *__restrict__ power_acc, double snr_db, uint64_t seed) {
    const double mean_power = *power_acc / (double)count;
    const double sigma = sqrt(mean_power / pow(10.0, snr_db / 10.0));
    const double amp = sigma / sqrt(2.0);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t h1 = mix64(seed + 0x632BE59BD9B4E019ULL * (uint64_t)(i + 1));
        const uint64_t h2 = mix64(h1 ^ 0xD1B54A32D192ED03ULL);
        const double u1 = ((double)(h1 >> 11) + 1.0) * (1.0 / 9007199254740992.0);
        const double u2 = (double)(h2 >> 11) * (1.0 / 9007199254740992.0);
        const double rad = sqrt(-2.0 * log(u1));
        double sn, cs;
        sincospi(2.0 * u2, &sn, &cs);
        float2 v = echo[i];
        v.x = (float)((double)v.x + amp * rad * cs);
        v.y = (float)((double)v.y + amp * rad * sn);
        echo[i] = v;
    }
}

// generateEchoKernel semantics (BPA_CUDA_kernels.cu:18-42) in FP64.
__global__ void ref_echo_kernel(float2 *__restrict__ Srnm, const float *__restrict__ Ptarget,
                                const float *__restrict__ ta, const float *__restrict__ tr,
                                sarbp_ref_params prm, int Mslow, int Nfast) {
    const int64_t total = (int64_t)Mslow * Nfast;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / Nfast), j = (int)(idx % Nfast);
        const double t_a = ta[i], t_r = tr[j];
        double sr = 0.0, si = 0.0;
        for (int k = 0; k < prm.Ntarget; ++k) {
            const double Az = t_a * (double)prm.vr - (double)Ptarget[3 * k];
            const double Rg = Ptarget[3 * k + 1];
            const double sig = Ptarget[3 * k + 2];
            const double H = prm.H;
            const double R = sqrt(Az * Az + Rg * Rg + H * H);
            const double tk = t_r - 2.0 * R / (double)prm.c;
            if (tk > 0.0 && tk < (double)prm.Tr && fabs(Az) < (double)prm.La / 2.0) {
                // phase / pi = Kr tk^2 - 4 R / lambda
                const double cyc2 = 2.0 * R / (double)prm.lambda;
                const double ph = (double)prm.Kr * tk * tk - 2.0 * (cyc2 - floor(cyc2));
                double sn, cs;
                sincospi(ph, &sn, &cs);
                sr += sig * cs;
                si += sig * sn;
            }
        }
        Srnm[idx] = make_float2((float)sr, (float)si);
    }
}

}  // namespace

cudaError_t launch_echo_synth(const double *apc, int np, int ns, const sarbp_target *tg, int nt,
                              double t_rec0, double fs, double kr, double tp, double tc,
                              double fc, double c, float2 *echo, double *power_acc,
                              cudaStream_t s) {
    if (np <= 0 || ns <= 0) return cudaSuccess;
    if (nt < 0 || nt > kMaxTargets) return cudaErrorInvalidValue;
    const size_t smem = sizeof(TgtPre) * (size_t)(nt > 0 ? nt : 1);
    cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void *>(echo_synth_kernel));
    if (e != cudaSuccess) return e;
    echo_synth_kernel<<<np, kSynthThreads, smem, s>>>(apc, ns, tg, nt, t_rec0, fs, kr, tp, tc, fc, c, echo,
                                                   power_acc);
    return cudaGetLastError();
}

cudaError_t launch_echo_noise(float2 *echo, int64_t count, const double *power_acc, double snr_db,
                              uint64_t seed, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>((count + 255) / 256, (int64_t)current_sms() * 16);
    echo_noise_kernel<<<blocks, 256, 0, s>>>(echo, count, power_acc, snr_db, seed);
    return cudaGetLastError();
}

cudaError_t launch_ref_echo(float2 *Srnm, const float *Ptarget, const float *ta, const float *tr,
                            const sarbp_ref_params &p, int Mslow, int Nfast, cudaStream_t s) {
    const int64_t total = (int64_t)Mslow * Nfast;
    if (total <= 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)current_sms() * 16);
    ref_echo_kernel<<<blocks, 256, 0, s>>>(Srnm, Ptarget, ta, tr, p, Mslow, Nfast);
    return cudaGetLastError();
}

}  // namespace sarbp
