// probe.cu -- issue-rate microbenchmarks for the back-projection roofline.
//
// The back-projection kernel is bound by instruction issue on the FP32 (FMA)
// and MUFU (sin/cos) pipes, not by HBM bandwidth or tensor cores.  These two
// kernels measure the device's sustained FP32 FMA lane rate and MUFU lane rate
// (independent dependency chains, every SM fully occupied), timed with CUDA
// events on the launching stream.
#include "sarbp_internal.h"

namespace sarbp {
namespace {

constexpr int kProbeThreads = 256;
constexpr int kChains = 8;

__global__ void __launch_bounds__(kProbeThreads) fma_probe_kernel(float *out, int iters, float a, float b) {
    float v[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) v[c] = threadIdx.x * 1e-3f + c;
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 16; ++r) {
#pragma unroll
            for (int c = 0; c < kChains; ++c) v[c] = fmaf(v[c], a, b);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += v[c];
    if (s == 12345.678f) out[0] = s;  // keeps the chains live
}

__global__ void __launch_bounds__(kProbeThreads) mufu_probe_kernel(float *out, int iters) {
    float v[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) v[c] = threadIdx.x * 1e-3f + c * 0.1f;
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 8; ++r) {
#pragma unroll
            for (int c = 0; c < kChains; ++c) {
                float sn, cs;
                __sincosf(v[c], &sn, &cs);  // one sin and one cos per step
                v[c] = sn + cs;
            }
        }
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += v[c];
    if (s == 12345.678f) out[0] = s;
}

}  // namespace

cudaError_t run_issue_probe(int sms, double *fp32_lanes_per_s, double *mufu_lanes_per_s, cudaStream_t s) {
    float *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(float));
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 8;  // 2048 threads per SM
    const int fma_iters = 2048, mufu_iters = 256;
    // warm-up then timed run of each
    for (int rep = 0; rep < 2; ++rep) {
        cudaEventRecord(a, s);
        fma_probe_kernel<<<blocks, kProbeThreads, 0, s>>>(d, fma_iters, 0.999f, 1e-3f);
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
    }
    float ms_fma = 0.f;
    cudaEventElapsedTime(&ms_fma, a, b);
    for (int rep = 0; rep < 2; ++rep) {
        cudaEventRecord(a, s);
        mufu_probe_kernel<<<blocks, kProbeThreads, 0, s>>>(d, mufu_iters);
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
    }
    float ms_mufu = 0.f;
    cudaEventElapsedTime(&ms_mufu, a, b);
    e = cudaGetLastError();
    const double threads = (double)blocks * kProbeThreads;
    if (fp32_lanes_per_s) *fp32_lanes_per_s = threads * fma_iters * 16.0 * kChains / (ms_fma * 1e-3);
    if (mufu_lanes_per_s) *mufu_lanes_per_s = threads * mufu_iters * 8.0 * kChains * 2.0 / (ms_mufu * 1e-3);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(d);
    return e;
}

}  // namespace sarbp
