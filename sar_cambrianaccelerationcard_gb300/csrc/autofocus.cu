// autofocus.cu -- image-domain pieces of the sharpness autofocus.
//
// The autofocus (sarbp_autofocus in api.cpp) maximises S = sum |I|^4 over
// per-pulse phases.  Its gradient with respect to pulse p's phase is
// -4 Im(sum conj(W) term_p) with W = |I|^2 I, so each iteration needs W and S
// of the current image (this file) and one weighted projection (bp.cu,
// launch_project).  The reference has no autofocus; its imaging uses the
// nominal track (code/SAR_BP/matlab/BPA_SAR.m:182).
#include "sarbp_internal.h"

namespace sarbp {
namespace {

constexpr int kThreads = 256;

// w[i] = |img[i]|^2 img[i] (skipped when w is null); partial[block] = the
// block's sum of |img|^4 in FP64 (fixed reduction order per block).
__global__ void __launch_bounds__(kThreads) sharpness_weight_kernel(const float2 *__restrict__ img, size_t n,
                                                                      float2 *__restrict__ w,
                                                                      double *__restrict__ partial) {
    __shared__ double red[kThreads];
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)kThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kThreads) {
        const float2 v = img[i];
        const float a2 = fmaf(v.x, v.x, v.y * v.y);
        if (w) w[i] = make_float2(a2 * v.x, a2 * v.y);
        acc += (double)a2 * (double)a2;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

}  // namespace

int sharpness_blocks(size_t n) {
    const size_t b = (n + kThreads - 1) / kThreads;
    return (int)(b < 1024 ? (b > 0 ? b : 1) : 1024);
}

cudaError_t launch_sharpness_weight(const float2 *img, size_t n, float2 *w, double *partial, cudaStream_t s) {
    sharpness_weight_kernel<<<sharpness_blocks(n), kThreads, 0, s>>>(img, n, w, partial);
    return cudaGetLastError();
}

}  // namespace sarbp
