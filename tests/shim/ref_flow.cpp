// The reference program's flow (code/SAR_BP/CUDA/main.cpp:3-19 ->
// SAR_Processor::processImage, BPA_CUDA.cpp:70-90) written against the
// reference's launch interface and linked to libsarbp through
// include/sarbp_reference_shim.hpp.  The scene keeps the reference's target
// list (BPA_CUDA.cpp:26-32) and time axes (:35-48); the record is long enough
// (Nfast samples from delay 0) to contain the targets' echoes and the aperture
// La is widened so the image focuses.  Prints "peak i j |value|" of the image.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <vector>

typedef float2 cufftComplex;

struct SARParams {  // byte layout of the reference's SARParams (BPA_CUDA.h:28-50)
    float c, fc, lambda, Kr, Tr, Br, Fr, vr, H, La, Rg0, Az0;
    int Nfast, Mslow, Ntarget;
};

#include "sarbp_reference_shim.hpp"

#define CK(x)                                                             \
    do {                                                                  \
        cudaError_t e = (x);                                              \
        if (e != cudaSuccess) {                                           \
            std::printf("cuda error %s\n", cudaGetErrorString(e));        \
            return 20;                                                    \
        }                                                                 \
    } while (0)

int main() {
    SARParams p;
    p.c = 3e8f; p.fc = 5.3e9f; p.lambda = p.c / p.fc; p.Kr = 4e12f; p.Tr = 2.5e-6f; p.Br = 1e8f;
    p.Fr = 1.2e8f; p.vr = 150.f; p.H = 5000.f; p.La = 100.f; p.Rg0 = 10000.f; p.Az0 = 0.f;
    p.Nfast = 9600; p.Mslow = 256; p.Ntarget = 5;
    const float pt[15] = {p.Az0 - 10, p.Rg0 - 20, 1.0f, p.Az0 + 20, p.Rg0 + 30, 0.8f, p.Az0 - 30, p.Rg0 + 10, 1.2f,
                          p.Az0 + 40, p.Rg0 - 40, 0.9f, p.Az0,      p.Rg0,      1.5f};
    std::vector<float> ta(p.Mslow), tr(p.Nfast);
    const float ta0 = -p.La / (2 * p.vr), ta1 = p.La / (2 * p.vr), step = (ta1 - ta0) / (p.Mslow - 1);
    for (int i = 0; i < p.Mslow; ++i) ta[i] = ta0 + i * step;
    for (int i = 0; i < p.Nfast; ++i) tr[i] = i * (1.0f / p.Fr);
    const size_t n = (size_t)p.Mslow * p.Nfast;
    cufftComplex *d_s = nullptr, *d_img = nullptr;
    float *d_pt = nullptr, *d_ta = nullptr, *d_tr = nullptr;
    CK(cudaMalloc(&d_s, n * sizeof(cufftComplex)));
    CK(cudaMalloc(&d_img, n * sizeof(cufftComplex)));
    CK(cudaMalloc(&d_pt, sizeof pt));
    CK(cudaMalloc(&d_ta, ta.size() * sizeof(float)));
    CK(cudaMalloc(&d_tr, tr.size() * sizeof(float)));
    CK(cudaMemcpy(d_pt, pt, sizeof pt, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_ta, ta.data(), ta.size() * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_tr, tr.data(), tr.size() * sizeof(float), cudaMemcpyHostToDevice));
    launchGenerateEcho(d_s, d_pt, d_ta, d_tr, p, p.Mslow, p.Nfast);
    launchBackProjection(d_s, d_img, p, p.Mslow, p.Nfast);
    std::vector<cufftComplex> img(n);
    CK(cudaMemcpy(img.data(), d_img, n * sizeof(cufftComplex), cudaMemcpyDeviceToHost));
    size_t best = 0;
    float bv = -1.f;
    for (size_t k = 0; k < n; ++k) {
        const float v = std::hypot(img[k].x, img[k].y);
        if (v > bv) { bv = v; best = k; }
    }
    std::printf("peak %zu %zu %g\n", best / p.Nfast, best % p.Nfast, bv);
    cudaFree(d_s); cudaFree(d_img); cudaFree(d_pt); cudaFree(d_ta); cudaFree(d_tr);
    return 0;
}
