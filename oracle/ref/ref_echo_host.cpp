// Runs the reference's generateEchoKernel (code/SAR_BP/CUDA/BPA_CUDA_kernels.cu:3-45)
// on the host: the kernel's definition is included unchanged from the
// reference source (cut out by the Makefile into ref_echo_kernel.inc), with
// the CUDA built-ins it reads replaced by host variables, and called once per
// thread of the reference's launch grid (ceil(Mslow Nfast / 256) x 256,
// BPA_CUDA_kernels.cu:79-89).  FP32 throughout, as on the GPU; sincosf,
// sqrtf and fabsf come from the host C library.  Test infrastructure only.
//
// usage: ref_echo_host <in.bin> <out.bin>
//   in.bin:  SARParams (60 bytes, BPA_CUDA.h:28-50) then Ptarget [Ntarget][3],
//            ta [Mslow], tr [Nfast] as float32
//   out.bin: Srnm [Mslow][Nfast] as interleaved float32 (re, im)
#include <cstdio>
#include <vector>

#include "BPA_CUDA.h"

#undef __global__
#define __global__
static uint3 blockIdx, threadIdx;
static dim3 blockDim;

#include "ref_echo_kernel.inc"

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
        return 2;
    }
    std::FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    SARParams p;
    if (std::fread(&p, sizeof p, 1, f) != 1 || p.Mslow <= 0 || p.Nfast <= 0 || p.Ntarget < 0) return 4;
    std::vector<float> pt(3 * (size_t)p.Ntarget), ta(p.Mslow), tr(p.Nfast);
    if (std::fread(pt.data(), sizeof(float), pt.size(), f) != pt.size() ||
        std::fread(ta.data(), sizeof(float), ta.size(), f) != ta.size() ||
        std::fread(tr.data(), sizeof(float), tr.size(), f) != tr.size())
        return 5;
    std::fclose(f);
    const long long total = (long long)p.Mslow * p.Nfast;
    std::vector<cufftComplex> out((size_t)total);
    blockDim.x = 256;
    const long long blocks = (total + 255) / 256;
    for (long long b = 0; b < blocks; ++b)
        for (unsigned t = 0; t < 256; ++t) {
            blockIdx.x = (unsigned)b;
            threadIdx.x = t;
            generateEchoKernel(out.data(), pt.data(), ta.data(), tr.data(), p, p.Mslow, p.Nfast);
        }
    std::FILE *g = std::fopen(argv[2], "wb");
    if (!g || std::fwrite(out.data(), sizeof(cufftComplex), out.size(), g) != out.size()) return 6;
    std::fclose(g);
    return 0;
}
