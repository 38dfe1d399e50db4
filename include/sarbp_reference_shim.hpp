// sarbp_reference_shim.hpp -- the reference program's launch functions on top of libsarbp.
//
// Include this header in exactly ONE C++ translation unit of a program that
// uses the reference's BP interface, after the header that defines SARParams
// and cufftComplex (code/SAR_BP/CUDA/BPA_CUDA.h), in place of compiling
// BPA_CUDA_kernels.cu.  It defines, with the reference's C++ signatures,
//
//   void launchGenerateEcho(cufftComplex* Srnm, float* Ptarget, float* ta, float* tr,
//                           const SARParams params, int Mslow, int Nfast);
//       declared BPA_CUDA.cpp:4-6, defined BPA_CUDA_kernels.cu:79-89
//   void launchBackProjection(cufftComplex* Srnm, cufftComplex* Image,
//                             const SARParams params, int Na, int Nr);
//       declared BPA_CUDA.cpp:8-9, defined BPA_CUDA_kernels.cu:91-98
//
// and forwards them to sarbp_launch_generate_echo / sarbp_launch_back_projection.
// Error behaviour follows the reference's CHECK_CUDA (BPA_CUDA.h:11-17): print
// the failure and exit() with the status code.  Link with -lsarbp.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "sarbp.h"

namespace sarbp_shim {

template <class Params>
inline sarbp_ref_params to_ref(const Params &p) {
    static_assert(sizeof(Params) == sizeof(sarbp_ref_params),
                  "SARParams must have the reference layout: 12 floats then 3 ints");
    static_assert(std::is_trivially_copyable<Params>::value, "SARParams must be trivially copyable");
    sarbp_ref_params r;
    std::memcpy(&r, &p, sizeof r);
    return r;
}

inline void check_or_exit(sarbp_status st, const char *what) {
    if (st != SARBP_OK) {
        std::printf("sarbp error in %s: %s\n", what, sarbp_status_string(st));
        std::exit(static_cast<int>(st));
    }
}

}  // namespace sarbp_shim

void launchGenerateEcho(cufftComplex *Srnm, float *Ptarget, float *ta, float *tr, const SARParams params,
                        int Mslow, int Nfast) {
    const sarbp_ref_params r = sarbp_shim::to_ref(params);
    sarbp_shim::check_or_exit(
        sarbp_launch_generate_echo(reinterpret_cast<sarbp_complex64 *>(Srnm), Ptarget, ta, tr, &r, Mslow, Nfast),
        "launchGenerateEcho");
}

void launchBackProjection(cufftComplex *Srnm, cufftComplex *Image, const SARParams params, int Na, int Nr) {
    const sarbp_ref_params r = sarbp_shim::to_ref(params);
    sarbp_shim::check_or_exit(sarbp_launch_back_projection(reinterpret_cast<sarbp_complex64 *>(Srnm),
                                                           reinterpret_cast<sarbp_complex64 *>(Image), &r, Na, Nr),
                              "launchBackProjection");
}
