// The reference program links against libsarbp through this translation unit
// alone: its BPA_CUDA.h, then the shim that defines launchGenerateEcho and
// launchBackProjection (in place of compiling BPA_CUDA_kernels.cu).
#include "BPA_CUDA.h"
#include "sarbp_reference_shim.hpp"
