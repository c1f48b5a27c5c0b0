// composite_FP32_emulated.h — drop-in declaration of the reference's
// BF16x9-emulated FP32 composite filter (ComputationalRobotics/psd_projection
// include/psd_projection/composite_FP32_emulated.h:17-35, CUDA >= 12.9).
//
// On GB300 every product splits both operands into three BF16 terms and sums
// all nine term products on the tensor cores (FP32 accumulation).
#ifndef PSD_PROJECTION_COMPOSITE_FP32_EMULATED_H
#define PSD_PROJECTION_COMPOSITE_FP32_EMULATED_H

#include "cuda.h"

#if defined(CUDA_VERSION) && (CUDA_VERSION >= 12090)

#include <cublas_v2.h>
#include <cusolverDn.h>

void composite_FP32_emulated(cublasHandle_t cublasH, double* mat, const int mat_size, float* workspace = nullptr);

void composite_FP32_emulated_auto_scale(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat,
                                        const int mat_size, float* workspace = nullptr);

#endif  // CUDA_VERSION >= 12090

#endif  // PSD_PROJECTION_COMPOSITE_FP32_EMULATED_H
