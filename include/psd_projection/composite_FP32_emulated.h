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

/// The deflated projection with BF16x9 products.  The reference defines and
/// exports it (src/composite_FP32_emulated.cu:264-325) without declaring it in
/// its header; the declaration here gives the same symbol.  No defaults, as
/// there is no reference declaration to take them from.
void composite_FP32_emulated_auto_scale_deflate(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat,
                                                const int n, const size_t k, const double tol, const double ortho_tol,
                                                const bool verbose);

#endif  // CUDA_VERSION >= 12090

#endif  // PSD_PROJECTION_COMPOSITE_FP32_EMULATED_H
