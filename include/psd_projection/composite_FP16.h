// composite_FP16.h — drop-in declaration of the reference's FP16 composite
// filter (ComputationalRobotics/psd_projection include/psd_projection/composite_FP16.h:12-33).
//
// On GB300 the products take one FP16 term per operand on the tensor cores
// with FP32 accumulation, the reference's 7-step table and safety factor 1.01.
#ifndef PSD_PROJECTION_COMPOSITE_FP16_H
#define PSD_PROJECTION_COMPOSITE_FP16_H

#include <cublas_v2.h>
#include <cusolverDn.h>
#include <cuda_fp16.h>

/// Projects a symmetric matrix whose spectrum lies in [-1, 1] onto the PSD
/// cone, in place (n x n, column-major, device).  The optional workspaces are
/// used together as one buffer when float_workspace holds at least
/// psdgb_composite_workspace_size(n, PSDGB_PREC_FP16) bytes; half_workspace is
/// not needed by this implementation.
void composite_FP16(cublasHandle_t cublasH, double* mat, const int n, float* float_workspace = nullptr,
                    __half* half_workspace = nullptr);

/// Lanczos bound, scaling by 1/up, composite_FP16, rescaling by up.
void composite_FP16_auto_scale(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat, const int mat_size,
                               float* float_workspace = nullptr, __half* half_workspace = nullptr);

/// Deflated FP16 projection (include/psd_projection/composite_FP16.h:35-50,
/// work in progress in the reference): the k largest and k smallest
/// eigenpairs (LOBPCG, maxiter, tol) are subtracted, the rest is bounded,
/// scaled by 1.1 * bound + 1e-5 and filtered, and the positive pairs are
/// added back.  Needs 3 k <= mat_size.  The workspaces are not needed.
void composite_FP16_auto_scale_deflate(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat,
                                       const int mat_size, float* float_workspace = nullptr,
                                       __half* half_workspace = nullptr, const size_t k = 40, const int maxiter = 100,
                                       const double tol = 1e-10, const bool verbose = false);

#endif  // PSD_PROJECTION_COMPOSITE_FP16_H
