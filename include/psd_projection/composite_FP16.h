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

#endif  // PSD_PROJECTION_COMPOSITE_FP16_H
