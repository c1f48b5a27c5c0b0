// composite_FP32.h — drop-in declaration of the reference's FP32 composite
// filter (ComputationalRobotics/psd_projection include/psd_projection/composite_FP32.h:12-30).
// Same names, argument order, default arguments and C++ linkage, so code
// written against the reference links against libpsdgb.so unchanged.
//
// On GB300 the products run on the tensor cores with FP16 hi/lo split
// operands (three products per matrix product, FP32 accumulation), which
// gives FP32-class accuracy; the chain, coefficients and safety factors are
// the reference's 10-step table.
#ifndef PSD_PROJECTION_COMPOSITE_FP32_H
#define PSD_PROJECTION_COMPOSITE_FP32_H

#include <cublas_v2.h>
#include <cusolverDn.h>

/// Projects a symmetric matrix whose spectrum lies in [-1, 1] onto the PSD
/// cone, in place.  `mat` is n x n, column-major, on the device.  `workspace`
/// is used when it holds at least psdgb_composite_workspace_size(n,
/// PSDGB_PREC_FP16X3) bytes (12 * Np^2 with Np = n rounded up to 128, which
/// equals the reference's 3*n*n floats when n is a multiple of 128);
/// otherwise the library's cached workspace is used.
void composite_FP32(cublasHandle_t cublasH, double* mat, const int mat_size, float* workspace = nullptr);

/// Lanczos bound, scaling by 1/up, composite_FP32, rescaling by up.
void composite_FP32_auto_scale(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat, const int mat_size,
                               float* workspace = nullptr);

/// Deflated projection (include/psd_projection/composite_FP32.h:32-45, work
/// in progress in the reference): the k largest-|lambda| eigenpairs
/// (compute_eigenpairs with max_iter = n and ortho_tol) are subtracted, the
/// rest is scaled by 1.1 * bound + 1e-5 and filtered, and the positive pairs
/// are added back.
void composite_FP32_auto_scale_deflate(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat,
                                       const int mat_size, const size_t k = 40, const double tol = 1e-10,
                                       const double ortho_tol = 1e-3, const bool verbose = false);

#endif  // PSD_PROJECTION_COMPOSITE_FP32_H
