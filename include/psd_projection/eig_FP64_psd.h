// eig_FP64_psd.h — drop-in declaration of the reference's FP64 EVD projection
// (ComputationalRobotics/psd_projection include/psd_projection/eig_FP64_psd.h:14-20).
#ifndef PSD_PROJECTION_EIG_FP64_PSD_H
#define PSD_PROJECTION_EIG_FP64_PSD_H

#include <cstddef>
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <cuda_runtime.h>

/// Projects mat (n x n, column-major, device) onto the PSD cone with
/// cuSOLVER Dsyevd.  With return_eigenvalues, returns a device array of the n
/// unclipped eigenvalues in ascending order that the caller frees with
/// cudaFree; otherwise returns nullptr.
double* eig_FP64_psd(cusolverDnHandle_t solverH, cublasHandle_t cublasH, double* mat, size_t mat_size,
                     bool return_eigenvalues = false);

/// Deflated EVD projection (include/psd_projection/eig_FP64_psd.h:22-31):
/// the k largest and k smallest eigenpairs (LOBPCG) are subtracted, the rest
/// is projected with Dsyevd, and the positive pairs are added back.  Needs
/// 3 k <= mat_size.
void eig_FP64_deflate(cusolverDnHandle_t solverH, cublasHandle_t cublasH, double* mat, size_t mat_size,
                      const size_t k = 40, const int maxiter = 100, const double tol = 1e-10,
                      const bool verbose = false);

#endif  // PSD_PROJECTION_EIG_FP64_PSD_H
