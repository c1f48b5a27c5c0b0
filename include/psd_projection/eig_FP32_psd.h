// eig_FP32_psd.h — drop-in declaration of the reference's FP32 EVD projection
// (ComputationalRobotics/psd_projection include/psd_projection/eig_FP32_psd.h:14-20).
#ifndef PSD_PROJECTION_EIG_FP32_PSD_H
#define PSD_PROJECTION_EIG_FP32_PSD_H

#include <cstddef>
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <cuda_runtime.h>

/// Projects mat (n x n, column-major, device) onto the PSD cone with
/// cuSOLVER Ssyevd on an FP32 copy.  With return_eigenvalues, returns a
/// device array (FP64) of the unclipped eigenvalues that the caller frees;
/// otherwise nullptr.
double* eig_FP32_psd(cusolverDnHandle_t solverH, cublasHandle_t cublasH, double* mat, size_t mat_size,
                     bool return_eigenvalues = false);

#endif  // PSD_PROJECTION_EIG_FP32_PSD_H
