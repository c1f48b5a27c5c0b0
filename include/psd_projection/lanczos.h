// lanczos.h — drop-in declaration of the reference's spectral-norm bound
// (ComputationalRobotics/psd_projection include/psd_projection/lanczos.h:11-17).
#ifndef PSD_PROJECTION_LANCZOS_H
#define PSD_PROJECTION_LANCZOS_H

#include <cstddef>
#include <cublas_v2.h>
#include <cusolverDn.h>

/// Lanczos on A^T A for a square n x n device matrix A (column-major).
/// Writes to the host doubles lo and up with lo = sqrt(theta) and
/// up = sqrt(theta + ||r||), theta being the largest Ritz value and r the
/// residual the reference computes.  max_iter is capped at n; the recurrence
/// stops early when beta_k <= tol * alpha_k (k > 1) or beta_k == 0.
void approximate_two_norm(cublasHandle_t cublasH, cusolverDnHandle_t cusolverH, const double* A, size_t n,
                          double* lo, double* up, size_t max_iter = 20, double tol = 1e-10);

#endif  // PSD_PROJECTION_LANCZOS_H
