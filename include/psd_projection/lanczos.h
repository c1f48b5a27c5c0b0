// lanczos.h — drop-in declarations of the reference's spectral-norm bound and
// Lanczos eigenpairs (ComputationalRobotics/psd_projection
// include/psd_projection/lanczos.h:11-44).
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

/// The k largest-|lambda| eigenpairs of a symmetric device matrix by Lanczos
/// (the reference's compute_eigenpairs, include/psd_projection/lanczos.h:19-44,
/// marked work in progress there): max_iter steps (0 = n), Ritz pairs kept
/// when their residual is below ortho_tol and their vector is within
/// ortho_tol of orthogonal to the pairs already kept; *r <= k pairs go to the
/// device arrays eigenvalues (r) and eigenvectors (n x r, vector i at i n).
/// Returns |theta_max| + its residual + 1e-3.  As in the reference, tol is
/// not used and *r is not written when upper_bound_only.
double compute_eigenpairs(cublasHandle_t cublasH, cusolverDnHandle_t cusolverH, const double* A, size_t n,
                          const size_t k, size_t* r, double* eigenvalues, double* eigenvectors,
                          const bool upper_bound_only = false, const size_t max_iter = 0, const double tol = 1e-10,
                          const double ortho_tol = 1e-5, const bool verbose = false);

#endif  // PSD_PROJECTION_LANCZOS_H
