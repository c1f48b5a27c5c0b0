// lobpcg.h — drop-in declaration of the reference's LOBPCG eigensolver
// (ComputationalRobotics/psd_projection include/psd_projection/lobpcg.h).
#ifndef PSD_PROJECTION_LOBPCG_H
#define PSD_PROJECTION_LOBPCG_H

#include <cublas_v2.h>
#include <cusolverDn.h>

/// The m largest eigenpairs of the symmetric n x n device matrix A
/// (column-major): V (n x m, device) receives the eigenvectors and D (m
/// values, device) the eigenvalues in decreasing order.  warmstart takes V as
/// the orthonormal start block.  Stops when ||A X - X Lambda||_F < tol or after
/// maxiter iterations.  Needs 3 m <= n.
void lobpcg(cublasHandle_t cublasH, cusolverDnHandle_t cusolverH, const double* A, double* V, double* D, const int n,
            const int m, const bool warmstart = false, const int maxiter = 100, const double tol = 1e-8,
            const bool verbose = false);

#endif  // PSD_PROJECTION_LOBPCG_H
