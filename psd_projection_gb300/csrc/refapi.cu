// refapi.cu — the reference library's C++ entry points, exported with the
// same C++ signatures (and so the same mangled symbols) as
// ComputationalRobotics/psd_projection's libpsd_lib, forwarding to the C ABI.
//
// Conventions kept from the reference:
//   * the stream is the one set on the cuBLAS handle (the reference issues
//     everything on it; cublasGetStream gives it);
//   * functions return void and report failures by printing, then continue
//     (include/psd_projection/check.h:18-57); psdgb_last_error() holds the
//     message as well;
//   * calls block until the result is in `mat` (the reference ends with
//     cudaDeviceSynchronize).
// The composite functions map to these precisions:
//   composite_FP16           -> PSDGB_PREC_FP16,   7-step schedule
//   composite_FP32           -> PSDGB_PREC_FP16X3, 10-step schedule
//   composite_FP32_emulated  -> PSDGB_PREC_BF16X9, 10-step schedule
// Their _auto_scale variants run the Lanczos bound with the reference
// defaults (max_iter 20, tol 1e-10, src/composite_FP32.cu:177-179).
#include <cstdio>

#include "psd_projection/composite_FP16.h"
#include "psd_projection/composite_FP32.h"
#include "psd_projection/composite_FP32_emulated.h"
#include "psd_projection/eig_FP32_psd.h"
#include "psd_projection/eig_FP64_psd.h"
#include "psd_projection/lanczos.h"
#include "psd_projection/lobpcg.h"
#include "psdgb.h"

namespace {

constexpr uint64_t kSeed = 0x5eed5eedull;

cudaStream_t stream_of(cublasHandle_t h) {
    cudaStream_t s = nullptr;
    if (h) cublasGetStream(h, &s);
    return s;
}

void report(psdgb_status st, const char* fn) {
    if (st != PSDGB_OK) std::printf("psdgb error %d in %s: %s\n", static_cast<int>(st), fn, psdgb_last_error());
}

// The reference documents its workspace as at least 3*n*n floats.
size_t ref_ws_bytes(const void* ws, int n) {
    return ws ? static_cast<size_t>(3) * n * n * sizeof(float) : 0;
}

void composite_any(int precision, int schedule, cublasHandle_t h, double* mat, int n, void* ws, const char* fn) {
    report(psdgb_composite(precision, schedule, mat, n, ws, ref_ws_bytes(ws, n), stream_of(h)), fn);
}

void composite_auto_any(int precision, int schedule, cublasHandle_t h, double* mat, int n, void* ws, const char* fn) {
    report(psdgb_composite_auto_scale(precision, schedule, mat, n, 20, 1e-10, kSeed, PSDGB_RESIDUAL_REFERENCE, ws,
                                      ref_ws_bytes(ws, n), stream_of(h), nullptr),
           fn);
}

double* eig_any(int fp64, cublasHandle_t h, double* mat, size_t n, bool return_eigenvalues, const char* fn) {
    double* eigs = nullptr;
    if (return_eigenvalues && n > 0) {
        if (cudaMalloc(&eigs, sizeof(double) * n) != cudaSuccess) {
            std::printf("psdgb error in %s: eigenvalue allocation failed\n", fn);
            eigs = nullptr;
        }
    }
    report(psdgb_eig_psd(fp64, mat, static_cast<int64_t>(n), eigs, stream_of(h)), fn);
    return eigs;
}

}  // namespace

void composite_FP16(cublasHandle_t cublasH, double* mat, const int n, float* float_workspace, __half* half_workspace) {
    (void)half_workspace;
    composite_any(PSDGB_PREC_FP16, PSDGB_SCHEDULE_FP16, cublasH, mat, n, float_workspace, "composite_FP16");
}

void composite_FP16_auto_scale(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat, const int mat_size,
                               float* float_workspace, __half* half_workspace) {
    (void)solverH;
    (void)half_workspace;
    composite_auto_any(PSDGB_PREC_FP16, PSDGB_SCHEDULE_FP16, cublasH, mat, mat_size, float_workspace,
                       "composite_FP16_auto_scale");
}

void composite_FP32(cublasHandle_t cublasH, double* mat, const int mat_size, float* workspace) {
    composite_any(PSDGB_PREC_FP16X3, PSDGB_SCHEDULE_FP32, cublasH, mat, mat_size, workspace, "composite_FP32");
}

void composite_FP32_auto_scale(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat, const int mat_size,
                               float* workspace) {
    (void)solverH;
    composite_auto_any(PSDGB_PREC_FP16X3, PSDGB_SCHEDULE_FP32, cublasH, mat, mat_size, workspace,
                       "composite_FP32_auto_scale");
}

void composite_FP32_emulated(cublasHandle_t cublasH, double* mat, const int mat_size, float* workspace) {
    composite_any(PSDGB_PREC_BF16X9, PSDGB_SCHEDULE_FP32, cublasH, mat, mat_size, workspace,
                  "composite_FP32_emulated");
}

void composite_FP32_emulated_auto_scale(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat,
                                        const int mat_size, float* workspace) {
    (void)solverH;
    composite_auto_any(PSDGB_PREC_BF16X9, PSDGB_SCHEDULE_FP32, cublasH, mat, mat_size, workspace,
                       "composite_FP32_emulated_auto_scale");
}

void approximate_two_norm(cublasHandle_t cublasH, cusolverDnHandle_t cusolverH, const double* A, size_t n, double* lo,
                          double* up, size_t max_iter, double tol) {
    (void)cusolverH;
    report(psdgb_two_norm(A, static_cast<int64_t>(n), lo, up, static_cast<int64_t>(max_iter), tol, kSeed,
                          PSDGB_RESIDUAL_REFERENCE, nullptr, 0, stream_of(cublasH)),
           "approximate_two_norm");
}

double compute_eigenpairs(cublasHandle_t cublasH, cusolverDnHandle_t cusolverH, const double* A, size_t n,
                          const size_t k, size_t* r, double* eigenvalues, double* eigenvectors,
                          const bool upper_bound_only, const size_t max_iter, const double tol, const double ortho_tol,
                          const bool verbose) {
    (void)cusolverH;
    int64_t rr = 0;
    double up = 0.0;
    report(psdgb_compute_eigenpairs(A, static_cast<int64_t>(n), static_cast<int64_t>(k), &rr, eigenvalues,
                                    eigenvectors, upper_bound_only ? 1 : 0, static_cast<int64_t>(max_iter), tol,
                                    ortho_tol, kSeed, &up, stream_of(cublasH)),
           "compute_eigenpairs");
    if (!upper_bound_only) {
        if (r) *r = static_cast<size_t>(rr);
        if (verbose && static_cast<size_t>(rr) < k)
            std::fprintf(stderr, "Warning: only %zu eigenpairs found, requested %zu.\n", static_cast<size_t>(rr), k);
    }
    return up;
}

namespace {
void deflate_any(int precision, cublasHandle_t h, double* mat, int n, size_t k, double tol, double ortho_tol,
                 const char* fn) {
    report(psdgb_composite_auto_scale_deflate(precision, PSDGB_SCHEDULE_FP32, mat, n, static_cast<int64_t>(k), tol,
                                              ortho_tol, kSeed, stream_of(h)),
           fn);
}
}  // namespace

void composite_FP32_auto_scale_deflate(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat,
                                       const int mat_size, const size_t k, const double tol, const double ortho_tol,
                                       const bool verbose) {
    (void)solverH;
    (void)verbose;
    deflate_any(PSDGB_PREC_FP16X3, cublasH, mat, mat_size, k, tol, ortho_tol, "composite_FP32_auto_scale_deflate");
}

void composite_FP32_emulated_auto_scale_deflate(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat,
                                                const int n, const size_t k, const double tol, const double ortho_tol,
                                                const bool verbose) {
    (void)solverH;
    (void)verbose;
    deflate_any(PSDGB_PREC_BF16X9, cublasH, mat, n, k, tol, ortho_tol, "composite_FP32_emulated_auto_scale_deflate");
}

double* eig_FP64_psd(cusolverDnHandle_t solverH, cublasHandle_t cublasH, double* mat, size_t mat_size,
                     bool return_eigenvalues) {
    (void)solverH;
    return eig_any(1, cublasH, mat, mat_size, return_eigenvalues, "eig_FP64_psd");
}

double* eig_FP32_psd(cusolverDnHandle_t solverH, cublasHandle_t cublasH, double* mat, size_t mat_size,
                     bool return_eigenvalues) {
    (void)solverH;
    return eig_any(0, cublasH, mat, mat_size, return_eigenvalues, "eig_FP32_psd");
}

void lobpcg(cublasHandle_t cublasH, cusolverDnHandle_t cusolverH, const double* A, double* V, double* D, const int n,
            const int m, const bool warmstart, const int maxiter, const double tol, const bool verbose) {
    (void)cusolverH;
    int iters = 0;
    report(psdgb_lobpcg(A, V, D, n, m, warmstart ? 1 : 0, maxiter, tol, 0, &iters, stream_of(cublasH)), "lobpcg");
    if (verbose) std::printf("LOBPCG: %d iterations\n", iters);
}

void eig_FP64_deflate(cusolverDnHandle_t solverH, cublasHandle_t cublasH, double* mat, size_t mat_size, const size_t k,
                      const int maxiter, const double tol, const bool verbose) {
    (void)solverH;
    (void)verbose;
    report(psdgb_eig_FP64_deflate(mat, static_cast<int64_t>(mat_size), static_cast<int64_t>(k), maxiter, tol, 0,
                                  stream_of(cublasH)),
           "eig_FP64_deflate");
}

void composite_FP16_auto_scale_deflate(cublasHandle_t cublasH, cusolverDnHandle_t solverH, double* mat,
                                       const int mat_size, float* float_workspace, __half* half_workspace,
                                       const size_t k, const int maxiter, const double tol, const bool verbose) {
    (void)solverH;
    (void)float_workspace;
    (void)half_workspace;
    (void)verbose;
    report(psdgb_composite_auto_scale_deflate_two_ends(PSDGB_PREC_FP16, PSDGB_SCHEDULE_FP16, mat, mat_size,
                                                       static_cast<int64_t>(k), maxiter, tol, 0, stream_of(cublasH)),
           "composite_FP16_auto_scale_deflate");
}
