// ref_replay.cu — TEST / BENCHMARK INFRASTRUCTURE ONLY (bench.py --impl
// reference).  Never linked into libpsdgb.so.
//
// The reference library is built with CMake from sources that do not travel
// to the GPU host, so its GPU methods are restated here as the sequence of
// cuBLAS / cuSOLVER calls and small kernels they issue, in the same order,
// with the same operand types and compute types, the same per-call
// cudaMalloc / cudaFree (or caller workspaces) and the same blocking
// synchronisations, on the legacy default stream:
//
//   approximate_two_norm   src/lanczos.cu:41-293  (Lanczos on A^T A: two Dgemv
//                          per step, Ddot / Dnrm2 read on the host, Dsyevd of
//                          the tridiagonal, the r = A y - theta y residual)
//   composite_FP32         src/composite_FP32.cu:15-164  (cublasSgemm chain)
//   composite_FP16         src/composite_FP16.cu:16-246  (cublasGemmEx FP16 ->
//                          FP32, CUBLAS_COMPUTE_32F_FAST_16F, FP32 master copies)
//   composite_FP32_emulated  src/composite_FP32_emulated.cu:20-235
//                          (cublasGemmEx, CUBLAS_COMPUTE_32F_EMULATED_16BFX9)
//   *_auto_scale           src/composite_FP32.cu:166-191 and twins: bound,
//                          Dscal(1/up), filter, Dscal(up)
//   symmetrizeFloat, add_identity, the conversions   src/utils.cu:7-131
//
// The coefficient table comes from the caller (the oracle's pinned copy), so
// this file holds no method data of its own.  The Lanczos start vector is a
// seeded host Gaussian (the reference seeds curand from the clock).
#include <cublas_v2.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

namespace {

struct Ctx {
    cublasHandle_t blas = nullptr;
    cusolverDnHandle_t solver = nullptr;
    int failed = 0;
};

Ctx& ctx() {
    static Ctx c;
    if (!c.blas) {
        if (cublasCreate(&c.blas) != CUBLAS_STATUS_SUCCESS) c.failed = 1;
        if (cusolverDnCreate(&c.solver) != CUSOLVER_STATUS_SUCCESS) c.failed = 1;
    }
    return c;
}

// Failures are counted (the reference prints and continues); the caller
// reads the count.
int g_errors = 0;
#define RC(x)                                                                              \
    do {                                                                                   \
        if ((x) != 0) {                                                                    \
            ++g_errors;                                                                    \
            std::fprintf(stderr, "ref_replay: %s failed at line %d\n", #x, __LINE__);      \
        }                                                                                  \
    } while (0)

__global__ void k_d2f(const double* in, float* out, int64_t count) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < count) out[i] = static_cast<float>(in[i]);
}
__global__ void k_f2d(const float* in, double* out, int64_t count) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < count) out[i] = static_cast<double>(in[i]);
}
// Four floats to four halves per thread (src/utils.cu:106-131).
__global__ void k_f2h4(const float4* in, __half2* out, int64_t count4) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= count4) return;
    const float4 v = in[i];
    out[2 * i] = __float22half2_rn(make_float2(v.x, v.y));
    out[2 * i + 1] = __float22half2_rn(make_float2(v.z, v.w));
}
__global__ void k_add_identity(float* m, int n) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < static_cast<int64_t>(n) * n && i / n == i % n) m[i] += 1.0f;
}

unsigned blocks(int64_t count, int threads) { return static_cast<unsigned>((count + threads - 1) / threads); }

// The reference's conversions end in cudaDeviceSynchronize (src/utils.cu:48-60).
void d2f(const double* in, float* out, int64_t count) {
    k_d2f<<<blocks(count, 1024), 1024>>>(in, out, count);
    RC(cudaDeviceSynchronize());
}
void f2d(const float* in, double* out, int64_t count) {
    k_f2d<<<blocks(count, 1024), 1024>>>(in, out, count);
    RC(cudaDeviceSynchronize());
}
void f2h4(const float* in, __half* out, int64_t count) {
    const int64_t c4 = (count + 3) / 4;
    k_f2h4<<<blocks(c4, 1024), 1024>>>(reinterpret_cast<const float4*>(in), reinterpret_cast<__half2*>(out), c4);
}

// M = (M + M^T) / 2 through a workspace: two Sgeam and an Sscal (src/utils.cu:7-32).
void symmetrize(cublasHandle_t h, float* m, int n, float* tmp) {
    const float one = 1.f, zero = 0.f, half = 0.5f;
    RC(cublasSgeam(h, CUBLAS_OP_T, CUBLAS_OP_N, n, n, &one, m, n, &zero, m, n, tmp, n));
    RC(cublasSgeam(h, CUBLAS_OP_N, CUBLAS_OP_N, n, n, &one, m, n, &one, tmp, n, m, n));
    RC(cublasSscal(h, n * n, &half, m, 1));
}

void lanczos_bound(const double* A, int64_t n64, int64_t max_iter, double tol, uint64_t seed, double* lo, double* up) {
    Ctx& c = ctx();
    const int n = static_cast<int>(n64);
    const int m = static_cast<int>(max_iter < n64 ? max_iter : n64);
    const double zero = 0.0, one = 1.0;
    double *V = nullptr, *Vold = nullptr, *q = nullptr, *w = nullptr, *w1 = nullptr;
    RC(cudaMalloc(&V, sizeof(double) * n * (m > 0 ? m : 1)));
    RC(cudaMalloc(&Vold, sizeof(double) * n));
    RC(cudaMalloc(&q, sizeof(double) * n));
    RC(cudaMalloc(&w, sizeof(double) * n));
    RC(cudaMalloc(&w1, sizeof(double) * n));
    std::vector<double> h(n);
    std::mt19937_64 gen(seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    for (auto& v : h) v = nd(gen);
    RC(cudaMemcpy(q, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    double nq = 0.0;
    RC(cublasDnrm2(c.blas, n, q, 1, &nq));
    if (nq != 0.0) {
        const double inv = 1.0 / nq;
        RC(cublasDscal(c.blas, n, &inv, q, 1));
    }
    RC(cublasDcopy(c.blas, n, q, 1, V, 1));
    RC(cudaMemset(Vold, 0, sizeof(double) * n));
    std::vector<double> alpha(m, 0.0), beta(m, 0.0);
    double minus_beta_old = 0.0;
    int nb = 0;
    for (int k = 0; k < m; ++k) {
        RC(cublasDgemv(c.blas, CUBLAS_OP_N, n, n, &one, A, n, q, 1, &zero, w, 1));
        RC(cublasDgemv(c.blas, CUBLAS_OP_T, n, n, &one, A, n, w, 1, &zero, w1, 1));
        RC(cublasDcopy(c.blas, n, w1, 1, w, 1));
        RC(cublasDdot(c.blas, n, q, 1, w, 1, &alpha[k]));
        const double minus_alpha = -alpha[k];
        RC(cublasDaxpy(c.blas, n, &minus_alpha, q, 1, w, 1));
        RC(cublasDaxpy(c.blas, n, &minus_beta_old, Vold, 1, w, 1));
        RC(cublasDnrm2(c.blas, n, w, 1, &beta[k]));
        if (beta[k] <= tol * alpha[k] && k > 1) break;
        RC(cublasDcopy(c.blas, n, q, 1, Vold, 1));
        RC(cudaMemcpy(q, w, sizeof(double) * n, cudaMemcpyDeviceToDevice));
        if (beta[k] == 0.0) break;
        const double binv = 1.0 / beta[k];
        RC(cublasDscal(c.blas, n, &binv, q, 1));
        if (k < m - 1) RC(cublasDcopy(c.blas, n, q, 1, V + static_cast<size_t>(k + 1) * n, 1));
        minus_beta_old = -beta[k];
        ++nb;
    }
    if (nb == 0) {
        *lo = 0.0;
        *up = 1.0;
    } else {
        // T = tridiag(beta, alpha, beta), its largest eigenpair by Dsyevd.
        std::vector<double> hT(static_cast<size_t>(nb) * nb, 0.0);
        for (int i = 0; i < nb; ++i) {
            hT[static_cast<size_t>(i) * nb + i] = alpha[i];
            if (i + 1 < nb) hT[static_cast<size_t>(i) * nb + i + 1] = hT[static_cast<size_t>(i + 1) * nb + i] = beta[i];
        }
        double *T = nullptr, *ev = nullptr, *work = nullptr, *uk = nullptr, *y = nullptr, *ry = nullptr;
        int *info = nullptr, lwork = 0;
        RC(cudaMalloc(&T, sizeof(double) * nb * nb));
        RC(cudaMalloc(&ev, sizeof(double) * nb));
        RC(cudaMemcpy(T, hT.data(), sizeof(double) * nb * nb, cudaMemcpyHostToDevice));
        RC(cusolverDnDsyevd_bufferSize(c.solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, nb, T, nb, ev,
                                       &lwork));
        RC(cudaMalloc(&work, sizeof(double) * (lwork > 0 ? lwork : 1)));
        RC(cudaMalloc(&info, sizeof(int)));
        RC(cusolverDnDsyevd(c.solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, nb, T, nb, ev, work, lwork,
                            info));
        RC(cudaDeviceSynchronize());
        double theta = 0.0;
        RC(cudaMemcpy(&theta, ev + nb - 1, sizeof(double), cudaMemcpyDeviceToHost));
        RC(cudaMalloc(&uk, sizeof(double) * nb));
        RC(cudaMalloc(&y, sizeof(double) * n));
        RC(cudaMalloc(&ry, sizeof(double) * n));
        RC(cublasDcopy(c.blas, nb, T + static_cast<size_t>(nb - 1) * nb, 1, uk, 1));
        RC(cublasDgemv(c.blas, CUBLAS_OP_N, n, nb, &one, V, n, uk, 1, &zero, y, 1));
        RC(cublasDgemv(c.blas, CUBLAS_OP_N, n, n, &one, A, n, y, 1, &zero, ry, 1));
        RC(cublasDgemv(c.blas, CUBLAS_OP_T, n, n, &one, A, n, ry, 1, &zero, w1, 1));
        RC(cublasDcopy(c.blas, n, ry, 1, w1, 1));  // leaves ry = A y (src/lanczos.cu:255)
        const double minus_theta = -theta;
        RC(cublasDaxpy(c.blas, n, &minus_theta, y, 1, ry, 1));
        double nr = 0.0;
        RC(cublasDnrm2(c.blas, n, ry, 1, &nr));
        *lo = std::sqrt(theta);
        *up = std::sqrt(theta + nr);
        cudaFree(T); cudaFree(ev); cudaFree(work); cudaFree(info); cudaFree(uk); cudaFree(y); cudaFree(ry);
    }
    cudaFree(V); cudaFree(Vold); cudaFree(q); cudaFree(w); cudaFree(w1);
    RC(cudaDeviceSynchronize());
}

enum Method { M_FP32 = 0, M_FP16 = 1, M_EMU = 2 };

// A <- coef * P * Q + beta * A in the method's arithmetic; P, Q in FP32 (the
// FP16 method converts them to the half buffers hp / hq first, as the
// reference does before each GemmEx).
void product(int method, int n, float alpha, const float* P, const float* Q, float beta, float* C) {
    Ctx& c = ctx();
    if (method == M_FP32) {
        RC(cublasSgemm(c.blas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &alpha, P, n, Q, n, &beta, C, n));
    } else {
        RC(cublasGemmEx(c.blas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &alpha, P, CUDA_R_32F, n, Q, CUDA_R_32F, n, &beta,
                        C, CUDA_R_32F, n, CUBLAS_COMPUTE_32F_EMULATED_16BFX9, CUBLAS_GEMM_DEFAULT_TENSOR_OP));
    }
}
void product_h(int n, float alpha, const __half* P, const __half* Q, float beta, float* C) {
    RC(cublasGemmEx(ctx().blas, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &alpha, P, CUDA_R_16F, n, Q, CUDA_R_16F, n, &beta, C,
                    CUDA_R_32F, n, CUBLAS_COMPUTE_32F_FAST_16F, CUBLAS_GEMM_DEFAULT_TENSOR_OP));
}

void composite(int method, double* mat, int n, const float* coef, int steps, float* fws, __half* hws) {
    Ctx& c = ctx();
    const int64_t nn = static_cast<int64_t>(n) * n;
    const int64_t stride = (nn + 3) / 4 * 4;
    float *A = nullptr, *A2 = nullptr, *A3 = nullptr;
    __half *hA = nullptr, *hA2 = nullptr, *hA3 = nullptr;
    if (fws) {
        A = fws; A2 = fws + (method == M_FP16 ? stride : nn); A3 = fws + 2 * (method == M_FP16 ? stride : nn);
    } else {
        RC(cudaMalloc(&A, sizeof(float) * nn));
        RC(cudaMalloc(&A2, sizeof(float) * nn));
        RC(cudaMalloc(&A3, sizeof(float) * nn));
    }
    if (method == M_FP16) {
        if (hws) {
            hA = hws; hA2 = hws + stride; hA3 = hws + 2 * stride;
        } else {
            RC(cudaMalloc(&hA, sizeof(__half) * nn));
            RC(cudaMalloc(&hA2, sizeof(__half) * nn));
            RC(cudaMalloc(&hA3, sizeof(__half) * nn));
        }
    }
    const float one = 1.f, zero = 0.f, half = 0.5f;
    d2f(mat, A, nn);
    for (int i = 0; i < steps; ++i) {
        float a = coef[3 * i], b = coef[3 * i + 1], cc = coef[3 * i + 2];
        if (method == M_FP16) {
            f2h4(A, hA, nn);
            product_h(n, one, hA, hA, zero, A2);
            f2h4(A2, hA2, nn);
            product_h(n, one, hA, hA2, zero, A3);
        } else {
            product(method, n, one, A, A, zero, A2);
            // A3 = A2 * A (src/composite_FP32.cu:108); the emulated method forms A * A2 (:119-131)
            if (method == M_EMU)
                product(method, n, one, A, A2, zero, A3);
            else
                product(method, n, one, A2, A, zero, A3);
        }
        RC(cublasSscal(c.blas, static_cast<int>(nn), &a, A, 1));
        RC(cublasSaxpy(c.blas, static_cast<int>(nn), &b, A3, 1, A, 1));
        if (method == M_FP16) {
            f2h4(A3, hA3, nn);
            product_h(n, cc, hA2, hA3, one, A);
        } else {
            product(method, n, cc, A3, A2, one, A);
        }
        symmetrize(c.blas, A, n, A2);
    }
    k_add_identity<<<blocks(nn, 1024), 1024>>>(A, n);
    RC(cudaGetLastError());
    RC(cublasSscal(c.blas, static_cast<int>(nn), &half, A, 1));
    d2f(mat, A2, nn);
    if (method == M_FP16) {
        f2h4(A, hA, nn);
        f2h4(A2, hA2, nn);
        product_h(n, one, hA2, hA, zero, A3);
    } else {
        product(method, n, one, A2, A, zero, A3);
    }
    symmetrize(c.blas, A3, n, A2);
    f2d(A3, mat, nn);
    if (!fws) {
        cudaFree(A); cudaFree(A2); cudaFree(A3);
    }
    if (method == M_FP16 && !hws) {
        cudaFree(hA); cudaFree(hA2); cudaFree(hA3);
    }
}

}  // namespace

extern "C" {

// Bytes of the FP32 and FP16 workspaces the reference documents for a method
// (3 n^2 floats; the FP16 method: 3 strides each of floats and halves, the
// stride being n^2 rounded up to a multiple of 4).
size_t ref_replay_ws_bytes(int method, int64_t n, int half) {
    const int64_t nn = n * n;
    const int64_t stride = (nn + 3) / 4 * 4;
    if (half) return method == M_FP16 ? static_cast<size_t>(3 * stride) * sizeof(__half) : 0;
    return static_cast<size_t>(3 * (method == M_FP16 ? stride : nn)) * sizeof(float);
}

// composite_*_auto_scale on the device FP64 matrix d_mat (n x n, column-major),
// in place.  fws / hws: caller workspaces (null: allocated and freed inside,
// as the reference does by default).  Returns the number of failed library
// calls (0 on success); *up_out receives the bound.
int ref_replay_auto_scale(int method, double* d_mat, int64_t n, const float* coef, int steps, uint64_t seed,
                          void* fws, void* hws, double* up_out) {
    Ctx& c = ctx();
    if (c.failed) return -1;
    g_errors = 0;
    const int64_t nn = n * n;
    double lo = 0.0, up = 1.0;
    lanczos_bound(d_mat, n, 20, 1e-10, seed, &lo, &up);
    const double scale = up > 0.0 ? up : 1.0, inv = 1.0 / scale;
    RC(cublasDscal(c.blas, static_cast<int>(nn), &inv, d_mat, 1));
    composite(method, d_mat, static_cast<int>(n), coef, steps, static_cast<float*>(fws), static_cast<__half*>(hws));
    RC(cublasDscal(c.blas, static_cast<int>(nn), &scale, d_mat, 1));
    RC(cudaDeviceSynchronize());
    if (up_out) *up_out = scale;
    return g_errors;
}

}  // extern "C"
