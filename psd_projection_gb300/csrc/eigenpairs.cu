// eigenpairs.cu — Lanczos eigenpairs (the reference's compute_eigenpairs,
// src/lanczos.cu:319-547) and the rank-r update of its deflation routines
// (the cublasDger loops of src/composite_FP32.cu:193-254,
// src/eig_FP64_psd.cu:87-177, src/composite_FP16.cu:276-380).
//
// GB300 design:
//   * the Lanczos recurrence on A runs on the device with no host round trip
//     per step: one FP64 matvec kernel (a warp per column, four independent
//     accumulators) and one single-block kernel for the recurrence, the dot
//     products, the norm and the stop test; a device flag skips the remaining
//     launches after a breakdown (beta <= machine epsilon, src/lanczos.cu:382);
//   * T's eigen-decomposition is cuSOLVER syevd, as in the reference;
//   * the ghost-orthogonality filter (src/lanczos.cu:451-497), which the
//     reference runs as one Gemv + one Gemv + host copy per candidate, forms a
//     chunk of candidate Ritz vectors with one GEMM (Q Z_c) and all their
//     overlaps with the accepted vectors and with each other with a second
//     GEMM (X^T X_c); the greedy accept/reject runs on the host on those dot
//     products, in the reference's candidate order;
//   * the rank-r update X += sum_i c_i v_i v_i^T is one pass over X (tiles of
//     32 x 32 elements, the vectors staged in shared memory) instead of r
//     cublasDger passes.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "internal.h"

namespace psdgb {

namespace {

struct EigState {
    int stopped;
    int nb_iter;
};

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ double block_sum_f64(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x / 32, l = threadIdx.x % 32, nw = blockDim.x / 32;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = (l < nw) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// Q[:, 0] = the seeded start vector (uniform (0, 1], the same stream as the
// bound's), normalised (src/lanczos.cu:339-353).
__global__ void eig_init_kernel(int64_t n, uint64_t seed, double* Q) {
    __shared__ double red[32];
    double ss = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint64_t h = mix64(seed ^ mix64(static_cast<uint64_t>(i)));
        const double u = static_cast<double>((h >> 11) + 1) * 0x1.0p-53;
        Q[i] = u;
        ss += u * u;
    }
    const double nrm = sqrt(block_sum_f64(ss, red));
    const double inv = nrm != 0.0 ? 1.0 / nrm : 1.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) Q[i] *= inv;
}

// y = A x for the symmetric FP64 matrix A (column-major, leading dimension
// n): y[c] = sum_r A[r + c n] x[r].  One warp per column.
__global__ void __launch_bounds__(256) eig_matvec_kernel(const double* __restrict__ A, int64_t n,
                                                         const double* __restrict__ x, double* __restrict__ y,
                                                         const EigState* st) {
    if (st->stopped) return;
    const int lane = threadIdx.x % 32;
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x / 32);
    for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x / 32) + threadIdx.x / 32; c < n; c += warps) {
        const double* col = A + c * n;
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int64_t r = lane;
        for (; r + 96 < n; r += 128) {
            s0 = fma(__ldg(col + r), __ldg(x + r), s0);
            s1 = fma(__ldg(col + r + 32), __ldg(x + r + 32), s1);
            s2 = fma(__ldg(col + r + 64), __ldg(x + r + 64), s2);
            s3 = fma(__ldg(col + r + 96), __ldg(x + r + 96), s3);
        }
        for (; r < n; r += 32) s0 = fma(__ldg(col + r), __ldg(x + r), s0);
        double s = (s0 + s1) + (s2 + s3);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) y[c] = s;
    }
}

// Step k of the recurrence (src/lanczos.cu:366-389), w = A Q[:, k] on entry:
//   w -= beta_{k-1} Q[:, k-1]; alpha_k = Q[:, k].w; w -= alpha_k Q[:, k];
//   beta_k = ||w||; stop when beta_k <= eps; Q[:, k+1] = w * (1 / beta_k).
__global__ void eig_update_kernel(int64_t n, int k, double* __restrict__ Q, double* __restrict__ w,
                                  double* __restrict__ alpha, double* __restrict__ beta, EigState* st) {
    if (st->stopped) return;
    __shared__ double red[32];
    const double* qk = Q + static_cast<int64_t>(k) * n;
    const double* qp = Q + static_cast<int64_t>(k > 0 ? k - 1 : 0) * n;
    const double bp = k > 0 ? beta[k - 1] : 0.0;
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        double v = w[i];
        if (k > 0) v -= bp * qp[i];
        w[i] = v;
        s += qk[i] * v;
    }
    const double a = block_sum_f64(s, red);
    s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = w[i] - a * qk[i];
        w[i] = v;
        s += v * v;
    }
    const double b = sqrt(block_sum_f64(s, red));
    if (threadIdx.x == 0) {
        alpha[k] = a;
        beta[k] = b;
        st->nb_iter = k + 1;
    }
    if (b <= DBL_EPSILON) {
        if (threadIdx.x == 0) st->stopped = 1;
        return;
    }
    const double inv = 1.0 / b;
    double* qn = Q + static_cast<int64_t>(k + 1) * n;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) qn[i] = w[i] * inv;
}

// T = tridiag(beta[0..m-2], alpha[0..m-1], beta[0..m-2]) (dense, column-major;
// T was zeroed), src/lanczos.cu:29-38.
__global__ void eig_fill_tridiag_kernel(double* T, const double* alpha, const double* beta, int m) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        T[static_cast<int64_t>(i) * m + i] = alpha[i];
        if (i + 1 < m) {
            T[static_cast<int64_t>(i) * m + i + 1] = beta[i];
            T[static_cast<int64_t>(i + 1) * m + i] = beta[i];
        }
    }
}

// X[p + q n] += sum_i coef[i] V[p + i n] V[q + i n] over a 32 x 32 tile per
// CTA (32 x 8 threads, four columns each); vectors staged 32 at a time.
__global__ void rank_update_kernel(double* __restrict__ X, int64_t n, const double* __restrict__ V,
                                   const double* __restrict__ coef, int r) {
    __shared__ double vp[32][33], vq[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t p0 = static_cast<int64_t>(blockIdx.x) * 32, q0 = static_cast<int64_t>(blockIdx.y) * 32;
    const int64_t p = p0 + tx;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int i0 = 0; i0 < r; i0 += 32) {
        for (int ii = ty; ii < 32; ii += 8) {
            const int i = i0 + ii;
            const bool ok = i < r;
            vp[ii][tx] = (ok && p < n) ? coef[i] * V[static_cast<int64_t>(i) * n + p] : 0.0;
            vq[ii][tx] = (ok && q0 + tx < n) ? V[static_cast<int64_t>(i) * n + q0 + tx] : 0.0;
        }
        __syncthreads();
        const int cnt = r - i0 < 32 ? r - i0 : 32;
        for (int ii = 0; ii < cnt; ++ii) {
            const double a = vp[ii][tx];
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[j] = fma(a, vq[ii][ty + 8 * j], acc[j]);
        }
        __syncthreads();
    }
    if (p >= n) return;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int64_t q = q0 + ty + 8 * j;
        if (q < n) X[p + q * n] += acc[j];
    }
}

// Device buffers of one call, freed on every return path.
struct Scratch {
    std::vector<void*> ptrs;
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <typename T>
    psdgb_status get(T** out, size_t count) {
        void* p = nullptr;
        const cudaError_t e = cudaMalloc(&p, sizeof(T) * (count > 0 ? count : 1));
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error("eigenpairs: device allocation failed");
            return PSDGB_ERR_OUT_OF_MEMORY;
        }
        ptrs.push_back(p);
        *out = static_cast<T*>(p);
        return PSDGB_OK;
    }
};

constexpr int kChunk = 32;  // candidate Ritz vectors formed per GEMM

}  // namespace

cudaError_t launch_rank_update(double* X, int64_t n, const double* V, const double* d_coef, int r, cudaStream_t s) {
    if (r <= 0 || n <= 0) return cudaSuccess;
    const dim3 grid(static_cast<unsigned>((n + 31) / 32), static_cast<unsigned>((n + 31) / 32));
    rank_update_kernel<<<grid, dim3(32, 8), 0, s>>>(X, n, V, d_coef, r);
    count_launch();
    return cudaGetLastError();
}

psdgb_status eigenpairs_run(DeviceState* ds, cublasHandle_t blas, cusolverDnHandle_t solver, const double* A,
                            int64_t n, int64_t k, bool upper_only, int64_t max_iter, double ortho_tol, uint64_t seed,
                            int64_t* r_out, double* d_vals, double* d_vecs, double* upper_out, cudaStream_t s) {
    if (n <= 0) {
        set_error("compute_eigenpairs: n must be > 0");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (max_iter <= 0) max_iter = n;  // src/lanczos.cu:330-331
    if (max_iter > (int64_t{1} << 30) / (n + 1) || max_iter > 1000000) {
        set_error("compute_eigenpairs: max_iter too large for the Lanczos basis");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (cublasSetStream(blas, s) != CUBLAS_STATUS_SUCCESS || cusolverDnSetStream(solver, s) != CUSOLVER_STATUS_SUCCESS) {
        set_error("compute_eigenpairs: cuBLAS/cuSOLVER set stream failed");
        return PSDGB_ERR_SOLVER;
    }
    Scratch sc;
    double *Q, *w, *alpha, *beta;
    EigState* st;
    PSDGB_TRY(sc.get(&Q, static_cast<size_t>(n) * (max_iter + 1)));
    PSDGB_TRY(sc.get(&w, n));
    PSDGB_TRY(sc.get(&alpha, max_iter));
    PSDGB_TRY(sc.get(&beta, max_iter));
    PSDGB_TRY(sc.get(&st, 1));
    PSDGB_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(EigState), s));
    PSDGB_CUDA_TRY(cudaMemsetAsync(alpha, 0, sizeof(double) * max_iter, s));
    PSDGB_CUDA_TRY(cudaMemsetAsync(beta, 0, sizeof(double) * max_iter, s));
    eig_init_kernel<<<1, 1024, 0, s>>>(n, seed, Q);
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    int64_t mv_blocks = (n + 7) / 8;
    if (mv_blocks > static_cast<int64_t>(ds->sm_count) * 8) mv_blocks = static_cast<int64_t>(ds->sm_count) * 8;
    for (int64_t kk = 0; kk < max_iter; ++kk) {
        eig_matvec_kernel<<<static_cast<unsigned>(mv_blocks), 256, 0, s>>>(A, n, Q + kk * n, w, st);
        eig_update_kernel<<<1, 1024, 0, s>>>(n, static_cast<int>(kk), Q, w, alpha, beta, st);
        count_launch(2);
    }
    PSDGB_CUDA_TRY(cudaGetLastError());
    EigState hst{};
    PSDGB_CUDA_TRY(cudaMemcpyAsync(&hst, st, sizeof(EigState), cudaMemcpyDeviceToHost, s));
    PSDGB_CUDA_TRY(cudaStreamSynchronize(s));
    const int m = hst.nb_iter;
    if (m <= 0) {
        set_error("compute_eigenpairs: no Lanczos step completed");
        return PSDGB_ERR_CUDA;
    }
    std::vector<double> hbeta(m);
    PSDGB_CUDA_TRY(cudaMemcpy(hbeta.data(), beta, sizeof(double) * m, cudaMemcpyDeviceToHost));

    // T and its eigen-decomposition (ascending; eigenvectors Z in T).
    double *T, *theta, *work;
    int* info;
    PSDGB_TRY(sc.get(&T, static_cast<size_t>(m) * m));
    PSDGB_TRY(sc.get(&theta, m));
    PSDGB_TRY(sc.get(&info, 1));
    PSDGB_CUDA_TRY(cudaMemsetAsync(T, 0, sizeof(double) * m * m, s));
    eig_fill_tridiag_kernel<<<(m + 255) / 256, 256, 0, s>>>(T, alpha, beta, m);
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    int lwork = 0;
    if (cusolverDnDsyevd_bufferSize(solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, m, T, m, theta,
                                    &lwork) != CUSOLVER_STATUS_SUCCESS) {
        set_error("compute_eigenpairs: syevd buffer query failed");
        return PSDGB_ERR_SOLVER;
    }
    PSDGB_TRY(sc.get(&work, lwork));
    if (cusolverDnDsyevd(solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, m, T, m, theta, work, lwork,
                         info) != CUSOLVER_STATUS_SUCCESS) {
        set_error("compute_eigenpairs: syevd failed");
        return PSDGB_ERR_SOLVER;
    }
    std::vector<double> htheta(m), zrow(m);
    int hinfo = 0;
    PSDGB_CUDA_TRY(cudaMemcpyAsync(htheta.data(), theta, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
    PSDGB_CUDA_TRY(cudaMemcpy2DAsync(zrow.data(), sizeof(double), T, sizeof(double) * m, sizeof(double), m,
                                     cudaMemcpyDeviceToHost, s));
    PSDGB_CUDA_TRY(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, s));
    PSDGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (hinfo != 0) {
        set_error("compute_eigenpairs: syevd reported info = " + std::to_string(hinfo));
        return PSDGB_ERR_SOLVER;
    }
    // Residuals |beta_m Z[0, j]| (the reference reads Z's first row,
    // src/lanczos.cu:295-300) and the order of decreasing |theta| (:436-438).
    const double beta_m = hbeta[m - 1];
    std::vector<double> res(m);
    for (int j = 0; j < m; ++j) res[j] = std::fabs(beta_m * zrow[j]);
    std::vector<int> idx(m);
    for (int j = 0; j < m; ++j) idx[j] = j;
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int a, int b) { return std::fabs(htheta[a]) > std::fabs(htheta[b]); });

    if (!upper_only) {
        std::vector<int> cand;  // residual filter, in the reference's order (:451-454)
        for (int j : idx)
            if (res[j] < ortho_tol) cand.push_back(j);
        std::vector<double> sel_vals;
        int64_t r = 0;
        if (k > 0 && !cand.empty()) {
            const int64_t cap = std::min<int64_t>(k, static_cast<int64_t>(cand.size()));
            double *X, *Zc, *G;
            PSDGB_TRY(sc.get(&X, static_cast<size_t>(n) * (cap + kChunk)));
            PSDGB_TRY(sc.get(&Zc, static_cast<size_t>(m) * kChunk));
            PSDGB_TRY(sc.get(&G, static_cast<size_t>(cap + kChunk) * kChunk));
            std::vector<double> hG;
            const double one = 1.0, zero = 0.0;
            for (size_t c0 = 0; c0 < cand.size() && r < k; c0 += kChunk) {
                const int c = static_cast<int>(std::min<size_t>(kChunk, cand.size() - c0));
                for (int t = 0; t < c; ++t)
                    PSDGB_CUDA_TRY(cudaMemcpyAsync(Zc + static_cast<int64_t>(t) * m,
                                                   T + static_cast<int64_t>(cand[c0 + t]) * m, sizeof(double) * m,
                                                   cudaMemcpyDeviceToDevice, s));
                // X[:, r .. r + c) = Q[:, 0 .. m) Zc   (x_candidate, :457-459)
                if (cublasDgemm(blas, CUBLAS_OP_N, CUBLAS_OP_N, static_cast<int>(n), c, m, &one, Q,
                                static_cast<int>(n), Zc, m, &zero, X + r * n, static_cast<int>(n)) !=
                    CUBLAS_STATUS_SUCCESS) {
                    set_error("compute_eigenpairs: Ritz vector GEMM failed");
                    return PSDGB_ERR_SOLVER;
                }
                // G = X[:, 0 .. r + c)^T X[:, r .. r + c)   (overlaps, :462-466)
                const int rows = static_cast<int>(r) + c;
                if (cublasDgemm(blas, CUBLAS_OP_T, CUBLAS_OP_N, rows, c, static_cast<int>(n), &one, X,
                                static_cast<int>(n), X + r * n, static_cast<int>(n), &zero, G, rows) !=
                    CUBLAS_STATUS_SUCCESS) {
                    set_error("compute_eigenpairs: overlap GEMM failed");
                    return PSDGB_ERR_SOLVER;
                }
                hG.resize(static_cast<size_t>(rows) * c);
                PSDGB_CUDA_TRY(cudaMemcpyAsync(hG.data(), G, sizeof(double) * rows * c, cudaMemcpyDeviceToHost, s));
                PSDGB_CUDA_TRY(cudaStreamSynchronize(s));
                // Greedy acceptance against the accepted vectors (:460-495).
                std::vector<int> accepted_rows;  // rows of G (columns of X) accepted so far
                for (int64_t i = 0; i < r; ++i) accepted_rows.push_back(static_cast<int>(i));
                std::vector<int> take;
                for (int t = 0; t < c && static_cast<int64_t>(sel_vals.size()) < k; ++t) {
                    bool accept = true;
                    if (!sel_vals.empty()) {
                        for (int row : accepted_rows)
                            if (std::fabs(hG[static_cast<size_t>(t) * rows + row]) > ortho_tol) {
                                accept = false;
                                break;
                            }
                    }
                    if (accept) {
                        accepted_rows.push_back(static_cast<int>(r) + t);
                        take.push_back(t);
                        sel_vals.push_back(htheta[cand[c0 + t]]);
                    }
                }
                // Compact the accepted candidates to columns r, r + 1, ...
                int64_t dst = r;
                for (int t : take) {
                    const int64_t src = r + t;
                    if (src != dst)
                        PSDGB_CUDA_TRY(cudaMemcpyAsync(X + dst * n, X + src * n, sizeof(double) * n,
                                                       cudaMemcpyDeviceToDevice, s));
                    ++dst;
                }
                r = dst;
            }
            if (r > 0) {
                if (d_vecs)
                    PSDGB_CUDA_TRY(cudaMemcpyAsync(d_vecs, X, sizeof(double) * n * r, cudaMemcpyDeviceToDevice, s));
                if (d_vals)
                    PSDGB_CUDA_TRY(cudaMemcpyAsync(d_vals, sel_vals.data(), sizeof(double) * r,
                                                   cudaMemcpyHostToDevice, s));
            }
            PSDGB_CUDA_TRY(cudaStreamSynchronize(s));
        }
        if (r_out) *r_out = r;
    }
    const int i0 = idx[0];
    if (upper_out) *upper_out = std::fabs(htheta[i0]) + res[i0] + 1e-3;  // :509-517, :546
    return PSDGB_OK;
}

}  // namespace psdgb
