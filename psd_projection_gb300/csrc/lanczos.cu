// lanczos.cu — spectral-norm bound by Lanczos on A^T A (approximate_two_norm).
//
// Follows src/lanczos.cu:41-293 of the reference step for step:
//   * start vector uniform in (0, 1], normalised (:69,:101-107);
//   * three-term recurrence without reorthogonalisation (:116-169):
//       w = A^T A q; alpha_k = q.w; w -= alpha_k q + beta_{k-1} q_old;
//       beta_k = ||w||; stop if beta_k <= tol*alpha_k and k > 1, or beta_k == 0;
//   * theta = largest eigenvalue of the tridiagonal T (:186-231), Ritz vector
//     y = V u (:236-242), residual r, lo = sqrt(theta), up = sqrt(theta + ||r||)
//     (:244-270).  The reference's residual is r = A y - theta y (its copy at
//     :255 runs ry -> w1, leaving ry = A y); PSDGB_RESIDUAL_EXACT uses
//     r = A^T A y - theta y instead.
//
// GB300 design: the matrix is streamed as FP32, FP64 for every vector and
// every cross-tile sum.  From n = 2048 up each matvec reads only the lower
// block triangle of the symmetric matrix (2 n^2 bytes instead of the
// reference's 8 n^2 per Dgemv, two per step): 128 x 128 tiles arrive by TMA
// in a three-stage mbarrier pipeline, and each off-diagonal tile A_ij yields
// both A_ij x_j (row sums, for y_i) and A_ij^T x_i (column sums, for y_j).
// The nb per-tile partial sums of a 128-row block are stored in FP64 and
// added in a fixed order by a second small kernel, so the result does not
// depend on scheduling.  Below n = 2048 a warp per column streams the
// whole matrix with 128-bit loads.  The whole bound runs on the device: the
// recurrence, the largest eigenpair of T (Sturm-sequence multisection in one
// warp and inverse iteration, instead of the reference's cuSOLVER Dsyevd
// with host round trips), the Ritz residual, and the scale 1/up the filter
// consumes — so a projection needs no host synchronisation and can be
// captured in a CUDA graph.  The start vector comes from a counter-based hash
// (SplitMix64) of a caller seed instead of the reference's nondeterministic
// curand seed (src/utils.cu:188-214), or from a caller-supplied warm start.
#include <cmath>
#include <vector>

#include "internal.h"
#include "tridiag.cuh"

namespace psdgb {

namespace {

struct LzState {
    int nb_iter;
    int stopped;    // the recurrence stopped (skip the remaining steps)
    int no_ritz;    // nb_iter == 0: skip the Ritz residual
    int pad;
    double beta_old;
    double resid_norm2;  // sum of squares of the Ritz residual
    double theta, lo, up;
    double scale, inv_scale;  // scale = up > 0 ? up : 1 (src/composite_FP32.cu:182)
};

// Layout of the Lanczos state inside its buffer.
struct LzLayout {
    size_t state, alpha, beta, q, w, vold, V, y, ry, q32, u32, uk, work, part, qdot, norm;
    size_t total;
};

inline size_t align256(size_t x) { return (x + 255) / 256 * 256; }

LzLayout lz_layout(int64_t n, int64_t m) {
    LzLayout L{};
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align256(off + bytes); return o; };
    const size_t n4 = static_cast<size_t>((n + 3) / 4 * 4);
    L.state = take(sizeof(LzState));
    L.alpha = take(sizeof(double) * (m + 1));
    L.beta = take(sizeof(double) * (m + 1));
    L.q = take(sizeof(double) * n);
    L.w = take(sizeof(double) * n);
    L.vold = take(sizeof(double) * n);
    L.V = take(sizeof(double) * n * (m > 0 ? m : 1));
    L.y = take(sizeof(double) * n);
    L.ry = take(sizeof(double) * n);
    L.q32 = take(sizeof(float) * n4);
    L.u32 = take(sizeof(float) * n4);
    L.uk = take(sizeof(double) * (m + 1));
    L.work = take(sizeof(double) * 8 * (m + 1));  // tridiagonal solver: LU (5 (m+1)) and staged T (3 (m+1))
    const size_t nb = static_cast<size_t>((n + 127) / 128);
    L.part = take(sizeof(double) * nb * nb * 128);  // tile matvec: partial sums [row block][source block][128]
    L.qdot = take(sizeof(double) * static_cast<size_t>((n + 31) / 32));   // q.w partials (reduce blocks)
    L.norm = take(sizeof(double) * static_cast<size_t>((n + 511) / 512)); // ||w||^2 partials
    L.total = off;
    return L;
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Block-wide FP64 sum (blockDim.x a multiple of 32, <= 1024).  All threads
// get the result.
__device__ double block_sum(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x / 32, l = threadIdx.x % 32, nw = blockDim.x / 32;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = (l < nw) ? red[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// q = start vector (uniform(0,1] from the seed, or the warm start), normalised;
// V[:,0] = q; q_old = 0.
__global__ void lz_init_kernel(int64_t n, uint64_t seed, const double* __restrict__ warm, LzState* st, double* q,
                               double* vold, double* V, float* q32) {
    __shared__ double red[32];
    double ss = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        double u;
        if (warm != nullptr) {
            u = warm[i];
        } else {
            const uint64_t h = splitmix64(seed ^ splitmix64(static_cast<uint64_t>(i)));
            u = static_cast<double>((h >> 11) + 1) * 0x1.0p-53;  // (0, 1]
        }
        q[i] = u;
        ss += u * u;
    }
    const double nrm = sqrt(block_sum(ss, red));
    const double inv = nrm != 0.0 ? 1.0 / nrm : 1.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = q[i] * inv;
        q[i] = v;
        V[i] = v;
        vold[i] = 0.0;
        q32[i] = static_cast<float>(v);
    }
    if (threadIdx.x == 0) {
        st->nb_iter = 0;
        st->stopped = 0;
        st->no_ritz = 0;
        st->beta_old = 0.0;
        st->resid_norm2 = 0.0;
        st->theta = 0.0;
        st->lo = 0.0;
        st->up = 1.0;
        st->scale = 1.0;
        st->inv_scale = 1.0;
    }
}

// y[c] = sum_r A[c*ld + r] * x[r] for every column c of the symmetric FP32
// matrix A (so y = A x = A^T x).  One or two adjacent columns per warp,
// float4 loads, FP32 partial sums per lane flushed to FP64 every 64 vectors,
// FP64 across lanes.
// x is staged in shared memory.  Writes y as FP64 (y64) and/or FP32 (y32).
// The whole kernel is skipped when *skip is non-zero.
__global__ void __launch_bounds__(256) lz_matvec_kernel(const float* __restrict__ A, int64_t n, int64_t ld,
                                                        const float* __restrict__ x, double* __restrict__ y64,
                                                        float* __restrict__ y32, const int* skip, int pair) {
    if (skip != nullptr && *skip) return;
    extern __shared__ float4 xs4[];
    float* xs = reinterpret_cast<float*>(xs4);
    const int64_t ld4 = ld / 4;
    for (int64_t i = threadIdx.x; i < ld; i += blockDim.x) xs[i] = (i < n) ? x[i] : 0.0f;
    __syncthreads();
    const int lane = threadIdx.x % 32;
    const int64_t warps_total = static_cast<int64_t>(gridDim.x) * (blockDim.x / 32);
    const int64_t units = pair ? (n + 1) / 2 : n;
    // With `pair` each warp streams two adjacent columns with interleaved
    // loads (twice the loads in flight per lane, for matrices with more
    // columns than resident warps); a column's own arithmetic is the same
    // either way.
    for (int64_t u = blockIdx.x * static_cast<int64_t>(blockDim.x / 32) + threadIdx.x / 32; u < units;
         u += warps_total) {
        const int64_t c0 = pair ? 2 * u : u;
        const bool has1 = pair && c0 + 1 < n;
        const float4* col0 = reinterpret_cast<const float4*>(A + c0 * ld);
        const float4* col1 = has1 ? col0 + ld4 : col0;
        float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, t0 = 0.f, t1 = 0.f, t2 = 0.f, t3 = 0.f;
        double acc0 = 0.0, acc1 = 0.0;
        int64_t k = lane;
        while (k < ld4) {
            const int64_t kend = (k + 32 * 64 < ld4) ? k + 32 * 64 : ld4;
#pragma unroll 8
            for (; k < kend; k += 32) {
                const float4 a = __ldg(col0 + k);
                const float4 c = __ldg(col1 + k);
                const float4 b = xs4[k];
                s0 = fmaf(a.x, b.x, s0);
                s1 = fmaf(a.y, b.y, s1);
                s2 = fmaf(a.z, b.z, s2);
                s3 = fmaf(a.w, b.w, s3);
                t0 = fmaf(c.x, b.x, t0);
                t1 = fmaf(c.y, b.y, t1);
                t2 = fmaf(c.z, b.z, t2);
                t3 = fmaf(c.w, b.w, t3);
            }
            acc0 += static_cast<double>(s0) + static_cast<double>(s1) + static_cast<double>(s2) +
                    static_cast<double>(s3);
            acc1 += static_cast<double>(t0) + static_cast<double>(t1) + static_cast<double>(t2) +
                    static_cast<double>(t3);
            s0 = s1 = s2 = s3 = 0.f;
            t0 = t1 = t2 = t3 = 0.f;
        }
        for (int o = 16; o > 0; o >>= 1) {
            acc0 += __shfl_xor_sync(0xffffffffu, acc0, o);
            acc1 += __shfl_xor_sync(0xffffffffu, acc1, o);
        }
        if (lane == 0) {
            if (y64) y64[c0] = acc0;
            if (y32) y32[c0] = static_cast<float>(acc0);
            if (has1) {
                if (y64) y64[c0 + 1] = acc1;
                if (y32) y32[c0 + 1] = static_cast<float>(acc1);
            }
        }
    }
}

// ---- matvec over the lower block triangle (n >= 2048) -----------------------
constexpr int SV_T = 128;                 // tile edge
constexpr int SV_STAGES = 3;              // TMA pipeline depth (64 KB a stage)
constexpr int SV_CWARPS_MAX = 16;
constexpr uint32_t SV_TILE_BYTES = SV_T * SV_T * sizeof(float);
constexpr size_t SV_SMEM = 128 + SV_STAGES * static_cast<size_t>(SV_TILE_BYTES) +
                           2 * SV_CWARPS_MAX * SV_T * sizeof(float) +  // column sums of the warps, two buffers
                           2 * SV_STAGES * sizeof(uint64_t) + 16;

// Barrier of the nthreads consumer threads that also ORs a predicate over
// them (every thread gets the same answer).
__device__ __forceinline__ bool consumer_sync_or(bool v, int nthreads) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(static_cast<uint32_t>(v)), "r"(nthreads)
        : "memory");
    return r != 0;
}

// Tile t of the lower block triangle in row-major order: row block bi holds
// tiles (bi, 0..bi).
__device__ __forceinline__ void sv_decode(int64_t t, int& bi, int& bj) {
    // FP32 square root for the estimate (FP64 issues slowly on this GPU); the
    // integer corrections below make it exact.
    int r = static_cast<int>((sqrtf(8.0f * static_cast<float>(t) + 1.0f) - 1.0f) * 0.5f);
    while (static_cast<int64_t>(r) * (r + 1) / 2 > t) --r;
    while (static_cast<int64_t>(r + 1) * (r + 2) / 2 <= t) ++r;
    bi = r;
    bj = static_cast<int>(t - static_cast<int64_t>(r) * (r + 1) / 2);
}

// Partial sums of y = A x for the symmetric FP32 matrix A (n x n, row stride
// ld) from its lower block triangle: part[(b * nb + s) * 128 + r] receives
// row r of row block b summed over column block s (each entry written once;
// lz_symv_reduce_kernel adds them up).  CW consumer warps (8 or 16) and one
// TMA warp; consumer warp w handles tile rows ROWS w .. ROWS w + ROWS - 1,
// lane l columns 4l..4l+3; the x segments of the next tile are loaded while
// the current one is consumed, and each tile costs its consumers one barrier.
// With `reverse` the tiles are visited last to first: consecutive matvecs
// alternate, so each starts on the tiles the previous one left in L2.
template <int CW>
__global__ void __launch_bounds__(32 * (CW + 1), 1)
    lz_symv_kernel(const __grid_constant__ CUtensorMap tmap, int64_t n, int nb, const float* __restrict__ x,
                   double* __restrict__ part, const int* skip, int* err, int reverse) {
    constexpr int SV_CWARPS = CW;
    constexpr int SV_ROWS = SV_T / CW;      // tile rows per consumer warp
    constexpr int SV_G = 32 / SV_ROWS;      // lanes that share a row after the halving steps
    static_assert(CW == 8 || CW == 16, "8 or 16 consumer warps");
    if (skip != nullptr && *skip) return;
    extern __shared__ uint8_t sv_raw[];
    uint8_t* smem = sv_raw + ((128u - (smem_u32(sv_raw) & 127u)) & 127u);
    float* stage = reinterpret_cast<float*>(smem);
    float* red = stage + SV_STAGES * SV_T * SV_T;
    uint64_t* full = reinterpret_cast<uint64_t*>(red + 2 * SV_CWARPS * SV_T);
    uint64_t* empty = full + SV_STAGES;
    volatile int* abort_flag = reinterpret_cast<volatile int*>(empty + SV_STAGES);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int64_t ntiles = static_cast<int64_t>(nb) * (nb + 1) / 2;
    if (threadIdx.x == 0) {
        for (int s = 0; s < SV_STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], SV_CWARPS);
        }
        *abort_flag = 0;
        fence_mbar_init();
    }
    __syncthreads();

    int issued = 0;
    if (warp == SV_CWARPS) {
        // ---- TMA producer ----
        if (lane == 0) {
            tma_prefetch_desc(&tmap);
            int k = 0;
            for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
                const int s = k % SV_STAGES;
                const uint32_t ph = static_cast<uint32_t>(k / SV_STAGES) & 1u;
                if (!mbar_wait_bounded(&empty[s], ph ^ 1u)) {
                    *abort_flag = 1;
                    atomicCAS(err, 0, DEVERR_SYMV_WAIT);
                    break;
                }
                if (*abort_flag) break;
                int bi, bj;
                sv_decode(reverse ? ntiles - 1 - t : t, bi, bj);
                mbar_arrive_expect_tx(&full[s], SV_TILE_BYTES);
                tma_load_2d(stage + s * SV_T * SV_T, &tmap, &full[s], bj * SV_T, bi * SV_T);
                issued = k + 1;
            }
        }
    } else {
        // ---- consumers ----
        const int tid = threadIdx.x;  // 0..32 CW - 1
        // x_j for this lane's four columns and x_i for the warp's 8 rows of a
        // tile (x_i: the same address in every lane, a broadcast load).
        auto load_x = [&](int64_t t, float (&xj)[4], float (&xi)[SV_ROWS]) {
            int bi, bj;
            sv_decode(reverse ? ntiles - 1 - t : t, bi, bj);
            const int64_t c0 = static_cast<int64_t>(bj) * SV_T + 4 * lane;
            const int64_t r0 = static_cast<int64_t>(bi) * SV_T + SV_ROWS * warp;
#pragma unroll
            for (int e = 0; e < 4; ++e) xj[e] = c0 + e < n ? __ldg(x + c0 + e) : 0.0f;
#pragma unroll
            for (int e = 0; e < SV_ROWS; ++e) xi[e] = r0 + e < n ? __ldg(x + r0 + e) : 0.0f;
        };
        float xj[4], xi[SV_ROWS], xj_n[4], xi_n[SV_ROWS];
        if (blockIdx.x < ntiles) load_x(blockIdx.x, xj, xi);
        int k = 0;
        for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) {
            const int s = k % SV_STAGES;
            const uint32_t ph = static_cast<uint32_t>(k / SV_STAGES) & 1u;
            int bi, bj;
            sv_decode(reverse ? ntiles - 1 - t : t, bi, bj);
            if (t + gridDim.x < ntiles) load_x(t + gridDim.x, xj_n, xi_n);
            const bool ok = mbar_wait_bounded(&full[s], ph);
            if (!ok && lane == 0) {
                *abort_flag = 1;
                atomicCAS(err, 0, DEVERR_SYMV_WAIT);
            }
            const float* tile = stage + s * SV_T * SV_T;
            float cs0 = 0.f, cs1 = 0.f, cs2 = 0.f, cs3 = 0.f;
            float rp[SV_ROWS];
#pragma unroll
            for (int rr = 0; rr < SV_ROWS; ++rr) {
                const float4 a = reinterpret_cast<const float4*>(tile + (SV_ROWS * warp + rr) * SV_T)[lane];
                cs0 = fmaf(a.x, xi[rr], cs0);
                cs1 = fmaf(a.y, xi[rr], cs1);
                cs2 = fmaf(a.z, xi[rr], cs2);
                cs3 = fmaf(a.w, xi[rr], cs3);
                rp[rr] = fmaf(a.x, xj[0], fmaf(a.y, xj[1], fmaf(a.z, xj[2], a.w * xj[3])));
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[s]);  // this warp is done with the stage
            // Row sums across the 32 lanes by recursive halving (ROWS
            // shuffles): afterwards lanes G r .. G r + G - 1 hold the sum of
            // the warp's row r.
#pragma unroll
            for (int h = SV_ROWS / 2; h >= 1; h >>= 1) {
                const int off = SV_G * h;  // 16, 8, 4 (, 2)
                const bool upper = (lane & off) != 0;
#pragma unroll
                for (int q = 0; q < h; ++q) {
                    const float send = upper ? rp[q] : rp[q + h];
                    const float keep = upper ? rp[q + h] : rp[q];
                    rp[q] = keep + __shfl_xor_sync(0xffffffffu, send, off);
                }
            }
#pragma unroll
            for (int off = SV_G / 2; off >= 1; off >>= 1) rp[0] += __shfl_xor_sync(0xffffffffu, rp[0], off);
            if ((lane & (SV_G - 1)) == 0)
                part[(static_cast<int64_t>(bi) * nb + bj) * SV_T + SV_ROWS * warp + lane / SV_G] =
                    static_cast<double>(rp[0]);
            // Column sums: the warps' partials through shared memory (two
            // buffers, so one barrier a tile keeps writers and readers apart).
            float* rb = red + (k & 1) * SV_CWARPS * SV_T;
            if (bi != bj) reinterpret_cast<float4*>(rb + warp * SV_T)[lane] = make_float4(cs0, cs1, cs2, cs3);
            if (consumer_sync_or(!ok, 32 * SV_CWARPS)) break;
            if (bi != bj && tid < SV_T) {
                float c = 0.f;
#pragma unroll
                for (int w = 0; w < SV_CWARPS; ++w) c += rb[w * SV_T + tid];
                part[(static_cast<int64_t>(bj) * nb + bi) * SV_T + tid] = static_cast<double>(c);
            }
#pragma unroll
            for (int e = 0; e < 4; ++e) xj[e] = xj_n[e];
#pragma unroll
            for (int e = 0; e < SV_ROWS; ++e) xi[e] = xi_n[e];
        }
    }

    // ---- teardown: after an abort, let the copies in flight land ----
    __syncthreads();
    if (*abort_flag && warp == SV_CWARPS && lane == 0) {
        for (int g = issued - SV_STAGES; g < issued; ++g) {
            if (g < 0) continue;
            if (!mbar_wait_bounded(&full[g % SV_STAGES], static_cast<uint32_t>(g / SV_STAGES) & 1u))
                atomicCAS(err, 0, DEVERR_DRAIN_WAIT);
        }
    }
}

// y[row] = sum over s = 0..nb-1 of part[(b * nb + s) * 128 + r], row = 128 b + r,
// in a fixed order: a block of 128 threads covers 32 rows; warp q sums the
// q-th quarter of the sources for its lane's row, then the quarters are added.
// With qd set, qdot_part[block] = sum over the block's rows of qd[row] y[row]
// (a fixed shuffle tree): the partials of the Lanczos alpha = q.w.
__global__ void __launch_bounds__(128) lz_symv_reduce_kernel(const double* __restrict__ part, int nb, int64_t n,
                                                            double* __restrict__ y64, float* __restrict__ y32,
                                                            const int* skip, const double* __restrict__ qd,
                                                            double* __restrict__ qdot_part) {
    if (skip != nullptr && *skip) return;
    __shared__ double qs[4][32];
    const int lane = threadIdx.x % 32, q = threadIdx.x / 32;
    const int64_t row = static_cast<int64_t>(blockIdx.x) * 32 + lane;
    const int64_t b = row / SV_T, r = row % SV_T;
    const int per = (nb + 3) / 4;
    const int sb = q * per, se = (sb + per < nb) ? sb + per : nb;
    double acc = 0.0;
    if (row < n) {
        const double* p = part + b * nb * SV_T + r;
        int s = sb;
        for (; s + 8 <= se; s += 8) {
            double v[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) v[e] = p[static_cast<int64_t>(s + e) * SV_T];
#pragma unroll
            for (int e = 0; e < 8; ++e) acc += v[e];
        }
        for (; s < se; ++s) acc += p[static_cast<int64_t>(s) * SV_T];
    }
    qs[q][lane] = acc;
    __syncthreads();
    if (q == 0) {
        const double v = ((qs[0][lane] + qs[1][lane]) + qs[2][lane]) + qs[3][lane];
        if (row < n) {
            if (y64) y64[row] = v;
            if (y32) y32[row] = static_cast<float>(v);
        }
        if (qd != nullptr) {
            double p = row < n ? qd[row] * v : 0.0;
            for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
            if (lane == 0) qdot_part[blockIdx.x] = p;
        }
    }
}

// ---- the Lanczos update spread over the GPU (with the tile matvec) ----------
// FP64 issues slowly on this GPU, so the update's vector arithmetic runs in
// UPB_BLOCKS-wide grids rather than one block.  Every block sums the same
// partials in the same order, so alpha, beta and the stop test agree.
constexpr int UPB_THREADS = 256;
constexpr int UPB_ROWS = 2 * UPB_THREADS;  // rows per block

// Sum of part[0..count) in a fixed order, returned to every thread of the
// block (red: 32 doubles of shared memory).
__device__ double sum_parts(const double* __restrict__ part, int count, double* red) {
    if (threadIdx.x < 32) {
        double s = 0.0;
        for (int i = threadIdx.x; i < count; i += 32) s += part[i];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) red[0] = s;
    }
    __syncthreads();
    const double s = red[0];
    __syncthreads();
    return s;
}

// Block-wide FP64 sum in a fixed order, result in thread 0.
__device__ double block_sum_fixed(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x / 32, l = threadIdx.x % 32;
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < static_cast<int>(blockDim.x / 32); ++i) s += red[i];
    __syncthreads();
    return s;
}

// alpha_k = sum of the q.w partials; w -= alpha_k q + beta_old q_old; the
// partial sums of ||w||^2 per block.
__global__ void __launch_bounds__(UPB_THREADS) lz_upd_axpy_kernel(int64_t n, int k, LzState* st, double* alpha,
                                                                  const double* __restrict__ q, double* w,
                                                                  const double* __restrict__ vold,
                                                                  const double* __restrict__ qdot_part, int nqdot,
                                                                  double* norm_part) {
    if (st->stopped) return;
    __shared__ double red[32];
    const double a = sum_parts(qdot_part, nqdot, red);
    const double b_old = st->beta_old;
    double s = 0.0;
#pragma unroll
    for (int r = 0; r < UPB_ROWS / UPB_THREADS; ++r) {
        const int64_t i = static_cast<int64_t>(blockIdx.x) * UPB_ROWS + r * UPB_THREADS + threadIdx.x;
        if (i < n) {
            const double v = w[i] - a * q[i] - b_old * vold[i];
            w[i] = v;
            s += v * v;
        }
    }
    s = block_sum_fixed(s, red);
    if (threadIdx.x == 0) {
        norm_part[blockIdx.x] = s;
        if (blockIdx.x == 0) alpha[k] = a;
    }
}

// beta_k = sqrt(sum of the partials); the stop tests of src/lanczos.cu:145-159;
// q_old = q; q = w / beta_k; V[:, k+1] = q when k < m-1; nb_iter++.
__global__ void __launch_bounds__(UPB_THREADS) lz_upd_scale_kernel(int64_t n, int64_t m, int k, double tol,
                                                                   LzState* st, const double* alpha, double* beta,
                                                                   double* q, const double* __restrict__ w,
                                                                   double* vold, double* V, float* q32,
                                                                   const double* __restrict__ norm_part,
                                                                   int nnorm) {
    if (st->stopped) return;
    __shared__ double red[32];
    const double b = sqrt(sum_parts(norm_part, nnorm, red));
    const double a = alpha[k];
    if (blockIdx.x == 0 && threadIdx.x == 0) beta[k] = b;
    if ((b <= tol * a && k > 1) || b == 0.0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) st->stopped = 1;
        return;
    }
    const double inv = 1.0 / b;
    const bool store_v = (k < m - 1);
#pragma unroll
    for (int r = 0; r < UPB_ROWS / UPB_THREADS; ++r) {
        const int64_t i = static_cast<int64_t>(blockIdx.x) * UPB_ROWS + r * UPB_THREADS + threadIdx.x;
        if (i < n) {
            const double qn = w[i] * inv;
            vold[i] = q[i];
            q[i] = qn;
            q32[i] = static_cast<float>(qn);
            if (store_v) V[static_cast<int64_t>(k + 1) * n + i] = qn;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->beta_old = b;
        st->nb_iter = k + 1;
    }
}

// One Lanczos update (single block of UPD_THREADS):
//   alpha_k = q.w; w -= alpha_k q + beta_old q_old; beta_k = ||w||;
//   stop tests of src/lanczos.cu:145-159; q_old = q; q = w / beta_k;
//   V[:, k+1] = q when k < m-1; nb_iter++.
// For n <= UPD_THREADS * UPD_R each thread loads its UPD_R elements of q, w
// and q_old once, all up front (one memory latency instead of one per
// element and pass); the sums run in the same per-thread order either way.
constexpr int UPD_THREADS = 1024;
constexpr int UPD_R = 8;

__global__ void __launch_bounds__(UPD_THREADS) lz_update_kernel(int64_t n, int64_t m, int k, double tol, LzState* st,
                                                                double* alpha, double* beta, double* q, double* w,
                                                                double* vold, double* V, float* q32) {
    if (st->stopped) return;
    __shared__ double red[32];
    const double b_old = st->beta_old;
    const bool store_v = (k < m - 1);
    double* vnext = V + static_cast<int64_t>(k + 1) * n;
    if (n <= static_cast<int64_t>(UPD_THREADS) * UPD_R) {
        double qv[UPD_R], wv[UPD_R], ov[UPD_R];
#pragma unroll
        for (int r = 0; r < UPD_R; ++r) {
            const int64_t i = threadIdx.x + static_cast<int64_t>(r) * UPD_THREADS;
            const bool in = i < n;
            qv[r] = in ? q[i] : 0.0;
            wv[r] = in ? w[i] : 0.0;
            ov[r] = in ? vold[i] : 0.0;
        }
        double s = 0.0;
#pragma unroll
        for (int r = 0; r < UPD_R; ++r) s += qv[r] * wv[r];
        const double a = block_sum(s, red);
        s = 0.0;
#pragma unroll
        for (int r = 0; r < UPD_R; ++r) {
            wv[r] = wv[r] - a * qv[r] - b_old * ov[r];
            s += wv[r] * wv[r];
        }
        const double b = sqrt(block_sum(s, red));
        if (threadIdx.x == 0) {
            alpha[k] = a;
            beta[k] = b;
        }
        if ((b <= tol * a && k > 1) || b == 0.0) {
#pragma unroll
            for (int r = 0; r < UPD_R; ++r) {
                const int64_t i = threadIdx.x + static_cast<int64_t>(r) * UPD_THREADS;
                if (i < n) w[i] = wv[r];
            }
            __syncthreads();
            if (threadIdx.x == 0) st->stopped = 1;
            return;
        }
        const double inv = 1.0 / b;
#pragma unroll
        for (int r = 0; r < UPD_R; ++r) {
            const int64_t i = threadIdx.x + static_cast<int64_t>(r) * UPD_THREADS;
            if (i < n) {
                const double qn = wv[r] * inv;
                w[i] = wv[r];
                vold[i] = qv[r];
                q[i] = qn;
                q32[i] = static_cast<float>(qn);
                if (store_v) vnext[i] = qn;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            st->beta_old = b;
            st->nb_iter = k + 1;
        }
        return;
    }
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += q[i] * w[i];
    const double a = block_sum(s, red);
    s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = w[i] - a * q[i] - b_old * vold[i];
        w[i] = v;
        s += v * v;
    }
    const double b = sqrt(block_sum(s, red));
    if (threadIdx.x == 0) {
        alpha[k] = a;
        beta[k] = b;
    }
    if ((b <= tol * a && k > 1) || b == 0.0) {
        __syncthreads();
        if (threadIdx.x == 0) st->stopped = 1;
        return;
    }
    const double inv = 1.0 / b;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double qn = w[i] * inv;
        vold[i] = q[i];
        q[i] = qn;
        q32[i] = static_cast<float>(qn);
        if (store_v) vnext[i] = qn;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        st->beta_old = b;
        st->nb_iter = k + 1;
    }
}

// The largest eigenpair of T, by one block of 128 threads (tridiag.cuh).  The solver's
// 8 (mx) doubles of work and scratch live in dynamic shared memory when the
// launch provides it (smem != 0), else in `work` (global, 8 mx doubles);
// mx = max_iter + 1 >= nb_iter.
__global__ void lz_tridiag_kernel(LzState* st, const double* alpha, const double* beta, double* uk, double* work,
                                  int64_t mx, int smem) {
    extern __shared__ double tsm[];
    const int lane = threadIdx.x;  // thread index in the block
    const int64_t m = st->nb_iter;
    if (m == 0) {  // the all-zero branch of src/lanczos.cu:171-184
        if (lane == 0) {
            st->no_ritz = 1;
            st->lo = 0.0;
            st->up = 1.0;
            st->theta = 0.0;
            st->scale = 1.0;
            st->inv_scale = 1.0;
        }
        return;
    }
    if (m == 1) {
        if (lane == 0) {
            st->no_ritz = 0;
            st->theta = alpha[0];
            uk[0] = 1.0;
        }
        return;
    }
    double* base = smem ? tsm : work;
    const double t = block_tridiag_top(alpha, beta, m, uk, base, base + 5 * mx);
    if (lane == 0) {
        st->no_ritz = 0;
        st->theta = t;
    }
}

// y = V[:, 0:m] u (m = nb_iter); y32 = FP32(y); optionally the Ritz vector out.
__global__ void lz_ritz_kernel(int64_t n, const LzState* st, const double* __restrict__ V,
                               const double* __restrict__ u, double* y, float* y32, double* ritz_out) {
    if (st->no_ritz) return;
    const int64_t m = st->nb_iter;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        double s = 0.0;
        for (int64_t j = 0; j < m; ++j) s += V[j * n + i] * u[j];
        y[i] = s;
        y32[i] = static_cast<float>(s);
        if (ritz_out) ritz_out[i] = s;
    }
}

// ||ry - theta y|| and the bound: lo = sqrt(theta), up = sqrt(theta + ||r||),
// scale = up > 0 ? up : 1 (single block).
__global__ void lz_resid_kernel(int64_t n, const double* ry, const double* y, LzState* st) {
    if (st->no_ritz) return;
    __shared__ double red[32];
    const double theta = st->theta;
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double r = ry[i] - theta * y[i];
        s += r * r;
    }
    const double t = block_sum(s, red);
    if (threadIdx.x == 0) {
        st->resid_norm2 = t;
        const double up = sqrt(theta + sqrt(t));
        st->lo = sqrt(theta);
        st->up = up;
        const double scale = up > 0.0 ? up : 1.0;
        st->scale = scale;
        st->inv_scale = 1.0 / scale;
    }
}

// No iteration at all (max_iter or n is 0): lo = 0, up = 1.
__global__ void lz_trivial_kernel(LzState* st) {
    st->nb_iter = 0;
    st->no_ritz = 1;
    st->theta = 0.0;
    st->lo = 0.0;
    st->up = 1.0;
    st->scale = 1.0;
    st->inv_scale = 1.0;
}

// The tile matvec's operands for one bound: the tensor map of the FP32
// matrix and the partial-sum buffers.
struct SymvCtx {
    bool on = false;
    CUtensorMap tmap;
    int nb = 0;
    double* part = nullptr;
    int* err = nullptr;
    int warps = 16;  // consumer warps of the tile kernel
    int sweeps = 0;  // matvecs launched so far (odd ones walk the tiles backwards)
};

cudaError_t matvec(const float* A, int64_t n, int64_t ld, const float* x, double* y64, float* y32, const int* skip,
                   int sm_count, cudaStream_t s, SymvCtx& sv, const double* qd = nullptr,
                   double* qdot_part = nullptr) {
    if (sv.on) {
        const int64_t ntiles = static_cast<int64_t>(sv.nb) * (sv.nb + 1) / 2;
        const int64_t grid = ntiles < sm_count ? ntiles : sm_count;
        const int reverse = sv.sweeps++ & 1;
        if (sv.warps == 8)
            lz_symv_kernel<8><<<static_cast<unsigned>(grid), 32 * 9, SV_SMEM, s>>>(sv.tmap, n, sv.nb, x, sv.part,
                                                                                 skip, sv.err, reverse);
        else
            lz_symv_kernel<16><<<static_cast<unsigned>(grid), 32 * 17, SV_SMEM, s>>>(sv.tmap, n, sv.nb, x, sv.part,
                                                                                   skip, sv.err, reverse);
        count_launch();
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        lz_symv_reduce_kernel<<<static_cast<unsigned>((n + 31) / 32), 128, 0, s>>>(sv.part, sv.nb, n, y64, y32,
                                                                                  skip, qd, qdot_part);
        count_launch();
        return cudaGetLastError();
    }
    const size_t smem = sizeof(float) * static_cast<size_t>(ld);
    const int threads = 256;
    // At most the CTAs that fit at once (the loop strides over the rest);
    // two columns per warp when one per warp would not fit in one wave.
    static size_t cached_smem = 0;
    static int per_sm = 0;
    if (smem != cached_smem || per_sm < 1) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lz_matvec_kernel, threads, smem) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        cached_smem = smem;
    }
    const int64_t cap = static_cast<int64_t>(sm_count) * per_sm;
    const int pair = (n + 7) / 8 > cap ? 1 : 0;
    int64_t blocks = pair ? ((n + 1) / 2 + 7) / 8 : (n + 7) / 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    lz_matvec_kernel<<<static_cast<unsigned>(blocks), threads, smem, s>>>(A, n, ld, x, y64, y32, skip, pair);
    count_launch();
    return cudaGetLastError();
}

struct LzPtrs {
    LzState* st;
    double *alpha, *beta, *q, *w, *vold, *V, *y, *ry, *uk, *work, *part, *qdot, *norm;
    float *q32, *u32;
};

LzPtrs lz_ptrs(void* d_state, int64_t n, int64_t m) {
    const LzLayout L = lz_layout(n, m);
    char* base = static_cast<char*>(d_state);
    LzPtrs p;
    p.st = reinterpret_cast<LzState*>(base + L.state);
    p.alpha = reinterpret_cast<double*>(base + L.alpha);
    p.beta = reinterpret_cast<double*>(base + L.beta);
    p.q = reinterpret_cast<double*>(base + L.q);
    p.w = reinterpret_cast<double*>(base + L.w);
    p.vold = reinterpret_cast<double*>(base + L.vold);
    p.V = reinterpret_cast<double*>(base + L.V);
    p.y = reinterpret_cast<double*>(base + L.y);
    p.ry = reinterpret_cast<double*>(base + L.ry);
    p.q32 = reinterpret_cast<float*>(base + L.q32);
    p.u32 = reinterpret_cast<float*>(base + L.u32);
    p.uk = reinterpret_cast<double*>(base + L.uk);
    p.work = reinterpret_cast<double*>(base + L.work);
    p.part = reinterpret_cast<double*>(base + L.part);
    p.qdot = reinterpret_cast<double*>(base + L.qdot);
    p.norm = reinterpret_cast<double*>(base + L.norm);
    return p;
}

}  // namespace

int g_lanczos_symv = -1;

size_t lanczos_state_bytes(int64_t n, int64_t max_iter) {
    const int64_t m = max_iter < n ? max_iter : n;
    return lz_layout(n, m < 0 ? 0 : m).total;
}

const double* lanczos_scale_ptr(void* d_state, int64_t n, int64_t max_iter) {
    const int64_t m = max_iter < n ? max_iter : n;
    return &lz_ptrs(d_state, n, m < 0 ? 0 : m).st->scale;
}

const double* lanczos_inv_scale_ptr(void* d_state, int64_t n, int64_t max_iter) {
    const int64_t m = max_iter < n ? max_iter : n;
    return &lz_ptrs(d_state, n, m < 0 ? 0 : m).st->inv_scale;
}

psdgb_status lanczos_bound_async(DeviceState* ds, const float* a32, int64_t n, int64_t ld, int64_t max_iter,
                                 double tol, uint64_t seed, int residual_mode, void* d_state, cudaStream_t s,
                                 const double* d_warm, double* d_ritz_out) {
    const int64_t m = max_iter < n ? max_iter : n;  // src/lanczos.cu:55
    const LzPtrs P = lz_ptrs(d_state, n, m < 0 ? 0 : m);
    if (m <= 0) {  // no iteration: the all-zero branch of src/lanczos.cu:171-184
        lz_trivial_kernel<<<1, 1, 0, s>>>(P.st);
        count_launch();
        PSDGB_CUDA_TRY(cudaGetLastError());
        return PSDGB_OK;
    }
    SymvCtx sv;
    // TMA reads need a 16-byte aligned matrix (a caller's workspace may not be).
    const bool aligned = (reinterpret_cast<uintptr_t>(a32) & 15u) == 0 && ld % 4 == 0;
    sv.on = aligned && (g_lanczos_symv >= 1 ? n >= 128 : (g_lanczos_symv < 0 && n >= 2048));
    if (sv.on) {
        sv.nb = static_cast<int>((n + SV_T - 1) / SV_T);
        sv.part = P.part;
        sv.err = ds->d_error;
        if (!make_tmap_f32(&sv.tmap, a32, ld, n, n, SV_T, SV_T)) {
            set_error("Lanczos bound: encoding the tensor map of the FP32 matrix failed");
            return PSDGB_ERR_CUDA;
        }
        sv.warps = g_lanczos_symv == 2 ? 8 : 16;
        static int smem_set_device = -1;
        if (smem_set_device != ds->device) {
            PSDGB_CUDA_TRY(cudaFuncSetAttribute(lz_symv_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                static_cast<int>(SV_SMEM)));
            PSDGB_CUDA_TRY(cudaFuncSetAttribute(lz_symv_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                static_cast<int>(SV_SMEM)));
            smem_set_device = ds->device;
        }
    }
    const size_t xs_bytes = sizeof(float) * static_cast<size_t>(ld);
    if (!sv.on && xs_bytes > 48 * 1024) {
        if (xs_bytes > 200 * 1024) {
            set_error("Lanczos bound: n too large for the shared-memory vector stage (n <= 51200)");
            return PSDGB_ERR_INVALID_ARGUMENT;
        }
        PSDGB_CUDA_TRY(cudaFuncSetAttribute(lz_matvec_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            static_cast<int>(xs_bytes)));
    }
    PSDGB_CUDA_TRY(cudaMemsetAsync(P.alpha, 0, sizeof(double) * (m + 1), s));
    PSDGB_CUDA_TRY(cudaMemsetAsync(P.beta, 0, sizeof(double) * (m + 1), s));
    lz_init_kernel<<<1, 1024, 0, s>>>(n, seed, d_warm, P.st, P.q, P.vold, P.V, P.q32);
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());

    const int* stopped = &P.st->stopped;
    const int nqdot = static_cast<int>((n + 31) / 32);
    const int nnorm = static_cast<int>((n + UPB_ROWS - 1) / UPB_ROWS);
    for (int64_t k = 0; k < m; ++k) {
        PSDGB_CUDA_TRY(matvec(a32, n, ld, P.q32, nullptr, P.u32, stopped, sm_budget(ds), s, sv));  // u = A q
        if (sv.on) {
            // w = A^T u with the q.w partials; the update over nnorm blocks.
            PSDGB_CUDA_TRY(matvec(a32, n, ld, P.u32, P.w, nullptr, stopped, sm_budget(ds), s, sv, P.q, P.qdot));
            lz_upd_axpy_kernel<<<static_cast<unsigned>(nnorm), UPB_THREADS, 0, s>>>(
                n, static_cast<int>(k), P.st, P.alpha, P.q, P.w, P.vold, P.qdot, nqdot, P.norm);
            count_launch();
            PSDGB_CUDA_TRY(cudaGetLastError());
            lz_upd_scale_kernel<<<static_cast<unsigned>(nnorm), UPB_THREADS, 0, s>>>(
                n, m, static_cast<int>(k), tol, P.st, P.alpha, P.beta, P.q, P.w, P.vold, P.V, P.q32, P.norm, nnorm);
            count_launch();
            PSDGB_CUDA_TRY(cudaGetLastError());
        } else {
            PSDGB_CUDA_TRY(matvec(a32, n, ld, P.u32, P.w, nullptr, stopped, sm_budget(ds), s, sv));  // w = A^T u
            lz_update_kernel<<<1, UPD_THREADS, 0, s>>>(n, m, static_cast<int>(k), tol, P.st, P.alpha, P.beta, P.q,
                                                       P.w, P.vold, P.V, P.q32);
            count_launch();
            PSDGB_CUDA_TRY(cudaGetLastError());
        }
    }
    {
        const size_t tsmem = sizeof(double) * 8 * static_cast<size_t>(m + 1);
        const int use_smem = tsmem <= 48 * 1024 ? 1 : 0;
        lz_tridiag_kernel<<<1, 128, use_smem ? tsmem : 0, s>>>(P.st, P.alpha, P.beta, P.uk, P.work, m + 1, use_smem);
    }
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    {
        int64_t blocks = (n + 255) / 256;
        if (blocks > 4096) blocks = 4096;
        lz_ritz_kernel<<<static_cast<unsigned>(blocks), 256, 0, s>>>(n, P.st, P.V, P.uk, P.y, P.q32, d_ritz_out);
        count_launch();
        PSDGB_CUDA_TRY(cudaGetLastError());
    }
    const int* no_ritz = &P.st->no_ritz;
    if (residual_mode == PSDGB_RESIDUAL_EXACT) {
        PSDGB_CUDA_TRY(matvec(a32, n, ld, P.q32, nullptr, P.u32, no_ritz, sm_budget(ds), s, sv));  // A y
        PSDGB_CUDA_TRY(matvec(a32, n, ld, P.u32, P.ry, nullptr, no_ritz, sm_budget(ds), s, sv));   // A^T A y
    } else {
        PSDGB_CUDA_TRY(matvec(a32, n, ld, P.q32, P.ry, nullptr, no_ritz, sm_budget(ds), s, sv));   // A y
    }
    lz_resid_kernel<<<1, 1024, 0, s>>>(n, P.ry, P.y, P.st);
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    return PSDGB_OK;
}

psdgb_status lanczos_read(void* d_state, int64_t n, int64_t max_iter, cudaStream_t s, LanczosResult* res,
                          double* h_alpha, double* h_beta) {
    const int64_t m0 = max_iter < n ? max_iter : n;
    const int64_t m = m0 < 0 ? 0 : m0;
    const LzPtrs P = lz_ptrs(d_state, n, m);
    LzState hst{};
    std::vector<double> ha(m + 1, 0.0), hb(m + 1, 0.0);
    PSDGB_CUDA_TRY(cudaMemcpyAsync(&hst, P.st, sizeof(LzState), cudaMemcpyDeviceToHost, s));
    if (m > 0) {
        PSDGB_CUDA_TRY(cudaMemcpyAsync(ha.data(), P.alpha, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
        PSDGB_CUDA_TRY(cudaMemcpyAsync(hb.data(), P.beta, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
    }
    PSDGB_CUDA_TRY(cudaStreamSynchronize(s));
    if (h_alpha) for (int64_t i = 0; i < max_iter; ++i) h_alpha[i] = (i < m) ? ha[i] : 0.0;
    if (h_beta) for (int64_t i = 0; i < max_iter; ++i) h_beta[i] = (i < m) ? hb[i] : 0.0;
    res->nb_iter = hst.nb_iter;
    res->theta = hst.theta;
    res->lo = hst.lo;
    res->up = hst.up;
    return PSDGB_OK;
}

}  // namespace psdgb
