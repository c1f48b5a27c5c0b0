// batch.cu — projection of a block-diagonal iterate: many independent
// symmetric blocks of uneven sizes in one pass.
//
// A block-diagonal SDP iterate is projected block by block; the reference
// offers only one call per block (each a full chain of ~100 library calls).
// Here the whole batch is one plan and a fixed number of kernel launches,
// independent of the number of blocks, so it can be captured in one CUDA
// graph:
//
//   batch_to_f32      every block's upper triangle -> FP32 symmetric copy
//   lz_batch_kernel   one CTA per block runs the whole Lanczos bound of its
//                     block (recurrence, tridiagonal eigenpair, Ritz residual)
//                     and leaves the block's scale 1/up on the device; one
//                     launch per size class (64 / 128 / 256 / 512 threads by
//                     n), so small blocks run many CTAs per SM
//   batch_chain       (FP16 / FP16x3) the blocks of n <= 128: the whole filter
//                     per block in one persistent kernel, operands in shared
//                     memory (batch_chain.cu); these blocks' Lanczos classes
//                     and this kernel run on a second stream, beside the
//                     larger blocks' bound
//   batch_split       scaled operand terms of the larger blocks into one
//                     strided layout
//   3 x steps         per product: grouped 128 x 128 tiles (gemm_tc.cu) over
//                     the tile list of the larger blocks, or also 256 x 256
//                     pair tiles where a block's tile rows pair up
//                     (gemm_pairwide.cu)
//   batch_split (Xs)  Xs = X / up per block
//   1 dual product    (X + up (Xs A + A Xs)/2) / 2 into the caller's blocks
//
// Layout: blocks are padded to np = n rounded up to 128 and shelf-packed into
// a strip of width ld = max np (blocks of one size side by side, a shelf per
// row band), so a single TMA descriptor per operand plane covers every block.
// The autotuner times the whole projection under each tile shape (pair tiles
// where two tile rows of a block fit, or 128 x 128 only), route of the small
// blocks (on chip or per product), accumulator configuration and tile order
// (LPT: largest blocks first, or block order) and keeps the fastest.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "internal.h"
#include "convert.h"
#include "tridiag.cuh"


namespace {

using namespace psdgb;

constexpr int LZ_CLASSES = 4;     // Lanczos CTA sizes 512, 256, 128, 64 threads

// Lanczos CTA size class of a block of size n: the smallest CTA of at least
// n threads, between 64 and 512.
inline int lz_class(int64_t n) { return n > 256 ? 0 : (n > 128 ? 1 : (n > 64 ? 2 : 3)); }
constexpr int COPY_THREADS = 256;  // 32 x 8 transpose tiles

struct BatchState {
    double theta, lo, up, scale, inv_scale;
    int nb_iter, pad;
};

struct LzBlockDesc {
    int n;
    int ld4;
    int m;
    int pad;
    long long a32_off;  // floats
    long long vec_off;  // doubles: V (n*m) | alpha, beta, uk (m+1 each) | work (5(m+1))
    long long x_off;    // doubles into the packed FP64 blocks
};

inline int64_t up_to(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Block-wide FP64 sum through shared memory: every thread stores its
// partial, warp 0 adds blockDim/32 values per lane and reduces across lanes,
// and the result is broadcast.  About 21 FP64 warp instructions per sum
// instead of 10 per warp for shuffle trees in every warp (FP64 issue is
// scarce on this part).  part holds blockDim.x doubles, red one.
__device__ double cta_sum(double v, double* part, double* red) {
    __syncthreads();
    part[threadIdx.x] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = 0.0;
        for (int i = threadIdx.x; i < static_cast<int>(blockDim.x); i += 32) t += part[i];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) red[0] = t;
    }
    __syncthreads();
    return red[0];
}

// The square root r of a block-wide sum and 1 / r (r == 0: rinv = if_zero),
// computed once by thread 0 and broadcast: an FP64 square root or division
// is a sequence of FP64 instructions, which every warp issuing them would
// queue on this part's scarce FP64 pipe.  IEEE-rounded either way, so the
// same bits.
__device__ void cta_sum_sqrt(double v, double* part, double* red, double if_zero, double& r, double& rinv) {
    __syncthreads();
    part[threadIdx.x] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = 0.0;
        for (int i = threadIdx.x; i < static_cast<int>(blockDim.x); i += 32) t += part[i];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) {
            const double s = sqrt(t);
            red[0] = s;
            red[1] = s != 0.0 ? 1.0 / s : if_zero;
        }
    }
    __syncthreads();
    r = red[0];
    rinv = red[1];
}

// y[c] = sum_r A[c*ld4 + r] x[r] for the block's symmetric FP32 matrix.
// Each warp takes four columns at a time and each lane keeps up to sixteen
// float4 loads in flight (the columns are L2-resident and the loop is
// latency-bound otherwise).  Lane partial sums and the shuffle reduction are
// FP32 (a column here is at most 4096 long), one FP64 conversion per column:
// on this part a warp-wide FP64 add occupies the FP64 pipe for many cycles,
// and FP64 shuffle reductions made the whole bound FP64-bound.
__device__ void cta_matvec(const float* __restrict__ A, int n, int ld4, const float* xs, double* y64, float* y32) {
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32, nw = blockDim.x / 32;
    const float4* xs4 = reinterpret_cast<const float4*>(xs);
    const int kv = ld4 / 4;
    for (int c0 = warp * 4; c0 < n; c0 += nw * 4) {
        float s[4] = {0.f, 0.f, 0.f, 0.f};
        const float4* col[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) col[j] = reinterpret_cast<const float4*>(A + static_cast<int64_t>(min(c0 + j, n - 1)) * ld4);
#pragma unroll 4
        for (int k = lane; k < kv; k += 32) {
            const float4 b = xs4[k];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float4 a = __ldg(col[j] + k);
                s[j] = fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, fmaf(a.w, b.w, s[j]))));
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float acc = s[j];
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            const int c = c0 + j;
            if (lane == 0 && c < n) {
                if (y64) y64[c] = f2d(acc);  // exact, off the FP64 pipe
                if (y32) y32[c] = acc;
            }
        }
    }
}

// y[c] = sum_r A[c*ld4 + r] x[r] with one column per thread (blocks of at
// most 128 in CTAs of 64 or 128 threads): each thread streams its own
// column with eight 16-byte loads in flight and sums it in FP32, one FP64
// conversion per column; no cross-lane reduction, so a matvec costs a few
// memory round trips instead of one per group of four columns.
__device__ void cta_matvec_cols(const float* __restrict__ A, int n, int ld4, const float* xs, double* y64,
                                float* y32) {
    const float4* xs4 = reinterpret_cast<const float4*>(xs);
    const int kv = ld4 / 4;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        const float4* col = reinterpret_cast<const float4*>(A + static_cast<int64_t>(c) * ld4);
        float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
        int k = 0;
        for (; k + 8 <= kv; k += 8) {
            float4 a[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) a[j] = __ldg(col + k + j);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const float4 xb = xs4[k + j];
                s0 = fmaf(a[j].x, xb.x, s0);
                s1 = fmaf(a[j].y, xb.y, s1);
                s2 = fmaf(a[j].z, xb.z, s2);
                s3 = fmaf(a[j].w, xb.w, s3);
            }
        }
        for (; k < kv; ++k) {
            const float4 a = __ldg(col + k);
            const float4 xb = xs4[k];
            s0 = fmaf(a.x, xb.x, s0);
            s1 = fmaf(a.y, xb.y, s1);
            s2 = fmaf(a.z, xb.z, s2);
            s3 = fmaf(a.w, xb.w, s3);
        }
        const float acc = (s0 + s1) + (s2 + s3);
        if (y64) y64[c] = f2d(acc);  // exact, off the FP64 pipe
        if (y32) y32[c] = acc;
    }
}

// The matvec of a T-thread Lanczos CTA.
template <int T>
__device__ __forceinline__ void lz_matvec(const float* __restrict__ A, int n, int ld4, const float* xs, double* y64,
                                          float* y32) {
    if (T <= 128)
        cta_matvec_cols(A, n, ld4, xs, y64, y32);
    else
        cta_matvec(A, n, ld4, xs, y64, y32);
}

// The Lanczos bound of one block per CTA (src/lanczos.cu:41-293, as in
// lanczos.cu): CTA blockIdx.x takes block idx[blockIdx.x].  T threads, at
// most 64 registers each (1024 / T CTAs per SM by registers).
template <int T>
__global__ void __launch_bounds__(T, 1024 / T) lz_batch_kernel(const LzBlockDesc* __restrict__ descs,
                                                              const int* __restrict__ idx,
                                                              const float* __restrict__ a32, double* vec,
                                                              BatchState* states, double tol, uint64_t seed,
                                                              int residual_mode) {
    extern __shared__ double sh[];
    __shared__ double red[32];
    __shared__ double part[T];
    const int bidx = idx[blockIdx.x];
    const LzBlockDesc d = descs[bidx];
    const int n = d.n, ld4 = d.ld4, m = d.m;
    BatchState* st = states + bidx;
    if (m <= 0) {
        if (threadIdx.x == 0) *st = BatchState{0.0, 0.0, 1.0, 1.0, 1.0, 0, 0};
        return;
    }
    double* q = sh;
    double* w = q + ld4;
    double* vold = w + ld4;
    double* y = vold + ld4;
    double* ry = y + ld4;
    float* x32 = reinterpret_cast<float*>(ry + ld4);  // ld4 floats
    float* u32 = x32 + ld4;
    const float* A = a32 + d.a32_off;
    double* V = vec + d.vec_off;
    double* alpha = V + static_cast<int64_t>(n) * m;
    double* beta = alpha + (m + 1);
    double* uk = beta + (m + 1);
    double* work = uk + (m + 1);
    for (int i = threadIdx.x; i < ld4; i += blockDim.x) {
        x32[i] = 0.f;
        u32[i] = 0.f;
    }
    // start vector (uniform (0, 1] from the seed), normalised
    double ss = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const uint64_t h = splitmix64(seed ^ splitmix64(static_cast<uint64_t>(i)));
        const double u = static_cast<double>((h >> 11) + 1) * 0x1.0p-53;
        q[i] = u;
        ss += u * u;
    }
    double nrm, inv0;
    cta_sum_sqrt(ss, part, red, 1.0, nrm, inv0);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        q[i] *= inv0;
        V[i] = q[i];
        vold[i] = 0.0;
        x32[i] = d2f_rn(q[i]);
    }
    double beta_old = 0.0;
    int nb = 0;
    for (int k = 0; k < m; ++k) {
        __syncthreads();
        lz_matvec<T>(A, n, ld4, x32, nullptr, u32);  // u = A q
        __syncthreads();
        lz_matvec<T>(A, n, ld4, u32, w, nullptr);    // w = A^T u
        __syncthreads();
        double s = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) s += q[i] * w[i];
        const double a = cta_sum(s, part, red);
        s = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double v = w[i] - a * q[i] - beta_old * vold[i];
            w[i] = v;
            s += v * v;
        }
        double b, binv;
        cta_sum_sqrt(s, part, red, 0.0, b, binv);
        if (threadIdx.x == 0) {
            alpha[k] = a;
            beta[k] = b;
        }
        if ((b <= tol * a && k > 1) || b == 0.0) break;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double qn = w[i] * binv;
            vold[i] = q[i];
            q[i] = qn;
            x32[i] = d2f_rn(qn);
            if (k < m - 1) V[static_cast<int64_t>(k + 1) * n + i] = qn;
        }
        beta_old = b;
        nb = k + 1;
    }
    __syncthreads();
    if (nb == 0) {
        if (threadIdx.x == 0) *st = BatchState{0.0, 0.0, 1.0, 1.0, 1.0, 0, 0};
        return;
    }
    double theta;
    if (nb == 1) {
        theta = alpha[0];
        if (threadIdx.x == 0) uk[0] = 1.0;
    } else {
        // Scratch for the staged T: the q / w / vold vectors (3 ld4 >= 3 nb
        // doubles of shared memory), unused from here on.
        theta = block_tridiag_top(alpha, beta, nb, uk, work, q);
    }
    __syncthreads();
    // Ritz vector y = V u and the residual
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < nb; ++j) s += V[static_cast<int64_t>(j) * n + i] * uk[j];
        y[i] = s;
        x32[i] = d2f_rn(s);
    }
    __syncthreads();
    if (residual_mode == PSDGB_RESIDUAL_EXACT) {
        lz_matvec<T>(A, n, ld4, x32, nullptr, u32);
        __syncthreads();
        lz_matvec<T>(A, n, ld4, u32, ry, nullptr);
    } else {
        lz_matvec<T>(A, n, ld4, x32, ry, nullptr);
    }
    __syncthreads();
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double r = ry[i] - theta * y[i];
        s += r * r;
    }
    const double rs = cta_sum(s, part, red);
    if (threadIdx.x == 0) {
        const double rn = sqrt(rs);
        const double up = sqrt(theta + rn);
        const double scale = up > 0.0 ? up : 1.0;
        *st = BatchState{theta, sqrt(theta), up, scale, 1.0 / scale, nb, 0};
    }
}

// The symmetric matrix defined by the upper triangle of column-major X_b,
// written as FP32 rows (a32, n x ld4): one warp per 32 x 32 tile of the
// batch's tile list (every block's tiles over rows < n, columns < ld4;
// columns >= n written as zero), transposed through the warp's own
// shared-memory tile, so no CTA idles on a small block and no CTA barrier
// is needed.
__global__ void __launch_bounds__(COPY_THREADS) batch_to_f32_kernel(const LzBlockDesc* __restrict__ descs,
                                                                    const int4* __restrict__ tiles, int num_tiles,
                                                                    const double* __restrict__ x, float* a32) {
    __shared__ float sm[COPY_THREADS / 32][32][33];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    float(&t)[32][33] = sm[warp];
    for (int w = blockIdx.x * (COPY_THREADS / 32) + warp; w < num_tiles; w += gridDim.x * (COPY_THREADS / 32)) {
        const int4 td = tiles[w];  // block, tile row, tile column
        const LzBlockDesc d = descs[td.x];
        const int n = d.n, ld4 = d.ld4, bi = td.y, bj = td.z;
        const double* X = x + d.x_off;
        float* A = a32 + d.a32_off;
        const int rbase = (bi <= bj) ? bi * 32 : bj * 32;
        const int cbase = (bi <= bj) ? bj * 32 : bi * 32;
        __syncwarp();
#pragma unroll 8
        for (int ty = 0; ty < 32; ++ty) {
            const int r = rbase + lane, c = cbase + ty;
            // Narrowed on the integer ALUs (convert.h): FP64 issues slowly here.
            t[ty][lane] = (r < n && c < n) ? d2f_rn(X[r + static_cast<int64_t>(c) * n]) : 0.0f;
        }
        __syncwarp();
#pragma unroll 8
        for (int ty = 0; ty < 32; ++ty) {
            const int i = bi * 32 + ty, j = bj * 32 + lane;
            if (i >= n || j >= ld4) continue;
            float v = (bi < bj) ? t[lane][ty] : (bi > bj) ? t[ty][lane] : ((ty <= lane) ? t[lane][ty] : t[ty][lane]);
            if (j >= n) v = 0.0f;
            A[static_cast<int64_t>(i) * ld4 + j] = v;
        }
    }
}

// Scaled operand terms of the blocks into the strided layout, from the FP32
// copy: the first split A = X / up, and again Xs = X / up for the final
// product (the copy holds exactly the FP32 narrowing of the symmetric matrix
// X's upper triangle defines, which is what Xs needs).  One warp per 32 x 32
// tile of the split's tile list (the tiles of each listed block that meet
// its n x n corner; the rest of the block's np x np area is zero from the
// plan's creation on and no product writes a nonzero there); lane l writes
// columns 8 (l % 4) .. + 7 of rows l / 4 + 8 k as one 16-byte store per
// term plane, 8 rows x 64 bytes per warp instruction.
__global__ void __launch_bounds__(COPY_THREADS) batch_split_kernel(const LzBlockDesc* __restrict__ lz,
                                                                   const BlockDesc* __restrict__ blocks,
                                                                   const BatchState* __restrict__ states,
                                                                   const float* __restrict__ a32, SplitMat out,
                                                                   int fmt, int64_t ld,
                                                                   const int4* __restrict__ tiles, int num_tiles) {
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int c8 = 8 * (lane & 3);
    for (int w = blockIdx.x * (COPY_THREADS / 32) + warp; w < num_tiles; w += gridDim.x * (COPY_THREADS / 32)) {
        const int4 td = tiles[w];  // block, tile row, tile column
        const LzBlockDesc d = lz[td.x];
        const BlockDesc bd = blocks[td.x];
        // The scaling runs in FP32, as in the single-matrix split.
        const float inv = d2f_rn(states[td.x].inv_scale);
        const int n = d.n, j0 = td.z * 32 + c8;
        const float* A = a32 + d.a32_off;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = td.y * 32 + (lane >> 2) + 8 * k;
            float v[8];
            if (i < n && j0 + 8 <= n) {  // ld4 is a multiple of 4: 16-byte rows
                const float* src = A + static_cast<int64_t>(i) * d.ld4 + j0;
                const float4 u0 = *reinterpret_cast<const float4*>(src);
                const float4 u1 = *reinterpret_cast<const float4*>(src + 4);
                const float w8[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = w8[e] * inv;
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const float val = (i < n && j0 + e < n) ? A[static_cast<int64_t>(i) * d.ld4 + j0 + e] : 0.0f;
                    v[e] = val * inv;
                }
            }
            split_store8(out, fmt, static_cast<size_t>(bd.row_base + i) * ld + bd.col_base + j0, v);
        }
    }
}

}  // namespace

struct psdgb_batch {
    int precision = 0, schedule = 0, fmt = 0;
    int64_t count = 0, ld = 0, rows = 0, max_iter = 20;
    double tol = 1e-10;
    uint64_t seed = 0x5eed5eedull;
    std::vector<int64_t> n;
    int64_t total_elems = 0;  // sum n^2 (the packed FP64 input)
    // device
    void* dev = nullptr;
    size_t dev_bytes = 0;
    BlockDesc* blocks = nullptr;
    LzBlockDesc* lz = nullptr;
    // Product tile lists.  t128[route][shape][order]: the 128 x 128 tiles
    // (route 1 leaves out the blocks of np = 128, which run on chip; shape 1
    // leaves to the pair tiles every pair of tile rows that lies inside a
    // block of np >= 256, keeping the odd last tile row); tpair[order]: those
    // 256 x 256 pair tiles (shape 1).  order 0: largest blocks first (LPT),
    // 1: block order.
    TileDesc* t128[2][2][2] = {};
    int64_t n128[2][2] = {};
    TileDesc* tpair[2] = {nullptr, nullptr};
    int64_t npair = 0;
    BatchState* states = nullptr;
    float* a32 = nullptr;
    double* vec = nullptr;
    SplitMat A{}, A2{}, A3{};
    int64_t num_tiles = 0;
    int* lz_idx = nullptr;              // block indices grouped by Lanczos size class
    int64_t lz_start[LZ_CLASSES + 1] = {0, 0, 0, 0, 0};
    size_t lz_smem[LZ_CLASSES] = {0, 0, 0, 0};
    // Blocks of n <= 128 (one 128 x 128 tile) with FP16-pair operands can run
    // their whole chain on chip (batch_chain.cu); the grouped products then
    // take only the larger blocks (t128[1], split_tiles[1]).
    bool chain_ok = false;
    ChainBlock* chain = nullptr;
    int* chain_next = nullptr;  // the chain kernel's work counter
    int chain_count = 0;
    int64_t big_count = 0;
    // The splits' 32 x 32 tiles [route]: (block, tile row, tile column) for
    // the tiles meeting each block's n x n corner, every block's (0) or the
    // larger blocks' (1).
    int4* split_tiles[2] = {nullptr, nullptr};
    int64_t num_split_tiles[2] = {0, 0};
    // The FP32 copy's 32 x 32 tiles (block, tile row, tile column).
    int4* copy_tiles = nullptr;
    int64_t num_copy_tiles = 0;
    // The small blocks' bound and chain run on a second stream (high
    // priority), forked from and joined back into the caller's stream.
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // tuning
    int acc_mode = ACC_1X4;
    int order = 0;
    int use_chain = 0;
    int shape = 0;          // 1: pair tiles where they fit (pairs_ok)
    // With the on-chip route, the Lanczos classes from side_from on (2: the
    // blocks of n <= 128; 1: also 128 < n <= 256, the caller's stream then
    // joins the side stream before the larger blocks' products) run on the
    // side stream.
    int side_from = 2;
    // Serpentine: every other product walks its tile lists backwards, so it
    // starts on the blocks whose operands the product before left in L2.
    int serpentine = 0;
    bool pairs_ok = false;
    // psdgb_batch_project_graph: the projection captured once on its own
    // stream and instantiated with the kernels' stream priorities kept, for
    // the blocks pointer and configuration it was captured with.
    cudaStream_t cap = nullptr;
    cudaGraphExec_t gexec = nullptr;
    const double* g_blocks = nullptr;
    bool g_stale = true;
    uint64_t g_kernels = 0;  // kernels in the graph (counted again at each launch)
};

namespace {

psdgb_status batch_enqueue(psdgb_batch* b, double* d_blocks, cudaStream_t s) {
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    if (b->num_copy_tiles > 0) {
        const int64_t warps_needed = b->num_copy_tiles;
        const int64_t ctas = std::min<int64_t>((warps_needed + COPY_THREADS / 32 - 1) / (COPY_THREADS / 32),
                                               16 * static_cast<int64_t>(ds->sm_count));
        batch_to_f32_kernel<<<static_cast<unsigned>(ctas), COPY_THREADS, 0, s>>>(
            b->lz, b->copy_tiles, static_cast<int>(b->num_copy_tiles), d_blocks, b->a32);
    }
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    // With the on-chip route, the blocks of n <= 128 (Lanczos classes 2 and
    // 3, then the chain kernel) go to the side stream and overlap the larger
    // blocks' latency-bound Lanczos launches; the two touch disjoint blocks.
    const bool chain = b->use_chain && b->chain_ok;
    if (chain) {
        PSDGB_CUDA_TRY(cudaEventRecord(b->ev_fork, s));
        PSDGB_CUDA_TRY(cudaStreamWaitEvent(b->side, b->ev_fork, 0));
    }
    const int class_order[LZ_CLASSES] = {1, 2, 3, 0};  // the side stream's classes first
    for (int ci = 0; ci < LZ_CLASSES; ++ci) {
        const int c = class_order[ci];
        const int64_t cnt = b->lz_start[c + 1] - b->lz_start[c];
        if (cnt == 0) continue;
        const int* idx = b->lz_idx + b->lz_start[c];
        const unsigned g = static_cast<unsigned>(cnt);
        const size_t sm = b->lz_smem[c];
        cudaStream_t ls = (chain && c >= b->side_from) ? b->side : s;
        switch (c) {
            case 0: lz_batch_kernel<512><<<g, 512, sm, ls>>>(b->lz, idx, b->a32, b->vec, b->states, b->tol, b->seed,
                                                            PSDGB_RESIDUAL_REFERENCE); break;
            case 1: lz_batch_kernel<256><<<g, 256, sm, ls>>>(b->lz, idx, b->a32, b->vec, b->states, b->tol, b->seed,
                                                            PSDGB_RESIDUAL_REFERENCE); break;
            case 2: lz_batch_kernel<128><<<g, 128, sm, ls>>>(b->lz, idx, b->a32, b->vec, b->states, b->tol, b->seed,
                                                            PSDGB_RESIDUAL_REFERENCE); break;
            default: lz_batch_kernel<64><<<g, 64, sm, ls>>>(b->lz, idx, b->a32, b->vec, b->states, b->tol, b->seed,
                                                           PSDGB_RESIDUAL_REFERENCE); break;
        }
        count_launch();
        PSDGB_CUDA_TRY(cudaGetLastError());
    }
    float coeffs[64];
    const int steps = psdgb_filter_coefficients(b->schedule, coeffs, 21);
    if (chain) {
        // The small blocks' whole filter, on chip; the rest below skips them.
        PSDGB_TRY(launch_batch_chain(ds, b->precision, b->chain, b->chain_count, coeffs, steps, d_blocks,
                                     b->chain_next, 0, b->side));
        PSDGB_CUDA_TRY(cudaEventRecord(b->ev_join, b->side));
        if (b->big_count == 0) {
            PSDGB_CUDA_TRY(cudaStreamWaitEvent(s, b->ev_join, 0));
            return PSDGB_OK;
        }
        // the larger blocks' bound of class 1 ran on the side stream
        if (b->side_from <= 1) PSDGB_CUDA_TRY(cudaStreamWaitEvent(s, b->ev_join, 0));
    }
    // the split's tiles: every block's (route 0) or the larger blocks' (route 1)
    const int4* split_tiles = b->split_tiles[chain ? 1 : 0];
    const int64_t num_split = b->num_split_tiles[chain ? 1 : 0];
    const unsigned split_ctas = static_cast<unsigned>(std::min<int64_t>(
        (num_split + COPY_THREADS / 32 - 1) / (COPY_THREADS / 32), 16 * static_cast<int64_t>(ds->sm_count)));
    if (num_split > 0) {
        batch_split_kernel<<<split_ctas, COPY_THREADS, 0, s>>>(b->lz, b->blocks, b->states, b->a32, b->A, b->fmt,
                                                               b->ld, split_tiles, static_cast<int>(num_split));
        count_launch();
        PSDGB_CUDA_TRY(cudaGetLastError());
    }
    PrecisionInfo pi{};
    precision_info(b->precision, &pi);
    const bool dual_step = pi.nprod == 1;
    const int route = chain ? 1 : 0, shape = (b->shape && b->pairs_ok) ? 1 : 0;
    GroupWork gw{b->t128[route][shape][b->order], b->blocks, 0};
    const int64_t num_tiles = b->n128[route][shape];
    GroupWork gpw{b->tpair[b->order], b->blocks, 0};
    const int64_t num_pairs = shape ? b->npair : 0;
    int nprod = 0;
    // One product over the big blocks: the pair tiles, then the 128 x 128
    // tiles (with the serpentine order, every other product the other way
    // round: its 128 x 128 tiles backwards first, then its pair tiles).
    auto product = [&](const SplitMat& P, const SplitMat& Q, const EpiParams& e) -> psdgb_status {
        const bool back = b->serpentine && (nprod++ & 1);
        gw.reverse = back ? static_cast<int>(num_tiles) : 0;
        gpw.reverse = back ? static_cast<int>(num_pairs) : 0;
        if (back && num_tiles > 0)
            PSDGB_TRY(gemm_tc_group(ds, b->precision, b->acc_mode, P, Q, b->ld, b->rows, e, gw, num_tiles, 0, s));
        if (num_pairs > 0)
            PSDGB_TRY(gemm_tc_pairwide_group(ds, b->precision, P, Q, b->ld, b->rows, e, gpw, num_pairs, s));
        if (!back && num_tiles > 0)
            PSDGB_TRY(gemm_tc_group(ds, b->precision, b->acc_mode, P, Q, b->ld, b->rows, e, gw, num_tiles, 0, s));
        return PSDGB_OK;
    };
    auto base = [&]() {
        EpiParams e{};
        e.fmt = b->fmt;
        e.ld = static_cast<int>(b->ld);
        e.acc_scale = 1.0f;
        e.up = 1.0;
        // Every operand plane was zeroed at plan creation and only zeros are
        // ever written outside the blocks, so the epilogues skip those runs.
        e.skip_pad = 1;
        return e;
    };
    for (int k = 0; k < steps; ++k) {
        EpiParams e1 = base();
        e1.kind = EPI_STORE;
        e1.out = b->A2;
        PSDGB_TRY(product(b->A, b->A, e1));
        EpiParams e2 = base();
        e2.kind = EPI_STORE;
        e2.out = b->A3;
        if (dual_step) {  // one-term precisions: symmetric part, as for a single matrix (composite.cu)
            e2.dual = 1;
            e2.acc_scale = 0.5f;
        }
        PSDGB_TRY(product(b->A2, b->A, e2));
        EpiParams e3 = base();
        e3.kind = EPI_STEP;
        e3.a = coeffs[3 * k];
        e3.b = coeffs[3 * k + 1];
        e3.c = coeffs[3 * k + 2];
        e3.A = b->A;
        e3.A3 = b->A3;
        e3.out = b->A;
        if (dual_step) {
            e3.dual = 1;
            e3.acc_scale = 0.5f;
        }
        PSDGB_TRY(product(b->A3, b->A2, e3));
    }
    if (num_split > 0) {
        batch_split_kernel<<<split_ctas, COPY_THREADS, 0, s>>>(b->lz, b->blocks, b->states, b->a32, b->A2, b->fmt,
                                                               b->ld, split_tiles, static_cast<int>(num_split));  // Xs
        count_launch();
        PSDGB_CUDA_TRY(cudaGetLastError());
    }
    EpiParams ef = base();
    ef.kind = EPI_FINAL;
    ef.dual = 1;
    ef.acc_scale = 0.5f;
    ef.x64 = d_blocks;
    ef.out64 = d_blocks;
    PSDGB_TRY(product(b->A2, b->A, ef));
    if (chain && b->side_from > 1) PSDGB_CUDA_TRY(cudaStreamWaitEvent(s, b->ev_join, 0));
    return PSDGB_OK;
}

}  // namespace

extern "C" {

psdgb_status psdgb_batch_create(const int64_t* sizes, int64_t count, int precision, int schedule,
                                psdgb_batch** out) {
    if (!out || (count > 0 && !sizes) || count < 0 || count > (1 << 24)) {
        set_error("psdgb_batch_create: bad arguments");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    PrecisionInfo pi{};
    if (!precision_info(precision, &pi) || precision == PSDGB_PREC_FP32_SIMT) {
        set_error("psdgb_batch_create: the batch runs the tensor-core precisions");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (precision == PSDGB_PREC_FP8) {
        set_error("psdgb_batch_create: FP8 products run on single matrices only");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (const char* why = schedule_error(precision, schedule)) {
        set_error(why);
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    auto b = new psdgb_batch();
    b->precision = precision;
    b->schedule = schedule;
    b->fmt = pi.fmt;
    b->count = count;
    b->n.assign(sizes, sizes + count);
    int64_t maxnp = 128;
    for (int64_t i = 0; i < count; ++i) {
        if (sizes[i] < 0 || sizes[i] > 4096) {
            delete b;
            set_error("psdgb_batch_create: block sizes must lie in [0, 4096]");
            return PSDGB_ERR_INVALID_ARGUMENT;
        }
        maxnp = std::max<int64_t>(maxnp, up_to(std::max<int64_t>(sizes[i], 1), 128));
    }
    b->ld = maxnp;
    // Shelf packing: blocks sorted by np (largest first); a shelf of height np
    // holds ld / np blocks side by side.
    std::vector<int64_t> order(count);
    std::iota(order.begin(), order.end(), 0);
    auto npof = [&](int64_t i) { return up_to(std::max<int64_t>(b->n[i], 1), 128); };
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t c) { return npof(a) > npof(c); });
    std::vector<BlockDesc> bd(count);
    std::vector<LzBlockDesc> lz(count);
    int64_t row = 0, col = 0, shelf_h = 0;
    for (int64_t idx : order) {
        const int64_t np = npof(idx);
        if (shelf_h != np || col + np > b->ld) {  // new shelf
            row += shelf_h;
            shelf_h = np;
            col = 0;
        }
        bd[idx].row_base = static_cast<int>(row);
        bd[idx].col_base = static_cast<int>(col);
        bd[idx].np = static_cast<int>(np);
        bd[idx].n = static_cast<int>(b->n[idx]);
        col += np;
    }
    b->rows = row + shelf_h;
    int64_t xoff = 0, aoff = 0, voff = 0;
    for (int64_t i = 0; i < count; ++i) {
        const int64_t n = b->n[i], ld4 = up_to(std::max<int64_t>(n, 1), 4);
        const int64_t m = std::min<int64_t>(b->max_iter, n);
        bd[i].x_off = xoff;
        lz[i] = LzBlockDesc{static_cast<int>(n), static_cast<int>(ld4), static_cast<int>(m), 0, aoff, voff, xoff};
        xoff += n * n;
        aoff += up_to(n * ld4, 64);
        voff += up_to(n * m + 8 * (m + 1), 32);
        const int c = lz_class(n);
        b->lz_smem[c] = std::max<size_t>(b->lz_smem[c], 5 * ld4 * sizeof(double) + 2 * ld4 * sizeof(float));
    }
    b->total_elems = xoff;
    // Lanczos launch order: blocks grouped by size class, largest class first.
    std::vector<int> lz_order;
    lz_order.reserve(count);
    for (int c = 0; c < LZ_CLASSES; ++c) {
        b->lz_start[c] = static_cast<int64_t>(lz_order.size());
        for (int64_t i = 0; i < count; ++i)
            if (lz_class(b->n[i]) == c) lz_order.push_back(static_cast<int>(i));
    }
    b->lz_start[LZ_CLASSES] = static_cast<int64_t>(lz_order.size());
    // Tile lists (block order; the LPT order, largest blocks first, is made
    // from it below).  Pair tiles (I, J), J <= I, cover tile rows 2I, 2I + 1
    // of blocks of np >= 256 up to the last even tile row.
    b->pairs_ok = pairwide_supported(precision);
    std::vector<TileDesc> l128[2][2], lpair;
    for (int64_t i = 0; i < count; ++i) {
        const int nt = bd[i].np / 128;
        const int full_rows = (nt >= 2 && b->pairs_ok) ? 2 * (nt / 2) : 0;  // tile rows on pair tiles (shape 1)
        for (int I = 0; I < full_rows / 2; ++I)
            for (int J = 0; J <= I; ++J) lpair.push_back(TileDesc{static_cast<int>(i), I, J, 0});
        for (int route = 0; route < 2; ++route) {
            if (route == 1 && nt == 1) continue;  // on chip
            for (int shape = 0; shape < 2; ++shape)
                for (int bi = (shape ? full_rows : 0); bi < nt; ++bi)
                    for (int bj = 0; bj <= bi; ++bj) l128[route][shape].push_back(TileDesc{static_cast<int>(i), bi, bj, 0});
        }
    }
    if (lpair.empty()) b->pairs_ok = false;
    b->shape = 0;  // 128 x 128 tiles until the autotuner or the caller picks pair tiles
    auto lpt = [&](std::vector<TileDesc> v) {
        std::stable_sort(v.begin(), v.end(),
                         [&](const TileDesc& a, const TileDesc& c) { return bd[a.block].np > bd[c.block].np; });
        return v;
    };
    b->num_tiles = static_cast<int64_t>(l128[0][0].size());
    b->npair = static_cast<int64_t>(lpair.size());
    // Small blocks (one 128 x 128 tile, n >= 1) for the on-chip chain with
    // FP16-pair operands; the larger blocks' tile lists and split list.
    b->chain_ok = precision == PSDGB_PREC_FP16X3 || precision == PSDGB_PREC_FP16;
    std::vector<int> chain_idx, big_idx;
    for (int64_t i = 0; i < count; ++i) {
        if (b->chain_ok && bd[i].np == 128 && b->n[i] >= 1)
            chain_idx.push_back(static_cast<int>(i));
        else if (b->n[i] >= 1 || !b->chain_ok)
            big_idx.push_back(static_cast<int>(i));
    }
    if (chain_idx.empty()) b->chain_ok = false;
    // the chain kernel claims blocks in list order: largest first
    std::stable_sort(chain_idx.begin(), chain_idx.end(), [&](int a, int c) { return b->n[a] > b->n[c]; });
    b->chain_count = static_cast<int>(chain_idx.size());
    b->big_count = static_cast<int64_t>(big_idx.size());
    b->use_chain = b->chain_ok ? 1 : 0;
    // Device memory: tables | states | FP32 copies | Lanczos vectors | operand planes.
    const size_t plane = static_cast<size_t>(b->rows) * b->ld * 2;
    const int nterms = format_terms(b->fmt);
    auto a256 = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t sz_blocks = a256(sizeof(BlockDesc) * std::max<int64_t>(count, 1));
    const size_t sz_lz = a256(sizeof(LzBlockDesc) * std::max<int64_t>(count, 1));
    // every tile list, both orders, one after the other
    size_t tile_entries = 2 * lpair.size();
    for (int r = 0; r < 2; ++r)
        for (int sh = 0; sh < 2; ++sh) tile_entries += 2 * l128[r][sh].size();
    const size_t sz_tiles = a256(sizeof(TileDesc) * std::max<size_t>(tile_entries, 1));
    const size_t sz_states = a256(sizeof(BatchState) * std::max<int64_t>(count, 1));
    const size_t sz_idx = a256(sizeof(int) * std::max<int64_t>(count, 1));
    const size_t sz_a32 = a256(sizeof(float) * std::max<int64_t>(aoff, 1));
    const size_t sz_vec = a256(sizeof(double) * std::max<int64_t>(voff, 1));
    const size_t sz_ops = 3 * nterms * a256(plane);
    const size_t sz_chain = a256(sizeof(ChainBlock) * std::max<size_t>(chain_idx.size(), 1)) + 256;
    std::vector<int4> split_list[2];
    for (int route = 0; route < 2; ++route) {
        auto add = [&](int64_t i) {
            const int64_t nt = (b->n[i] + 31) / 32;
            for (int64_t ti = 0; ti < nt; ++ti)
                for (int64_t tj = 0; tj < nt; ++tj)
                    split_list[route].push_back(make_int4(static_cast<int>(i), static_cast<int>(ti),
                                                          static_cast<int>(tj), 0));
        };
        if (route == 0)
            for (int64_t i = 0; i < count; ++i) add(i);
        else
            for (int i : big_idx) add(i);
        b->num_split_tiles[route] = static_cast<int64_t>(split_list[route].size());
    }
    const size_t sz_big_idx = a256(sizeof(int4) * std::max<size_t>(split_list[0].size(), 1)) +
                              a256(sizeof(int4) * std::max<size_t>(split_list[1].size(), 1));
    std::vector<int4> copy_list;
    for (int64_t i = 0; i < count; ++i) {
        const int64_t n = b->n[i], ld4 = lz[i].ld4;
        for (int64_t ti = 0; ti < (n + 31) / 32; ++ti)
            for (int64_t tj = 0; tj < (ld4 + 31) / 32; ++tj)
                copy_list.push_back(make_int4(static_cast<int>(i), static_cast<int>(ti), static_cast<int>(tj), 0));
    }
    b->num_copy_tiles = static_cast<int64_t>(copy_list.size());
    const size_t sz_copy = a256(sizeof(int4) * std::max<size_t>(copy_list.size(), 1));
    b->dev_bytes = sz_blocks + sz_lz + sz_idx + sz_tiles + sz_states + sz_a32 + sz_vec + sz_chain + sz_big_idx +
                   sz_copy + sz_ops;
    cudaError_t e = cudaMalloc(&b->dev, b->dev_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete b;
        set_error("psdgb_batch_create: device allocation failed");
        return PSDGB_ERR_OUT_OF_MEMORY;
    }
    // From here on a failing call frees the plan (memory, stream, events).
    struct PlanGuard {
        psdgb_batch* b;
        ~PlanGuard() {
            if (b) psdgb_batch_destroy(b);
        }
    } guard{b};
    char* p = static_cast<char*>(b->dev);
    b->blocks = reinterpret_cast<BlockDesc*>(p);
    p += sz_blocks;
    b->lz = reinterpret_cast<LzBlockDesc*>(p);
    p += sz_lz;
    b->lz_idx = reinterpret_cast<int*>(p);
    p += sz_idx;
    TileDesc* tile_store = reinterpret_cast<TileDesc*>(p);
    p += sz_tiles;
    b->states = reinterpret_cast<BatchState*>(p);
    p += sz_states;
    b->a32 = reinterpret_cast<float*>(p);
    p += sz_a32;
    b->vec = reinterpret_cast<double*>(p);
    p += sz_vec;
    b->chain = reinterpret_cast<ChainBlock*>(p);
    b->chain_next = reinterpret_cast<int*>(p + sz_chain - 256);
    p += sz_chain;
    b->split_tiles[0] = reinterpret_cast<int4*>(p);
    b->split_tiles[1] = reinterpret_cast<int4*>(p + a256(sizeof(int4) * std::max<size_t>(split_list[0].size(), 1)));
    p += sz_big_idx;
    b->copy_tiles = reinterpret_cast<int4*>(p);
    p += sz_copy;
    SplitMat* mats[3] = {&b->A, &b->A2, &b->A3};
    for (int mi = 0; mi < 3; ++mi)
        for (int t = 0; t < 3; ++t) {
            mats[mi]->term[t] = (t < nterms) ? p : nullptr;
            if (t < nterms) p += a256(plane);
        }
    for (int64_t i = 0; i < count; ++i) bd[i].up_dev = &b->states[i].scale;
    if (count > 0) {
        PSDGB_CUDA_TRY(cudaMemcpy(b->blocks, bd.data(), sizeof(BlockDesc) * count, cudaMemcpyHostToDevice));
        PSDGB_CUDA_TRY(cudaMemcpy(b->lz, lz.data(), sizeof(LzBlockDesc) * count, cudaMemcpyHostToDevice));
        PSDGB_CUDA_TRY(cudaMemcpy(b->lz_idx, lz_order.data(), sizeof(int) * count, cudaMemcpyHostToDevice));
    }
    {
        std::vector<TileDesc> all;
        all.reserve(tile_entries);
        auto place = [&](const std::vector<TileDesc>& v, TileDesc** out) {
            const std::vector<TileDesc> l = lpt(v);
            out[0] = tile_store + all.size();
            all.insert(all.end(), l.begin(), l.end());
            out[1] = tile_store + all.size();
            all.insert(all.end(), v.begin(), v.end());
        };
        for (int r = 0; r < 2; ++r)
            for (int sh = 0; sh < 2; ++sh) {
                place(l128[r][sh], b->t128[r][sh]);
                b->n128[r][sh] = static_cast<int64_t>(l128[r][sh].size());
            }
        place(lpair, b->tpair);
        if (!all.empty())
            PSDGB_CUDA_TRY(cudaMemcpy(tile_store, all.data(), sizeof(TileDesc) * all.size(), cudaMemcpyHostToDevice));
    }
    for (int route = 0; route < 2; ++route)
        if (!split_list[route].empty())
            PSDGB_CUDA_TRY(cudaMemcpy(b->split_tiles[route], split_list[route].data(),
                                      sizeof(int4) * split_list[route].size(), cudaMemcpyHostToDevice));
    if (!copy_list.empty())
        PSDGB_CUDA_TRY(cudaMemcpy(b->copy_tiles, copy_list.data(), sizeof(int4) * copy_list.size(),
                                  cudaMemcpyHostToDevice));
    if (b->chain_ok) {
        int least = 0, greatest = 0;
        PSDGB_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        PSDGB_CUDA_TRY(cudaStreamCreateWithPriority(&b->side, cudaStreamNonBlocking, greatest));
        PSDGB_CUDA_TRY(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
        PSDGB_CUDA_TRY(cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming));
    }
    if (!chain_idx.empty()) {
        std::vector<ChainBlock> cbs;
        for (int i : chain_idx)
            cbs.push_back(ChainBlock{b->a32 + lz[i].a32_off, lz[i].ld4, lz[i].n, lz[i].x_off, &b->states[i].scale,
                                     &b->states[i].inv_scale});
        PSDGB_CUDA_TRY(cudaMemcpy(b->chain, cbs.data(), sizeof(ChainBlock) * cbs.size(), cudaMemcpyHostToDevice));
    }
    // Padding rows/columns between blocks are never read; zero the planes once
    // so every TMA box reads finite values.
    PSDGB_CUDA_TRY(cudaMemset(b->A.term[0], 0, sz_ops));
    // Only the 512-thread class holds blocks large enough (n > 256) to need
    // more than 48 KB of dynamic shared memory.
    if (b->lz_smem[0] > 48 * 1024)
        PSDGB_CUDA_TRY(cudaFuncSetAttribute(lz_batch_kernel<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            static_cast<int>(b->lz_smem[0])));
    guard.b = nullptr;
    *out = b;
    return PSDGB_OK;
}

psdgb_status psdgb_batch_destroy(psdgb_batch* b) {
    if (!b) return PSDGB_OK;
    cudaDeviceSynchronize();
    if (b->dev) cudaFree(b->dev);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->cap) cudaStreamDestroy(b->cap);
    delete b;
    return PSDGB_OK;
}

psdgb_status psdgb_batch_info(const psdgb_batch* b, int64_t* total_elements, size_t* device_bytes,
                              int64_t* num_tiles, int* acc_mode, int* tile_order) {
    if (!b) return PSDGB_ERR_INVALID_ARGUMENT;
    if (total_elements) *total_elements = b->total_elems;
    if (device_bytes) *device_bytes = b->dev_bytes;
    if (num_tiles) *num_tiles = b->num_tiles;
    if (acc_mode) *acc_mode = b->acc_mode;
    if (tile_order) *tile_order = b->order;
    return PSDGB_OK;
}

psdgb_status psdgb_batch_project(psdgb_batch* b, double* d_blocks, void* stream) {
    if (!b || (b->total_elems > 0 && !d_blocks)) {
        set_error("psdgb_batch_project: bad arguments");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (b->count == 0) return PSDGB_OK;
    return batch_enqueue(b, d_blocks, static_cast<cudaStream_t>(stream));
}

psdgb_status psdgb_batch_project_graph(psdgb_batch* b, double* d_blocks, void* stream) {
    if (!b || (b->total_elems > 0 && !d_blocks)) {
        set_error("psdgb_batch_project_graph: bad arguments");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (b->count == 0) return PSDGB_OK;
    if (!b->gexec || b->g_stale || b->g_blocks != d_blocks) {
        if (b->gexec) {
            PSDGB_CUDA_TRY(cudaGraphExecDestroy(b->gexec));
            b->gexec = nullptr;
        }
        if (!b->cap) PSDGB_CUDA_TRY(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
        PSDGB_CUDA_TRY(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
        const uint64_t k0 = psdgb_kernel_launch_count();
        const psdgb_status st = batch_enqueue(b, d_blocks, b->cap);
        b->g_kernels = psdgb_kernel_launch_count() - k0;
        count_launch(0 - b->g_kernels);  // captured, not run: counted at each launch below
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(b->cap, &g);  // always ends the capture
        if (st != PSDGB_OK || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (st != PSDGB_OK) return st;
            set_error(cudaGetErrorString(ce));
            return PSDGB_ERR_CUDA;
        }
        // Node priorities: the small blocks' kernels keep the side stream's
        // high priority inside the graph (by default a graph runs every
        // kernel at the priority of the stream it is launched into).
        const cudaError_t ie = cudaGraphInstantiateWithFlags(&b->gexec, g, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            b->gexec = nullptr;
            set_error(cudaGetErrorString(ie));
            return PSDGB_ERR_CUDA;
        }
        b->g_blocks = d_blocks;
        b->g_stale = false;
    }
    PSDGB_CUDA_TRY(cudaGraphLaunch(b->gexec, static_cast<cudaStream_t>(stream)));
    count_launch(b->g_kernels);
    return PSDGB_OK;
}

psdgb_status psdgb_batch_configure(psdgb_batch* b, int acc_mode, int tile_order, int small_on_chip,
                                   int pair_tiles, int serpentine) {
    if (!b || acc_mode < -1 || acc_mode > ACC_1X4 || tile_order < -1 || tile_order > 1 || small_on_chip < -1 ||
        small_on_chip > 1 || pair_tiles < -1 || pair_tiles > 1 || serpentine < -1 || serpentine > 1) {
        set_error("psdgb_batch_configure: bad arguments");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (small_on_chip == 1 && !b->chain_ok) {
        set_error("psdgb_batch_configure: no blocks of n <= 128 with FP16 / FP16x3 operands to run on chip");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (pair_tiles == 1 && !b->pairs_ok) {
        set_error("psdgb_batch_configure: no blocks of n > 128 for 256 x 256 pair tiles at this precision");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (acc_mode >= 0) b->acc_mode = acc_mode;
    if (tile_order >= 0) b->order = tile_order;
    if (small_on_chip >= 0) b->use_chain = small_on_chip;
    if (pair_tiles >= 0) b->shape = pair_tiles;
    if (serpentine >= 0) b->serpentine = serpentine;
    b->g_stale = true;
    return PSDGB_OK;
}

psdgb_status psdgb_batch_tuning(const psdgb_batch* b, int* acc_mode, int* tile_order, int* small_on_chip,
                                int64_t* small_blocks, int* pair_tiles, int64_t* num_pair_tiles, int* serpentine) {
    if (!b) {
        set_error("psdgb_batch_tuning: null batch");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (acc_mode) *acc_mode = b->acc_mode;
    if (tile_order) *tile_order = b->order;
    if (small_on_chip) *small_on_chip = b->use_chain && b->chain_ok ? 1 : 0;
    if (small_blocks) *small_blocks = b->chain_ok ? b->chain_count : 0;
    if (pair_tiles) *pair_tiles = b->shape && b->pairs_ok ? 1 : 0;
    if (num_pair_tiles) *num_pair_tiles = b->pairs_ok ? b->npair : 0;
    if (serpentine) *serpentine = b->serpentine;
    return PSDGB_OK;
}

psdgb_status psdgb_batch_autotune(psdgb_batch* b, double* d_scratch_blocks, void* stream, double* best_ms) {
    if (!b || (b->total_elems > 0 && !d_scratch_blocks)) {
        set_error("psdgb_batch_autotune: bad arguments");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    if (b->count == 0) return PSDGB_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    PSDGB_CUDA_TRY(cudaEventCreate(&e0));
    PSDGB_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_acc = b->acc_mode, best_order = b->order, best_chain = b->use_chain, best_shape = b->shape,
        best_side = b->side_from;
    const int accs[3] = {ACC_1X4, ACC_2X2, ACC_4X1};
    // Every combination of: tile shape (128 x 128; pair tiles where
    // available), small-block route (per product; on chip with the side
    // stream taking the bound of n <= 128, or of n <= 256), accumulator
    // configuration (3) and tile order (LPT, block order).  The serpentine
    // order is left as configured (it measured no faster on the 4096-block
    // configuration and would double the trials).
    const int nsh = b->pairs_ok ? 2 : 1, nrt = b->chain_ok ? 3 : 1;
    for (int cfg = 0; cfg < nsh * nrt * 3 * 2; ++cfg) {
        int c = cfg;
        const int o = c % 2;
        c /= 2;
        const int ai = c % 3;
        c /= 3;
        const int rt = c % nrt;
        c /= nrt;
        const int sh = c % nsh;
        b->acc_mode = accs[ai];
        b->order = o;
        b->use_chain = rt > 0 ? 1 : 0;
        b->side_from = rt == 2 ? 1 : 2;
        b->shape = sh;
        PSDGB_TRY(batch_enqueue(b, d_scratch_blocks, s));  // warm (and leaves valid operands)
        PSDGB_CUDA_TRY(cudaEventRecord(e0, s));
        PSDGB_TRY(batch_enqueue(b, d_scratch_blocks, s));
        PSDGB_CUDA_TRY(cudaEventRecord(e1, s));
        PSDGB_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        PSDGB_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            best_acc = accs[ai];
            best_order = o;
            best_chain = b->use_chain;
            best_side = b->side_from;
            best_shape = sh;
        }
    }
    b->acc_mode = best_acc;
    b->order = best_order;
    b->use_chain = best_chain;
    b->side_from = best_side;
    b->shape = best_shape;
    b->g_stale = true;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_ms) *best_ms = best;
    DeviceState* ds = nullptr;
    PSDGB_TRY(device_state(&ds));
    return finish(ds, s);
}

}  // extern "C"
