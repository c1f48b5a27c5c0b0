// batch_chain.cu — the whole filter of a block-diagonal batch's small blocks
// (n <= 128, padded to one 128 x 128 tile) in one persistent launch, every
// operand resident in shared memory.
//
// In the grouped products (gemm_tc.cu) every product of every block reads its
// operands from and writes its result to global memory, and a batch's
// operands (3 split matrices of all blocks, about 3 GB for 4096 blocks) are
// far larger than L2: each product streams them from DRAM.  A block of
// n <= 128 is a single 128 x 128 tile, and its three FP16-pair split matrices
// (A, A2, A3: 3 x 64 KB) fit in one CTA's shared memory, so one CTA can run
// all of that block's products — the reference's per-step Sgemm / Sscal /
// Saxpy / symmetrisation sequence (src/composite_FP32.cu:103-118, its FP16
// twin src/composite_FP16.cu:118-166) and the final X (I + A) / 2
// (src/composite_FP32.cu:142-156) — without touching global memory between
// products:
//
//   load      A = split(a32 x 1/up) from the block's FP32 copy (the bound ran
//             before, lz_batch_kernel in batch.cu)
//   per step  A2 = A A; A3 = A2 A; A = a A + b A3 + c A3 A2   (tcgen05.mma from
//             shared memory into TMEM, the epilogue writes the next operand
//             straight back into shared memory)
//   final     Xs = split(X x 1/up), out = (X + up (Xs A + A Xs)/2) / 2
//             written to the caller's block in place.  The FP32 copy holds
//             exactly the FP32 narrowing of the symmetric matrix that X's
//             upper triangle defines (batch_to_f32_kernel), so Xs is split
//             from it again, as the first A was.
//
// The arithmetic is that of the grouped path with one TMEM accumulator
// (ACC_1X4): the same MMA order (K blocks, then K slices, then term
// products), the same K-block count (one for n <= 64), the same epilogue
// formulas (the lower triangle computed, the upper one its mirror), the same
// split, so a block's result is the same bit for bit.
//
// Shared memory: each split matrix is two planes (FP16 hi, lo) of two K
// blocks, each a 128-row x 128-byte tile in the layout TMA writes with the
// 128-byte swizzle (16-byte chunk c of row r at chunk c ^ (r & 7)), which is
// what the K-major shared-memory descriptors of the MMAs read.  Everything
// outside a block's n x n corner is zero: the split writes zeros there, A2
// and A3 are cleared when a block starts, and the epilogues skip the 32 x 32
// runs that lie wholly outside the first nr = 32 ceil(n / 32) rows (their
// values would be zero).
//
// Epilogue: 8 warps; warp w reads TMEM lanes 32 (w % 4) .. + 31 (the rows of
// its lane quarter) and takes every other 32 x 32 run of that row band's
// lower triangle.  Runs are read from TMEM as 16 x 256-bit fragments (thread
// t holds rows t / 4 and t / 4 + 8, columns 2 (t % 4) and + 1 of each 8 x 8
// matrix), the layout ldmatrix / stmatrix use: the step epilogue's A and A3
// come in with ldmatrix, each 8 x 8 matrix of results goes out with one
// stmatrix per plane and its mirror with one stmatrix .trans.  Diagonal 8 x 8
// matrices take their upper half from their lower half (warp shuffles);
// matrices above the diagonal are not stored (their mirror is).  Thread 0
// issues the MMAs.  One CTA per SM (199 KB of shared memory), persistent over
// the list of small blocks (claimed from a counter, largest first), each
// block's inputs prefetched into L2 one block ahead; every wait is bounded.
#include <cuda.h>

#include "convert.h"
#include "tc_kernel.cuh"

namespace psdgb {

namespace {

constexpr int CH_THREADS = 256;
constexpr int CH_WARPS = CH_THREADS / 32;
constexpr int CH_TILE = 128 * 128;                 // bytes of one plane's K block (128 rows x 128 B)
constexpr int CH_MAT = 2 * 2 * CH_TILE;            // two planes x two K blocks: 64 KB
constexpr int CH_DUMMY = CH_WARPS * 128;           // per-warp target of the stores that are skipped
constexpr int CH_SMEM = 3 * CH_MAT + CH_DUMMY + 1024 + 256;  // A, A2, A3, dummy rows, alignment, barriers
constexpr uint32_t CH_IDESC_F16 = idesc_f16(128, 128, false);

// Byte offset of the 16-byte chunk holding elements (r, k .. k + 7), k a
// multiple of 8, in the hi plane of a split matrix (the lo plane is
// 2 CH_TILE further).
__device__ __forceinline__ uint32_t ch_chunk(int r, int k) {
    const int kb = k >> 6, kk = k & 63;
    return static_cast<uint32_t>(kb * CH_TILE + r * 128 + (((kk >> 3) ^ (r & 7)) << 4));
}

// The FP16 pair of v (split_store's arithmetic for FMT_F16: hi / lo of v * 2^12).
__device__ __forceinline__ void ch_split(float v, __half& h, __half& l) {
    const float x = v * kF16Scale;
    h = __float2half_rn(x);
    l = __float2half_rn(x - __half2float(h));
}

__device__ __forceinline__ uint32_t pack2(__half a, __half b) {
    return static_cast<uint32_t>(__half_as_ushort(a)) | (static_cast<uint32_t>(__half_as_ushort(b)) << 16);
}

// A stored value from its hi / lo halves (load_run8's arithmetic: lo + hi, then 2^-12).
__device__ __forceinline__ float ch_value(uint32_t h, uint32_t l) {
    const __half hh = __ushort_as_half(static_cast<unsigned short>(h & 0xFFFFu));
    const __half ll = __ushort_as_half(static_cast<unsigned short>(l & 0xFFFFu));
    return ((0.f + __half2float(ll)) + __half2float(hh)) * kF16Unscale;
}

__device__ __forceinline__ void stmatrix4(uint32_t addr, const uint32_t (&r)[4]) {
    asm volatile("stmatrix.sync.aligned.m8n8.x4.shared.b16 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(r[0]),
                 "r"(r[1]), "r"(r[2]), "r"(r[3])
                 : "memory");
}
__device__ __forceinline__ void stmatrix4_trans(uint32_t addr, const uint32_t (&r)[4]) {
    asm volatile("stmatrix.sync.aligned.m8n8.x4.trans.shared.b16 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(r[0]),
                 "r"(r[1]), "r"(r[2]), "r"(r[3])
                 : "memory");
}
__device__ __forceinline__ void ldmatrix4(uint32_t addr, uint32_t (&r)[4]) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr)
                 : "memory");
}

// A 32 x 32 run of the accumulator: lanes lane0 .. lane0 + 31, columns col
// .. col + 31, as two 16-lane halves h: v[h][4 cb + 2 rg + e] = element
// (lane0 + 16 h + t / 4 + 8 rg, col + 8 cb + 2 (t % 4) + e) for thread t.
__device__ __forceinline__ void tmem_ld_run(uint32_t taddr, float (&v)[2][16]) {
    uint32_t r[32];
    __syncwarp();  // .sync.aligned: the whole warp, converged
    asm volatile(
        "tcgen05.ld.sync.aligned.16x256b.x4.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%32];\n\t"
        "tcgen05.ld.sync.aligned.16x256b.x4.b32 "
        "{%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%33];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr), "r"(taddr + (16u << 16))
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        v[0][i] = __uint_as_float(r[i]);
        v[1][i] = __uint_as_float(r[16 + i]);
    }
}

// The MMAs of C = P Q (kbh K blocks of 64; a dual product also adds Q P^T
// with K doubled), issued by one thread into the accumulator at tmem, in the
// grouped kernel's order: K blocks, K slices of 16, term products.  Like the
// grouped kernel (tile_kblocks), a block of n <= 64 reads one K block: the
// second is zero.
template <int NPROD>
__device__ __forceinline__ void ch_mma(uint32_t tmem, uint32_t P, uint32_t Q, bool dual, int kbh) {
    const int kbs = dual ? 2 * kbh : kbh;
    for (int kb = 0; kb < kbs; ++kb) {
        const bool second = kb >= kbh;
        const int kk = second ? kb - kbh : kb;
        const uint32_t a = (second ? Q : P) + static_cast<uint32_t>(kk * CH_TILE);
        const uint32_t b = (second ? P : Q) + static_cast<uint32_t>(kk * CH_TILE);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
#pragma unroll
            for (int pi = 0; pi < NPROD; ++pi) {
                const uint64_t ad = sdesc_kmajor_sw128(a + static_cast<uint32_t>(prod_a(pi) * 2 * CH_TILE + k * 32));
                const uint64_t bd = sdesc_kmajor_sw128(b + static_cast<uint32_t>(prod_b(pi) * 2 * CH_TILE + k * 32));
                umma_f16(tmem, ad, bd, CH_IDESC_F16, (kb != 0 || k != 0 || pi != 0) ? 1u : 0u);
            }
        }
    }
}

enum ChEpi : int { CH_STORE = 0, CH_STEP = 1, CH_FINAL = 2 };

struct ChainParams {
    const ChainBlock* blocks;
    int count;
    float coef[3 * 16];  // per step: a, b, c (after the safety scaling)
    int steps;
    int dual_steps;      // one-term products: the second and third products of a step take the symmetric part
    double* x;           // the batch's packed FP64 blocks (input, and output in place)
    int* next;           // work counter (zero at launch): CTAs claim blocks in list order
    int* err;
};

// Split matrix m = split(a32 x inv) for the block: the FP32 copy (n rows of
// ld4 floats, ld4 a multiple of 4, rows 16-byte aligned), zero outside
// n x n.  Warp w takes rows w, w + 8, ...; lane l columns 4 l .. 4 l + 3.
__device__ __forceinline__ void ch_split_from_f32(uint8_t* m, const ChainBlock& cb, float inv) {
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int n = cb.n, c0 = 4 * lane;
#pragma unroll 4
    for (int r = warp; r < 128; r += CH_WARPS) {
        float w[4] = {0.f, 0.f, 0.f, 0.f};
        if (r < n) {
            const float* src = cb.a32 + static_cast<int64_t>(r) * cb.ld4 + c0;
            if (c0 + 4 <= n) {
                const float4 u = *reinterpret_cast<const float4*>(src);
                w[0] = u.x;
                w[1] = u.y;
                w[2] = u.z;
                w[3] = u.w;
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (c0 + e < n) w[e] = src[e];
            }
        }
        __half h[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) ch_split(w[e] * inv, h[e], l[e]);
        const uint32_t off = ch_chunk(r, c0 & ~7) + ((c0 & 7) << 1);
        *reinterpret_cast<uint2*>(m + off) = make_uint2(pack2(h[0], h[1]), pack2(h[2], h[3]));
        *reinterpret_cast<uint2*>(m + off + 2 * CH_TILE) = make_uint2(pack2(l[0], l[1]), pack2(l[2], l[3]));
    }
}

__device__ __forceinline__ void ch_zero(uint8_t* m) {
    for (int i = threadIdx.x; i < CH_MAT / 16; i += CH_THREADS) reinterpret_cast<uint4*>(m)[i] = make_uint4(0, 0, 0, 0);
}

// The epilogue of one product: each warp's runs of the lower triangle from
// TMEM (rows below nr only), combined (CH_STEP: a A + b A3 + c acc) and
// stored with their mirrors into `out` (CH_STORE / CH_STEP), or
// reconstructed into the caller's FP64 block (CH_FINAL).
__device__ __forceinline__ void ch_epilogue(int kind, float acc_scale, float a, float b, float c, uint8_t* out,
                                            const uint8_t* Am, const uint8_t* A3m, uint8_t* dummy, uint32_t tmem,
                                            const ChainBlock& cb, int nr, double* x) {
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int qd = warp & 3, half = warp >> 2;
    const int p0 = 32 * qd;
    if (p0 >= nr) return;                           // rows of padding only (warp-uniform)
    const int g = lane / 4, cq = 2 * (lane % 4);  // fragment row and first column within an 8 x 8 matrix
    const int mi = lane / 8, mr = lane % 8;      // stmatrix / ldmatrix: matrix and row this lane addresses
    const uint32_t out_s = out ? smem_u32(out) : 0u, a_s = smem_u32(Am), a3_s = smem_u32(A3m);
    const uint32_t dummy_s = smem_u32(dummy) + static_cast<uint32_t>(warp * 128 + mr * 16);
    for (int j = half; j <= qd; j += 2) {
        const int q0 = 32 * j;
        const bool diag = q0 == p0;
        float v[2][16];
        tmem_ld_run(tmem + (static_cast<uint32_t>(p0) << 16) + static_cast<uint32_t>(q0), v);
        if (kind == CH_FINAL) {
            const int n = cb.n;
            const double up = *cb.scale;
            double* X = x + cb.x_off;
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int p = p0 + 16 * h + g + 8 * ((i >> 1) & 1);
                    const int q = q0 + 8 * (i >> 2) + cq + (i & 1);
                    if (q <= p && p < n) {
                        const double o = 0.5 * (X[static_cast<int64_t>(p) * n + q] +
                                                up * static_cast<double>(acc_scale * v[h][i]));
                        X[static_cast<int64_t>(p) * n + q] = o;
                        if (q != p) X[static_cast<int64_t>(q) * n + p] = o;
                    }
                }
            continue;
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            float* w = v[h];
#pragma unroll
            for (int i = 0; i < 16; ++i) w[i] *= acc_scale;
            const int rbase = p0 + 16 * h;  // first row of this half
            if (kind == CH_STEP) {
#pragma unroll
                for (int rg = 0; rg < 2; ++rg) {
                    // matrices (rg, cb = 0..3): rows rbase + 8 rg .., columns q0 + 8 cb ..
                    const uint32_t off = ch_chunk(rbase + 8 * rg + mr, q0 + 8 * mi);
                    uint32_t ah[4], al[4], bh[4], bl[4];
                    ldmatrix4(a_s + off, ah);
                    ldmatrix4(a_s + off + 2 * CH_TILE, al);
                    ldmatrix4(a3_s + off, bh);
                    ldmatrix4(a3_s + off + 2 * CH_TILE, bl);
#pragma unroll
                    for (int cbk = 0; cbk < 4; ++cbk)
#pragma unroll
                        for (int e = 0; e < 2; ++e) {
                            const int sh = 16 * e;
                            const float av = ch_value(ah[cbk] >> sh, al[cbk] >> sh);
                            const float a3 = ch_value(bh[cbk] >> sh, bl[cbk] >> sh);
                            float& y = w[4 * cbk + 2 * rg + e];
                            y = fmaf(c, y, fmaf(b, a3, a * av));
                        }
                }
            }
            if (diag) {
                // Diagonal 8 x 8 matrices (cb == 2 h + rg): the upper half
                // takes the lower half's values, element (r, c) <- (c, r).
#pragma unroll
                for (int rg = 0; rg < 2; ++rg) {
                    const int i0 = 4 * (2 * h + rg) + 2 * rg;
                    const float s00 = __shfl_sync(0xffffffffu, w[i0], 4 * cq + (g >> 1));
                    const float s01 = __shfl_sync(0xffffffffu, w[i0 + 1], 4 * cq + (g >> 1));
                    const float s10 = __shfl_sync(0xffffffffu, w[i0], 4 * (cq + 1) + (g >> 1));
                    const float s11 = __shfl_sync(0xffffffffu, w[i0 + 1], 4 * (cq + 1) + (g >> 1));
                    if (cq > g) w[i0] = (g & 1) ? s01 : s00;
                    if (cq + 1 > g) w[i0 + 1] = (g & 1) ? s11 : s10;
                }
            }
#pragma unroll
            for (int rg = 0; rg < 2; ++rg) {
                uint32_t hi[4], lo[4];
#pragma unroll
                for (int cbk = 0; cbk < 4; ++cbk) {
                    __half h0, l0, h1, l1;
                    ch_split(w[4 * cbk + 2 * rg], h0, l0);
                    ch_split(w[4 * cbk + 2 * rg + 1], h1, l1);
                    hi[cbk] = pack2(h0, h1);
                    lo[cbk] = pack2(l0, l1);
                }
                const int R0 = rbase + 8 * rg;  // rows of matrices (rg, *)
                const int bi = (R0 - p0) >> 3;  // its 8-row block within the run
                // rows: matrix mi at rows R0 .., columns q0 + 8 mi ..; above the diagonal: skipped
                const bool row_ok = !diag || mi <= bi;
                const uint32_t ra = out_s + ch_chunk(R0 + mr, q0 + 8 * mi);
                stmatrix4(row_ok ? ra : dummy_s, hi);
                stmatrix4(row_ok ? ra + 2 * CH_TILE : dummy_s, lo);
                // mirrors: matrix mi transposed at rows q0 + 8 mi .., columns R0 ..; strictly below the diagonal
                const bool mir_ok = !diag || mi < bi;
                const uint32_t ma = out_s + ch_chunk(q0 + 8 * mi + mr, R0);
                stmatrix4_trans(mir_ok ? ma : dummy_s, hi);
                stmatrix4_trans(mir_ok ? ma + 2 * CH_TILE : dummy_s, lo);
            }
        }
    }
}

template <int NPROD>
__global__ void __launch_bounds__(CH_THREADS, 1) batch_chain_kernel(const __grid_constant__ ChainParams cp) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw_addr = smem_u32(smem_raw);
    uint8_t* smem = smem_raw + ((1024u - (raw_addr & 1023u)) & 1023u);
    uint8_t* mA = smem;
    uint8_t* mA2 = smem + CH_MAT;
    uint8_t* mA3 = smem + 2 * CH_MAT;
    uint8_t* dummy = smem + 3 * CH_MAT;
    uint64_t* bar = reinterpret_cast<uint64_t*>(dummy + CH_DUMMY);
    uint64_t* drain = bar + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    volatile int* claim = abort_flag + 1;  // [0] the block being run, [1] the next one (thread 0)
    const int warp = threadIdx.x / 32;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_init(drain, 1);
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, 128);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t sA = smem_u32(mA), sA2 = smem_u32(mA2), sA3 = smem_u32(mA3);
    uint32_t phase = 0;
    bool stop = false;
    int kbh = 2;
    // One product: MMAs by thread 0, then every thread waits for them (bounded).
    auto product = [&](uint32_t P, uint32_t Q, bool dual) {
        if (threadIdx.x == 0) {
            tc_fence_after();
            ch_mma<NPROD>(tmem, P, Q, dual, kbh);
            umma_commit(bar);
        }
        if (!mbar_wait_warp(bar, phase)) {  // warp-uniform: TMEM loads follow
            *abort_flag = 1;
            atomicCAS(cp.err, 0, DEVERR_EPI_WAIT);
        }
        phase ^= 1u;
        tc_fence_after();
    };
    // Shared-memory operands written by the threads become visible to the MMAs
    // (async proxy); TMEM reads finish before the next MMAs overwrite it.
    auto operands_ready = [&]() {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
    };
    // Bring a block's FP32 copy and FP64 input into L2 ahead of its turn
    // (16-byte-aligned interiors; the bulk prefetch reads nothing else).
    auto prefetch = [&](int bi) {
        if (threadIdx.x != 0 || bi >= cp.count) return;
        const ChainBlock nb = cp.blocks[bi];
        const uint32_t abytes = static_cast<uint32_t>(nb.n) * static_cast<uint32_t>(nb.ld4) * 4u;
        const uint64_t x0 = reinterpret_cast<uint64_t>(cp.x + nb.x_off);
        const uint64_t x1 = x0 + static_cast<uint64_t>(nb.n) * static_cast<uint64_t>(nb.n) * 8u;
        const uint64_t xa = (x0 + 15u) & ~15ull, xb = x1 & ~15ull;
        if (abytes >= 16u)
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(reinterpret_cast<uint64_t>(nb.a32)), "r"(abytes & ~15u) : "memory");
        if (xb > xa)
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(xa), "r"(static_cast<uint32_t>(xb - xa))
                         : "memory");
    };
    // Blocks are claimed from the counter one ahead (the list runs largest
    // first), so CTAs that start late or draw small blocks take more.
    if (threadIdx.x == 0) {
        const int c0 = atomicAdd(cp.next, 1);
        claim[0] = c0;
        prefetch(c0);
    }
    __syncthreads();
    for (;;) {
        const int bi = claim[0];
        if (bi >= cp.count || stop) break;
        if (threadIdx.x == 0) {
            const int c1 = atomicAdd(cp.next, 1);
            claim[1] = c1;
            prefetch(c1);
        }
        const ChainBlock cb = cp.blocks[bi];
        kbh = cb.n > 64 ? 2 : 1;
        const int nr = (cb.n + 31) & ~31;
        const float inv = d2f_rn(*cb.inv_scale);
        ch_split_from_f32(mA, cb, inv);
        if (nr < 128) {  // the epilogues leave the padding runs alone: clear what the last block left there
            ch_zero(mA2);
            ch_zero(mA3);
        }
        operands_ready();
        for (int s = 0; s < cp.steps && !stop; ++s) {
            const float sc = (cp.dual_steps ? 0.5f : 1.0f) * kF16AccUnscale;
            product(sA, sA, false);  // A2 = A A
            ch_epilogue(CH_STORE, kF16AccUnscale, 0.f, 0.f, 0.f, mA2, mA, mA3, dummy, tmem, cb, nr, cp.x);
            operands_ready();
            product(sA2, sA, cp.dual_steps != 0);  // A3 = A2 A
            ch_epilogue(CH_STORE, sc, 0.f, 0.f, 0.f, mA3, mA, mA3, dummy, tmem, cb, nr, cp.x);
            operands_ready();
            product(sA3, sA2, cp.dual_steps != 0);  // A = a A + b A3 + c A3 A2
            ch_epilogue(CH_STEP, sc, cp.coef[3 * s], cp.coef[3 * s + 1], cp.coef[3 * s + 2], mA, mA, mA3, dummy, tmem,
                        cb, nr, cp.x);
            operands_ready();
            stop = __syncthreads_or(*abort_flag != 0) != 0;  // one answer for the whole CTA
        }
        if (stop) break;
        ch_split_from_f32(mA2, cb, inv);  // Xs
        operands_ready();
        product(sA2, sA, true);  // (Xs A + A Xs) / 2
        ch_epilogue(CH_FINAL, 0.5f * kF16AccUnscale, 0.f, 0.f, 0.f, nullptr, mA, mA3, dummy, tmem, cb, nr, cp.x);
        operands_ready();
        stop = __syncthreads_or(*abort_flag != 0) != 0;
        if (threadIdx.x == 0) claim[0] = claim[1];
        __syncthreads();
    }
    // ---- teardown ----
    tc_fence_before();
    __syncthreads();
    if (*abort_flag && threadIdx.x == 0) {
        umma_commit(drain);  // every MMA issued so far has completed
        if (!mbar_wait_bounded(drain, 0)) atomicCAS(cp.err, 0, DEVERR_DRAIN_WAIT);
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 128);
    }
}

}  // namespace

psdgb_status launch_batch_chain(DeviceState* ds, int precision, const ChainBlock* d_blocks, int count,
                                const float* coef, int steps, double* d_x, int* d_counter, int grid,
                                cudaStream_t s) {
    if (count <= 0) return PSDGB_OK;
    if (steps > 16 || (precision != PSDGB_PREC_FP16X3 && precision != PSDGB_PREC_FP16)) {
        set_error("batch chain: FP16-pair precisions with at most 16 steps");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    ChainParams cp{};
    cp.blocks = d_blocks;
    cp.count = count;
    for (int i = 0; i < 3 * steps; ++i) cp.coef[i] = coef[i];
    cp.steps = steps;
    cp.dual_steps = precision == PSDGB_PREC_FP16 ? 1 : 0;
    cp.x = d_x;
    cp.next = d_counter;
    cp.err = ds->d_error;
    PSDGB_CUDA_TRY(cudaMemsetAsync(d_counter, 0, sizeof(int), s));
    int g = grid > 0 ? grid : sm_budget(ds);
    if (g > count) g = count;
    if (precision == PSDGB_PREC_FP16X3) {
        static bool configured = false;
        if (!configured) {
            PSDGB_CUDA_TRY(cudaFuncSetAttribute(batch_chain_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                CH_SMEM));
            configured = true;
        }
        batch_chain_kernel<3><<<static_cast<unsigned>(g), CH_THREADS, CH_SMEM, s>>>(cp);
    } else {
        static bool configured = false;
        if (!configured) {
            PSDGB_CUDA_TRY(cudaFuncSetAttribute(batch_chain_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                CH_SMEM));
            configured = true;
        }
        batch_chain_kernel<1><<<static_cast<unsigned>(g), CH_THREADS, CH_SMEM, s>>>(cp);
    }
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    return PSDGB_OK;
}

}  // namespace psdgb
