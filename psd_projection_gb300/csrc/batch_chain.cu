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
//   final     Xs = split(X x 1/up) from the FP64 input; out = (X + up (Xs A +
//             A Xs)/2) / 2 written to the caller's block in place.
//
// The arithmetic is that of the grouped path with one TMEM accumulator
// (ACC_1X4): the same MMA order (K blocks, then K slices, then term
// products), the same epilogue (lower triangle computed, mirrored), the same
// split, so a block's result is the same bit for bit.
//
// Shared memory: each split matrix is two planes (FP16 hi, lo) of two K
// blocks, each a 128-row x 128-byte tile in the layout TMA writes with the
// 128-byte swizzle (16-byte chunk c of row r at chunk c ^ (r & 7)), which is
// what the K-major shared-memory descriptors of the MMAs read.  128 threads:
// thread r owns row r (TMEM lane r, warp r / 32 on lane quarter r / 32);
// thread 0 also issues the MMAs.  One CTA per SM (197 KB of shared memory),
// persistent over the list of small blocks.  Every wait is bounded.
#include <cuda.h>

#include "convert.h"
#include "tc_kernel.cuh"

namespace psdgb {

namespace {

constexpr int CH_THREADS = 128;
constexpr int CH_TILE = 128 * 128;                 // bytes of one plane's K block (128 rows x 128 B)
constexpr int CH_MAT = 2 * 2 * CH_TILE;            // two planes x two K blocks: 64 KB
constexpr int CH_SMEM = 3 * CH_MAT + 1024 + 256;   // A, A2, A3, alignment, barriers
constexpr uint32_t CH_IDESC_F16 = idesc_f16(128, 128, false);

// Byte offset of element (r, k) in a split matrix's plane t.
__device__ __forceinline__ uint32_t ch_off(int t, int r, int k) {
    const int kb = k >> 6, kk = k & 63;
    return static_cast<uint32_t>((t * 2 + kb) * CH_TILE + r * 128 + ((((kk >> 3) ^ (r & 7)) << 4) | ((kk & 7) << 1)));
}

// Eight consecutive values (k a multiple of 8) of row r, as split_store8
// writes them: FP16 hi / lo of v * 2^12, one 16-byte chunk per plane.
__device__ __forceinline__ void ch_store8(uint8_t* m, int r, int k, const float (&v)[8]) {
    __align__(16) __half h[8];
    __align__(16) __half l[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const float x = v[e] * kF16Scale;
        h[e] = __float2half_rn(x);
        l[e] = __float2half_rn(x - __half2float(h[e]));
    }
    *reinterpret_cast<uint4*>(m + ch_off(0, r, k)) = *reinterpret_cast<const uint4*>(h);
    *reinterpret_cast<uint4*>(m + ch_off(1, r, k)) = *reinterpret_cast<const uint4*>(l);
}

// Eight consecutive stored values of row r (load_run8's arithmetic: lo + hi, then 2^-12).
__device__ __forceinline__ void ch_load8(const uint8_t* m, int r, int k, float (&out)[8]) {
    const uint4 hv = *reinterpret_cast<const uint4*>(m + ch_off(0, r, k));
    const uint4 lv = *reinterpret_cast<const uint4*>(m + ch_off(1, r, k));
    const __half* h = reinterpret_cast<const __half*>(&hv);
    const __half* l = reinterpret_cast<const __half*>(&lv);
#pragma unroll
    for (int e = 0; e < 8; ++e) out[e] = ((0.f + __half2float(l[e])) + __half2float(h[e])) * kF16Unscale;
}

// One element's terms at (r, k) in both planes (split_store's arithmetic).
__device__ __forceinline__ void ch_store1(uint8_t* m, int r, int k, float v) {
    const float x = v * kF16Scale;
    const __half h = __float2half_rn(x);
    const __half l = __float2half_rn(x - __half2float(h));
    *reinterpret_cast<__half*>(m + ch_off(0, r, k)) = h;
    *reinterpret_cast<__half*>(m + ch_off(1, r, k)) = l;
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
    int* err;
};

// The epilogue of one product for thread `row`: the lower-triangle elements of
// its row from TMEM, combined and written to `out` and mirrored (CH_STORE /
// CH_STEP), or to the caller's FP64 block (CH_FINAL).
__device__ __forceinline__ void ch_epilogue(int kind, float acc_scale, float a, float b, float c, uint8_t* out,
                                            const uint8_t* Am, const uint8_t* A3m, uint32_t tmem_row, int row,
                                            const ChainBlock& cb, double* x) {
    const int p0 = row & ~31;
    for (int q0 = 0; q0 <= p0; q0 += 32) {
        float v[32];
        tmem_ld_32cols(tmem_row + static_cast<uint32_t>(q0), v);
        if (kind == CH_FINAL) {
            const int n = cb.n;
            if (row >= n) continue;
            const double up = *cb.scale;
            double* X = x + cb.x_off;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int q = q0 + j;
                if (q <= row && q < n) {
                    const double o = 0.5 * (X[static_cast<int64_t>(row) * n + q] + up * static_cast<double>(acc_scale * v[j]));
                    X[static_cast<int64_t>(row) * n + q] = o;
                    if (q != row) X[static_cast<int64_t>(q) * n + row] = o;
                }
            }
            continue;
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] *= acc_scale;
        if (kind == CH_STEP) {
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                float av[8], a3[8];
                ch_load8(Am, row, q0 + 8 * g, av);
                ch_load8(A3m, row, q0 + 8 * g, a3);
#pragma unroll
                for (int j = 0; j < 8; ++j) v[8 * g + j] = fmaf(c, v[8 * g + j], fmaf(b, a3[j], a * av[j]));
            }
        }
        if (q0 + 31 < row) {  // the whole run lies below the diagonal: row and mirror
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                const float w[8] = {v[8 * g], v[8 * g + 1], v[8 * g + 2], v[8 * g + 3],
                                    v[8 * g + 4], v[8 * g + 5], v[8 * g + 6], v[8 * g + 7]};
                ch_store8(out, row, q0 + 8 * g, w);
            }
#pragma unroll
            for (int j = 0; j < 32; ++j) ch_store1(out, q0 + j, row, v[j]);
        } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int q = q0 + j;
                if (q <= row) {
                    ch_store1(out, row, q, v[j]);
                    if (q != row) ch_store1(out, q, row, v[j]);
                }
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
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 3 * CH_MAT);
    uint64_t* drain = bar + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const int row = threadIdx.x, warp = threadIdx.x / 32;
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
    const uint32_t tmem_row = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    const uint32_t sA = smem_u32(mA), sA2 = smem_u32(mA2), sA3 = smem_u32(mA3);
    uint32_t phase = 0;
    bool stop = false;
    // One product: MMAs by thread 0, then every thread waits for them (bounded).
    int kbh = 2;
    auto product = [&](uint32_t P, uint32_t Q, bool dual) {
        if (threadIdx.x == 0) {
            tc_fence_after();
            ch_mma<NPROD>(tmem, P, Q, dual, kbh);
            umma_commit(bar);
        }
        if (!mbar_wait_bounded(bar, phase)) {
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
    for (int bi = blockIdx.x; bi < cp.count && !stop; bi += gridDim.x) {
        const ChainBlock cb = cp.blocks[bi];
        const int n = cb.n;
        kbh = n > 64 ? 2 : 1;
        // A = split(a32 x 1/up): the FP32 copy (rows of ld4 floats, ld4 a
        // multiple of 4 and rows 16-byte aligned), zero padding.
        const float inv = d2f_rn(*cb.inv_scale);
        const float* arow = cb.a32 + static_cast<int64_t>(row) * cb.ld4;
        for (int k = 0; k < 128; k += 8) {
            float v[8];
            if (row < n && k + 8 <= n) {
                const float4 u0 = *reinterpret_cast<const float4*>(arow + k);
                const float4 u1 = *reinterpret_cast<const float4*>(arow + k + 4);
                const float w[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
#pragma unroll
                for (int e = 0; e < 8; ++e) v[e] = w[e] * inv;
            } else {
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const float val = (row < n && k + e < n) ? arow[k + e] : 0.0f;
                    v[e] = val * inv;
                }
            }
            ch_store8(mA, row, k, v);
        }
        operands_ready();
        for (int s = 0; s < cp.steps && !stop; ++s) {
            product(sA, sA, false);  // A2 = A A
            ch_epilogue(CH_STORE, kF16AccUnscale, 0.f, 0.f, 0.f, mA2, mA, mA3, tmem_row, row, cb, cp.x);
            operands_ready();
            product(sA2, sA, cp.dual_steps != 0);  // A3 = A2 A
            ch_epilogue(CH_STORE, (cp.dual_steps ? 0.5f : 1.0f) * kF16AccUnscale, 0.f, 0.f, 0.f, mA3, mA, mA3,
                        tmem_row, row, cb, cp.x);
            operands_ready();
            product(sA3, sA2, cp.dual_steps != 0);  // A = a A + b A3 + c A3 A2
            ch_epilogue(CH_STEP, (cp.dual_steps ? 0.5f : 1.0f) * kF16AccUnscale, cp.coef[3 * s], cp.coef[3 * s + 1],
                        cp.coef[3 * s + 2], mA, mA, mA3, tmem_row, row, cb, cp.x);
            operands_ready();
            stop = *abort_flag != 0;
        }
        if (stop) break;
        // Xs = split(X x 1/up) into A2's storage; X's upper triangle (column
        // major) defines the symmetric matrix: Xs(i, j) = X[min + max * n].
        {
            const double* X = cp.x + cb.x_off;
            for (int k = 0; k < 128; k += 8) {
                float v[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int j = k + e;
                    float val = 0.0f;
                    if (row < n && j < n) {
                        const int lo = row < j ? row : j, hi = row < j ? j : row;
                        val = d2f_rn(X[lo + static_cast<int64_t>(hi) * n]);
                    }
                    v[e] = val * inv;
                }
                ch_store8(mA2, row, k, v);
            }
        }
        operands_ready();
        product(sA2, sA, true);  // (Xs A + A Xs) / 2
        ch_epilogue(CH_FINAL, 0.5f * kF16AccUnscale, 0.f, 0.f, 0.f, nullptr, mA, mA3, tmem_row, row, cb, cp.x);
        operands_ready();
        stop = *abort_flag != 0;
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
                                const float* coef, int steps, double* d_x, int grid, cudaStream_t s) {
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
    cp.err = ds->d_error;
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
