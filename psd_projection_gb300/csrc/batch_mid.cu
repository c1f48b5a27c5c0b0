// batch_mid.cu — the whole filter of a block-diagonal batch's blocks of
// 128 < n <= 256 (padded to 256: three lower 128 x 128 tiles), one CTA per
// block running all of that block's products back to back.
//
// In the grouped products (gemm_tc.cu) every launch sweeps the tiles of all
// blocks, so between two products of one block the whole batch's operands
// (far more than L2) pass through and each product re-reads its operands
// from DRAM.  A block of np = 256 has three split matrices of 256 KB each
// (FP16 hi / lo), so one CTA per SM keeps about 120 MB of them in flight —
// what L2 holds — and runs the block's chain, the reference's per-step
// Sgemm / Sscal / Saxpy / symmetrisation sequence
// (src/composite_FP32.cu:103-118, its FP16 twin src/composite_FP16.cu:118-166)
// and the final X (I + A) / 2 (src/composite_FP32.cu:142-156), product after
// product while the block stays in L2:
//
//   per step  A2 = A A; A3 = A2 A; A = a A + b A3 + c A3 A2   (3 tiles each)
//   final     Xs = split(X x 1/up) from the FP32 copy; out = (X + up (Xs A +
//             A Xs)/2) / 2 written to the caller's block in place
//
// (the first split A = split(a32 / up) is batch_split_kernel's, before this
// launch).  The CTA is the grouped kernel's (TMA producer, MMA issuer, 8
// epilogue warps, a ring of operand stages, four TMEM accumulators of one
// 128 x 128 tile each, the staged epilogue of tc_kernel.cuh) with the work
// list replaced by the block's jobs: a job's loads wait until every
// epilogue warp has finished the job before (its writes fenced for the
// async proxy, then an arrival on job_done); the epilogue warps also wait
// there before each job, so the step epilogue reads the A and A3 that the
// other warps wrote.  Every tile sums the same products in the same order
// as the grouped kernel with one accumulator per tile (ACC_1X4), and the
// epilogue is the same code, so the result is the same bit for bit.  Every
// wait is bounded.
#include <cuda.h>

#include "convert.h"
#include "tc_kernel.cuh"

namespace psdgb {

namespace {

constexpr int MID_EW = 8;                          // epilogue warps
constexpr int MID_THREADS = 64 + 32 * MID_EW;
constexpr int MID_ACC_BUFS = 4;                    // 128-column accumulators in TMEM
constexpr int MID_TERMS = 2;                       // FP16 hi / lo planes
using MidCfg = TcCfg<MID_TERMS, MID_EW * RUN_STAGE_BYTES>;
constexpr uint32_t MID_IDESC = idesc_f16(BM, BN, false);

struct MidMaps {
    CUtensorMap m[3][MID_TERMS];  // A, A2, A3: hi and lo planes
};

struct MidParams {
    const ChainBlock* cb;  // the blocks (FP32 copy, scale) ...
    const int* bidx;       // ... and their indices into blocks[]
    const BlockDesc* blocks;
    int count;
    SplitMat mat[3];       // A, A2, A3
    int ld;
    float coef[3 * 16];    // per step: a, b, c (after the safety scaling)
    int steps;
    int dual_steps;        // one-term products: the second and third products of a step take the symmetric part
    double* x;             // the batch's packed FP64 blocks (input, and output in place)
    int* err;
};

// Job j of a block: the products of the steps, the Xs split, the final product.
struct MidJob {
    int p, q, out;  // operand and output matrices (0 A, 1 A2, 2 A3); p < 0: the split job (no tiles)
    int kind;
    int dual;
    int step;
};

__device__ __forceinline__ MidJob mid_job(int j, int steps, int dual_steps) {
    MidJob J{};
    if (j < 3 * steps) {
        const int r = j % 3;
        J.step = j / 3;
        J.kind = r == 2 ? EPI_STEP : EPI_STORE;
        J.p = r == 0 ? 0 : (r == 1 ? 1 : 2);
        J.q = r == 2 ? 1 : 0;
        J.out = r == 0 ? 1 : (r == 1 ? 2 : 0);
        J.dual = r > 0 ? dual_steps : 0;
    } else if (j == 3 * steps) {
        J.p = -1;  // Xs = split(a32 / up) into A2
    } else {
        J.p = 1;   // (Xs A + A Xs) / 2
        J.q = 0;
        J.out = -1;
        J.kind = EPI_FINAL;
        J.dual = 1;
    }
    return J;
}

// Tile t of a product job: (0, 0), (1, 0), (1, 1).
__device__ __forceinline__ void mid_tile(int t, int& bi, int& bj) {
    bi = t == 0 ? 0 : 1;
    bj = t == 2 ? 1 : 0;
}

template <int NPROD>
__global__ void __launch_bounds__(MID_THREADS, 1)
    batch_mid_kernel(const __grid_constant__ MidMaps tm, const __grid_constant__ MidParams mp) {
    constexpr int STAGES = MidCfg::STAGES;
    constexpr int STAGE_BYTES = MidCfg::STAGE_BYTES;
    constexpr uint32_t TMEM_COLS = MID_ACC_BUFS * BN;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw_addr = smem_u32(smem_raw);
    uint8_t* smem = smem_raw + ((1024u - (raw_addr & 1023u)) & 1023u);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* acc_full = empty + STAGES;
    uint64_t* acc_empty = acc_full + MID_ACC_BUFS;
    uint64_t* job_done = acc_empty + MID_ACC_BUFS;
    uint64_t* drain = job_done + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    volatile int* issued_slot = abort_flag + 1;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int njobs = 3 * mp.steps + 2;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < MID_ACC_BUFS; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], MID_EW);
        }
        mbar_init(job_done, MID_EW);  // one arrival per epilogue warp and job
        mbar_init(drain, 1);
        *abort_flag = 0;
        *issued_slot = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, TMEM_COLS);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---- TMA producer: a job's loads start once the job before is done ----
        for (int m = 0; m < 3; ++m)
            for (int t = 0; t < MID_TERMS; ++t) tma_prefetch_desc(&tm.m[m][t]);
        int g = 0, gj = 0;
        bool stop = false;
        for (int mb = blockIdx.x; mb < mp.count && !stop; mb += gridDim.x) {
            const BlockDesc blk = mp.blocks[mp.bidx[mb]];
            const int kb_half = (blk.n + BK - 1) / BK;
            for (int j = 0; j < njobs && !stop; ++j, ++gj) {
                if (gj > 0 && !mbar_wait_bounded(job_done, static_cast<uint32_t>(gj - 1) & 1u)) {
                    record_error(mp.err, abort_flag, DEVERR_TMA_WAIT);
                    stop = true;
                    break;
                }
                const MidJob J = mid_job(j, mp.steps, mp.dual_steps);
                if (J.p < 0) continue;
                const int kb_total = kb_half * (J.dual ? 2 : 1);
                for (int t = 0; t < 3 && !stop; ++t) {
                    int bi, bj;
                    mid_tile(t, bi, bj);
                    const int row_p = blk.row_base + bi * BM, row_q = blk.row_base + bj * BN;
                    for (int kb = 0; kb < kb_total; ++kb, ++g) {
                        const int s = g % STAGES;
                        const uint32_t ph = static_cast<uint32_t>(g / STAGES) & 1u;
                        if (!mbar_wait_bounded(&empty[s], ph ^ 1u)) {
                            record_error(mp.err, abort_flag, DEVERR_TMA_WAIT);
                            stop = true;
                            break;
                        }
                        if (*abort_flag) {
                            stop = true;
                            break;
                        }
                        uint8_t* st = smem + s * STAGE_BYTES;
                        // a dual product's second half: Q's rows bi against P's rows bj
                        const bool second = kb >= kb_half;
                        const CUtensorMap* mpp = second ? tm.m[J.q] : tm.m[J.p];
                        const CUtensorMap* mqq = second ? tm.m[J.p] : tm.m[J.q];
                        const int kx = blk.col_base + (second ? kb - kb_half : kb) * BK;
                        mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
#pragma unroll
                        for (int tt = 0; tt < MID_TERMS; ++tt)
                            tma_load_2d(st + tt * TILE_BYTES, &mpp[tt], &full[s], kx, row_p);
#pragma unroll
                        for (int tt = 0; tt < MID_TERMS; ++tt)
                            tma_load_2d(st + (MID_TERMS + tt) * TILE_BYTES, &mqq[tt], &full[s], kx, row_q);
                        *issued_slot = g + 1;
                    }
                }
            }
        }
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer: the grouped kernel's, one accumulator per tile ----
        int g = 0, it = 0;
        bool stop = false;
        for (int mb = blockIdx.x; mb < mp.count && !stop; mb += gridDim.x) {
            const BlockDesc blk = mp.blocks[mp.bidx[mb]];
            const int kb_half = (blk.n + BK - 1) / BK;
            for (int j = 0; j < njobs && !stop; ++j) {
                const MidJob J = mid_job(j, mp.steps, mp.dual_steps);
                if (J.p < 0) continue;
                const int kb_total = kb_half * (J.dual ? 2 : 1);
                for (int t = 0; t < 3 && !stop; ++t, ++it) {
                    const int buf = it % MID_ACC_BUFS;
                    const uint32_t use_ph = static_cast<uint32_t>(it / MID_ACC_BUFS) & 1u;
                    if (!mbar_wait_bounded(&acc_empty[buf], use_ph ^ 1u)) {
                        record_error(mp.err, abort_flag, DEVERR_MMA_WAIT);
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t acc = tmem + static_cast<uint32_t>(buf * BN);
                    for (int kb = 0; kb < kb_total; ++kb, ++g) {
                        const int s = g % STAGES;
                        const uint32_t ph = static_cast<uint32_t>(g / STAGES) & 1u;
                        if (!mbar_wait_bounded(&full[s], ph)) {
                            record_error(mp.err, abort_flag, DEVERR_MMA_WAIT);
                            stop = true;
                            break;
                        }
                        if (*abort_flag) {
                            stop = true;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t base = smem_u32(smem + s * STAGE_BYTES);
#pragma unroll
                        for (int k = 0; k < BK / 16; ++k) {
#pragma unroll
                            for (int pi = 0; pi < NPROD; ++pi) {
                                const uint64_t ad = sdesc_kmajor_sw128(base + prod_a(pi) * TILE_BYTES + k * 32);
                                const uint64_t bd =
                                    sdesc_kmajor_sw128(base + (MID_TERMS + prod_b(pi)) * TILE_BYTES + k * 32);
                                umma_f16(acc, ad, bd, MID_IDESC, (kb != 0 || k != 0 || pi != 0) ? 1u : 0u);
                            }
                        }
                        umma_commit(&empty[s]);
                    }
                    if (stop) break;
                    umma_commit(&acc_full[buf]);
                }
            }
        }
    } else if (warp >= 2) {
        // ---- epilogue: 8 warps, two per TMEM lane quarter, each on 64 columns ----
        const int q4 = warp & 3;
        constexpr int SLICE = BN / (MID_EW / 4);
        const int c_begin = ((warp - 2) / 4) * SLICE;
        uint8_t* stage = smem + STAGES * STAGE_BYTES + 512 + (warp - 2) * RUN_STAGE_BYTES;
        const int etid = threadIdx.x - 64;  // 0 .. 255
        int it = 0, gj = 0;
        bool stop = false;
        for (int mb = blockIdx.x; mb < mp.count && !stop; mb += gridDim.x) {
            const BlockDesc blk = mp.blocks[mp.bidx[mb]];
            const ChainBlock cbk = mp.cb[mb];
            for (int j = 0; j < njobs && !stop; ++j, ++gj) {
                // the job before is done by every epilogue warp: its writes are visible
                if (gj > 0 && !mbar_wait_bounded(job_done, static_cast<uint32_t>(gj - 1) & 1u)) {
                    record_error(mp.err, abort_flag, DEVERR_EPI_WAIT);
                    stop = true;
                    break;
                }
                const MidJob J = mid_job(j, mp.steps, mp.dual_steps);
                if (J.p < 0) {
                    // Xs = split(a32 x 1/up) into A2 over the block's np x np area
                    // (zero outside n): batch_split_kernel's values and split.
                    const float inv = d2f_rn(*cbk.inv_scale);
                    const int n = cbk.n;
                    for (int c = etid; c < blk.np * (blk.np / 8); c += 32 * MID_EW) {
                        const int i = c / (blk.np / 8), j0 = (c % (blk.np / 8)) * 8;
                        float v[8];
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            const float val =
                                (i < n && j0 + e < n) ? cbk.a32[static_cast<int64_t>(i) * cbk.ld4 + j0 + e] : 0.0f;
                            v[e] = val * inv;
                        }
                        split_store8(mp.mat[1], FMT_F16,
                                     static_cast<size_t>(blk.row_base + i) * mp.ld + blk.col_base + j0, v);
                    }
                } else {
                    EpiParams e{};
                    e.fmt = FMT_F16;
                    e.ld = mp.ld;
                    e.acc_scale = 1.0f;
                    e.up = 1.0;
                    e.skip_pad = 1;
                    e.kind = J.kind;
                    e.dual = J.dual;
                    if (J.dual) e.acc_scale = 0.5f;
                    if (J.out >= 0) e.out = mp.mat[J.out];
                    if (J.kind == EPI_STEP) {
                        e.a = mp.coef[3 * J.step];
                        e.b = mp.coef[3 * J.step + 1];
                        e.c = mp.coef[3 * J.step + 2];
                        e.A = mp.mat[0];
                        e.A3 = mp.mat[2];
                    }
                    if (J.kind == EPI_FINAL) {
                        e.x64 = mp.x;
                        e.out64 = mp.x;
                    }
                    for (int t = 0; t < 3; ++t, ++it) {
                        const int buf = it % MID_ACC_BUFS;
                        const uint32_t use_ph = static_cast<uint32_t>(it / MID_ACC_BUFS) & 1u;
                        if (!mbar_wait_bounded(&acc_full[buf], use_ph)) {
                            record_error(mp.err, abort_flag, DEVERR_EPI_WAIT);
                            stop = true;
                            break;
                        }
                        if (*abort_flag) {
                            stop = true;
                            break;
                        }
                        tc_fence_after();
                        TileInfo ti;
                        int bi, bj;
                        mid_tile(t, bi, bj);
                        ti.bi = bi;
                        ti.bj = bj;
                        ti.blk = blk;
                        const int64_t p0 = ti.bi * BM + q4 * 32;
                        const uint32_t tmem_row =
                            tmem + (static_cast<uint32_t>(q4 * 32) << 16) + static_cast<uint32_t>(buf * BN);
                        epilogue_tile<FMT_F16, 1, BN, false, false>(e, ti, tmem_row, p0, 1, c_begin, c_begin + SLICE,
                                                                     stage);
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&acc_empty[buf]);
                    }
                }
                if (stop) break;
                // this warp's writes of the job, for the async proxy (the next
                // job's TMA loads) and for the other warps
                asm volatile("fence.proxy.async.global;" ::: "memory");
                __threadfence_block();
                __syncwarp();
                if (lane == 0) mbar_arrive(job_done);
            }
        }
    }

    // ---- teardown ----
    tc_fence_before();
    __syncthreads();
    if (*abort_flag) {
        if (warp == 1 && lane == 0) {
            umma_commit(drain);  // every MMA issued so far has completed
            if (!mbar_wait_bounded(drain, 0)) atomicCAS(mp.err, 0, DEVERR_DRAIN_WAIT);
        }
        if (warp == 0 && lane == 0) {
            const int issued = *issued_slot;
            for (int g = issued - STAGES; g < issued; ++g) {
                if (g < 0) continue;
                const int s = g % STAGES;
                const uint32_t ph = static_cast<uint32_t>(g / STAGES) & 1u;
                if (!mbar_wait_bounded(&full[s], ph)) atomicCAS(mp.err, 0, DEVERR_DRAIN_WAIT);
            }
        }
        __syncthreads();
    }
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, TMEM_COLS);
    }
}

}  // namespace

psdgb_status launch_batch_mid(DeviceState* ds, int precision, const ChainBlock* d_cb, const int* d_bidx,
                              const BlockDesc* d_blocks, int count, const SplitMat (&mats)[3], int64_t ld,
                              int64_t rows, const float* coef, int steps, double* d_x, int grid, cudaStream_t s) {
    if (count <= 0) return PSDGB_OK;
    if (steps > 16 || (precision != PSDGB_PREC_FP16X3 && precision != PSDGB_PREC_FP16)) {
        set_error("batch mid chain: FP16-pair precisions with at most 16 steps");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    auto kern = precision == PSDGB_PREC_FP16X3 ? batch_mid_kernel<3> : batch_mid_kernel<1>;
    static bool configured[2] = {false, false};
    if (!configured[precision == PSDGB_PREC_FP16X3]) {
        PSDGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, MidCfg::SMEM_BYTES));
        configured[precision == PSDGB_PREC_FP16X3] = true;
    }
    MidMaps tm;
    for (int m = 0; m < 3; ++m)
        for (int t = 0; t < MID_TERMS; ++t)
            if (!make_tmap(&tm.m[m][t], mats[m].term[t], ld, rows, false, BM)) {
                set_error("cuTensorMapEncodeTiled failed");
                return PSDGB_ERR_CUDA;
            }
    MidParams mp{};
    mp.cb = d_cb;
    mp.bidx = d_bidx;
    mp.blocks = d_blocks;
    mp.count = count;
    for (int m = 0; m < 3; ++m) mp.mat[m] = mats[m];
    mp.ld = static_cast<int>(ld);
    for (int i = 0; i < 3 * steps; ++i) mp.coef[i] = coef[i];
    mp.steps = steps;
    mp.dual_steps = precision == PSDGB_PREC_FP16 ? 1 : 0;
    mp.x = d_x;
    mp.err = ds->d_error;
    int g = grid > 0 ? grid : sm_budget(ds);
    if (g > count) g = count;
    kern<<<static_cast<unsigned>(g), MID_THREADS, MidCfg::SMEM_BYTES, s>>>(tm, mp);
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    return PSDGB_OK;
}

}  // namespace psdgb
