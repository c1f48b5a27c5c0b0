// gemm_tc.cu — symmetric filter products on the sm_103a tensor cores.
//
// Replaces the reference's cublasSgemm / cublasGemmEx chain
// (src/composite_FP32.cu:103-115,150; src/composite_FP16.cu:118-163,218-227;
// src/composite_FP32_emulated.cu:108-153,210-221).  Each product C = P * Q of
// two symmetric, commuting matrices is computed on the 128x128 tiles (bi, bj)
// with bi >= bj only, so half the MMA work of a full GEMM.
//
// One persistent kernel serves a single matrix and a group of independent
// blocks (a block-diagonal iterate) alike: the operands of every block live
// in one strided row-major layout (row stride ld), block b occupying rows
// [row_base_b, row_base_b + np_b); one TMA descriptor per operand term plane
// covers all blocks.  The work is a list of tiles (block, bi, bj) — implicit
// (all lower tiles of one block) or a device table — walked round-robin by
// gridDim.x CTAs, one per SM.
//
// CTA structure (192 threads):
//   warp 0 lane 0  TMA producer: per 64-wide K block, loads the operand term
//                  tiles of P (rows bi) and Q (rows bj) into a STAGES-deep
//                  shared-memory ring (128-byte swizzle, K-major), running
//                  ahead across tile boundaries;
//   warp 1 lane 0  MMA issuer: tcgen05.mma kind::f16 (FP16 or BF16 in, FP32
//                  accumulate in TMEM), one MMA per term product per 16-wide
//                  K slice; the K blocks of a tile are dealt round-robin to
//                  ACC_SPLIT accumulators (each sees K/ACC_SPLIT additions);
//                  ACC_BUFS accumulator sets let the next tile's MMAs run while
//                  the epilogue drains the previous one;
//   warps 2-5      epilogue: tcgen05.ld of the accumulators (one TMEM lane per
//                  tile row), their FP32 sum, the polynomial step / ReLU
//                  reconstruction, operand splitting, and the stores at (p, q)
//                  and at the mirror (q, p); then it frees the accumulator set.
// Because P and Q are symmetric, the B operand "Q^T" is Q itself, so both
// operands are K-major row blocks of row-major matrices.
//
// Split precision: an operand x is stored as terms (FP16 hi + lo, or BF16
// b0 + b1 + b2); the product is the sum of the term products selected by
// the precision (1, 3, 6 or 9), all accumulated in the same FP32 TMEM tile.
//
// Every mbarrier wait is bounded (common.cuh); a wait that gives up records a
// DeviceError, drains the copies and MMAs it issued, frees TMEM and returns.
#include <mutex>

#include "tc_kernel.cuh"

namespace psdgb {

namespace {

// ---- the kernel --------------------------------------------------------------

template <int TERMS, int NPROD, bool BF16, int ACC_SPLIT, int ACC_BUFS, int EW, bool FP8 = false,
          bool STAGED_FINAL = false>
__global__ void __launch_bounds__(64 + 32 * EW, 1)
    tc_group_kernel(const __grid_constant__ TmapSet tm, const EpiParams ep, const GroupWork gw, int num_tiles,
                    int* err) {
    using Cfg = TcCfg<TERMS, EW * RUN_STAGE_BYTES>;
    // E4M3 operands (FP8 = true): 128 elements per 128-byte K block,
    // tcgen05.mma kind::f8f6f4 with K = 32 per instruction; the shared-memory
    // geometry in bytes is that of the 16-bit operands.
    constexpr int KBE = FP8 ? 2 * BK : BK;
    constexpr int STAGES = Cfg::STAGES;
    constexpr int STAGE_BYTES = Cfg::STAGE_BYTES;
    constexpr uint32_t IDESC = idesc_f16(BM, BN, BF16);
    constexpr uint32_t TMEM_COLS = ACC_SPLIT * ACC_BUFS * BN;
    static_assert(TMEM_COLS == 128 || TMEM_COLS == 256 || TMEM_COLS == 512, "TMEM allocation");

    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw_addr = smem_u32(smem_raw);
    uint8_t* smem = smem_raw + ((1024u - (raw_addr & 1023u)) & 1023u);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* acc_full = empty + STAGES;
    uint64_t* acc_empty = acc_full + ACC_BUFS;
    uint64_t* drain = acc_empty + ACC_BUFS;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    volatile int* issued_slot = abort_flag + 1;

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int dual_mult = ep.dual ? 2 : 1;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < ACC_BUFS; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], EW);  // one arrival per epilogue warp
        }
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
        // ---- TMA producer ----
        for (int t = 0; t < TERMS; ++t) {
            tma_prefetch_desc(&tm.P[t]);
            tma_prefetch_desc(&tm.Q[t]);
        }
        int g = 0;  // K blocks issued by this CTA (ring position)
        bool stop = false;
        for (int tile = blockIdx.x; tile < num_tiles && !stop; tile += gridDim.x) {
            const TileInfo ti = tile_info(gw, ep, tile);
            const int kb_half = tile_kblocks<KBE>(ep, ti);
            const int kb_total = kb_half * dual_mult;
            const int row_p = static_cast<int>(ti.blk.row_base + ti.bi * BM);
            const int row_q = static_cast<int>(ti.blk.row_base + ti.bj * BN);
            const int col0 = ti.blk.col_base;
            for (int kb = 0; kb < kb_total; ++kb, ++g) {
                const int s = g % STAGES;
                const uint32_t ph = static_cast<uint32_t>(g / STAGES) & 1u;
                if (!mbar_wait_bounded(&empty[s], ph ^ 1u)) {
                    record_error(err, abort_flag, DEVERR_TMA_WAIT);
                    stop = true;
                    break;
                }
                if (*abort_flag) {
                    stop = true;
                    break;
                }
                uint8_t* st = smem + s * STAGE_BYTES;
                // In a dual product the second half of the K loop multiplies Q's
                // rows bi by P's rows bj (the transpose-side term Q * P^T).
                const bool second = kb >= kb_half;
                const CUtensorMap* mp = second ? tm.Q : tm.P;
                const CUtensorMap* mq = second ? tm.P : tm.Q;
                const int kx = col0 + (second ? kb - kb_half : kb) * KBE;
                mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
#pragma unroll
                for (int t = 0; t < TERMS; ++t) tma_load_2d(st + t * TILE_BYTES, &mp[t], &full[s], kx, row_p);
#pragma unroll
                for (int t = 0; t < TERMS; ++t)
                    tma_load_2d(st + (TERMS + t) * TILE_BYTES, &mq[t], &full[s], kx, row_q);
                *issued_slot = g + 1;
            }
        }
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        int g = 0, it = 0;
        bool stop = false;
        for (int tile = blockIdx.x; tile < num_tiles && !stop; tile += gridDim.x, ++it) {
            const TileInfo ti = tile_info(gw, ep, tile);
            const int kb_total = tile_kblocks<KBE>(ep, ti) * dual_mult;
            const int buf = it % ACC_BUFS;
            const uint32_t use_ph = static_cast<uint32_t>(it / ACC_BUFS) & 1u;
            if (!mbar_wait_bounded(&acc_empty[buf], use_ph ^ 1u)) {
                record_error(err, abort_flag, DEVERR_MMA_WAIT);
                break;
            }
            tc_fence_after();
            const uint32_t acc_base = tmem + static_cast<uint32_t>(buf * ACC_SPLIT * BN);
            for (int kb = 0; kb < kb_total; ++kb, ++g) {
                const int s = g % STAGES;
                const uint32_t ph = static_cast<uint32_t>(g / STAGES) & 1u;
                if (!mbar_wait_bounded(&full[s], ph)) {
                    record_error(err, abort_flag, DEVERR_MMA_WAIT);
                    stop = true;
                    break;
                }
                if (*abort_flag) {
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t base = smem_u32(smem + s * STAGE_BYTES);
                const uint32_t acc = acc_base + static_cast<uint32_t>((kb % ACC_SPLIT) * BN);
#pragma unroll
                for (int k = 0; k < BK / 16; ++k) {
#pragma unroll
                    for (int pi = 0; pi < NPROD; ++pi) {
                        const uint64_t ad = sdesc_kmajor_sw128(base + prod_a(pi) * TILE_BYTES + k * 32);
                        const uint64_t bd = sdesc_kmajor_sw128(base + (TERMS + prod_b(pi)) * TILE_BYTES + k * 32);
                        const uint32_t accum = (kb >= ACC_SPLIT || k != 0 || pi != 0) ? 1u : 0u;
                        if (FP8)
                            umma_f8(acc, ad, bd, IDESC, accum);
                        else
                            umma_f16(acc, ad, bd, IDESC, accum);
                    }
                }
                umma_commit(&empty[s]);
            }
            if (stop) break;
            umma_commit(&acc_full[buf]);
        }
    } else if (warp >= 2) {
        // ---- epilogue: EW warps, EW / 4 per TMEM lane quarter, each on a
        // slice of the tile's columns ----
        const int q4 = warp & 3;  // TMEM lane quarter this warp may access
        constexpr int SLICE = BN / (EW / 4);
        const int c_begin = ((warp - 2) / 4) * SLICE;
        // this warp's staging buffer, after the barriers
        uint8_t* stage = smem + STAGES * STAGE_BYTES + 512 + (warp - 2) * RUN_STAGE_BYTES;
        int it = 0;
        for (int tile = blockIdx.x; tile < num_tiles; tile += gridDim.x, ++it) {
            const TileInfo ti = tile_info(gw, ep, tile);
            const int kb_total = tile_kblocks<KBE>(ep, ti) * dual_mult;
            const int buf = it % ACC_BUFS;
            const uint32_t use_ph = static_cast<uint32_t>(it / ACC_BUFS) & 1u;
            if (!mbar_wait_warp(&acc_full[buf], use_ph)) {
                record_error(err, abort_flag, DEVERR_EPI_WAIT);
                break;
            }
            if (warp_flag(abort_flag)) break;
            tc_fence_after();
            const int64_t p0 = ti.bi * BM + q4 * 32;
            const uint32_t tmem_row =
                tmem + (static_cast<uint32_t>(q4 * 32) << 16) + static_cast<uint32_t>(buf * ACC_SPLIT * BN);
            const int nacc = kb_total < ACC_SPLIT ? kb_total : ACC_SPLIT;
            // The storage format follows the operands: F16Q8 for E4M3 products,
            // BF16 for BF16 ones, FP16 otherwise (ep.fmt says the same), so
            // each instantiation compiles one epilogue.
            constexpr int FMT = FP8 ? FMT_F16Q8 : (BF16 ? FMT_BF16 : FMT_F16);
            epilogue_tile<FMT, ACC_SPLIT, BN, FP8, STAGED_FINAL>(ep, ti, tmem_row, p0, nacc, c_begin, c_begin + SLICE,
                                                                stage);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[buf]);
        }
    }

    // ---- teardown ----
    tc_fence_before();
    __syncthreads();
    if (*abort_flag) {
        if (warp == 1 && lane == 0) {
            // Wait until every MMA issued so far has completed.
            umma_commit(drain);
            if (!mbar_wait_bounded(drain, 0)) atomicCAS(err, 0, DEVERR_DRAIN_WAIT);
        }
        if (warp == 0 && lane == 0) {
            // Wait for the loads of the last STAGES issued K blocks to land.
            const int issued = *issued_slot;
            for (int g = issued - STAGES; g < issued; ++g) {
                if (g < 0) continue;
                const int s = g % STAGES;
                const uint32_t ph = static_cast<uint32_t>(g / STAGES) & 1u;
                if (!mbar_wait_bounded(&full[s], ph)) atomicCAS(err, 0, DEVERR_DRAIN_WAIT);
            }
        }
        __syncthreads();
    }
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, TMEM_COLS);
    }
}

// ---- host side -------------------------------------------------------------

template <int TERMS, int NPROD, bool BF16, int ACC_SPLIT, int ACC_BUFS, int EW, bool FP8 = false,
          bool STAGED_FINAL = false>
psdgb_status launch_tc(DeviceState* ds, const SplitMat& P, const SplitMat& Q, int64_t ld, int64_t rows,
                       const EpiParams& ep, const GroupWork& gw, int64_t num_tiles, int grid, cudaStream_t s) {
    using Cfg = TcCfg<TERMS, EW * RUN_STAGE_BYTES>;
    auto kern = tc_group_kernel<TERMS, NPROD, BF16, ACC_SPLIT, ACC_BUFS, EW, FP8, STAGED_FINAL>;
    if (ep.kind != EPI_FINAL && ep.kind != EPI_FINAL32 && ep.fmt != (FP8 ? FMT_F16Q8 : (BF16 ? FMT_BF16 : FMT_F16))) {
        set_error("gemm_tc: the epilogue's storage format does not match the operand type");
        return PSDGB_ERR_INVALID_ARGUMENT;
    }
    static bool configured = false;  // attribute set once per process (per instantiation)
    if (!configured) {
        PSDGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM_BYTES));
        configured = true;
    }
    TmapSet tm;
    for (int t = 0; t < 3; ++t) {
        if (FP8) {  // the E4M3 plane (term 2 of the F16Q8 format)
            if (!make_tmap_u8(&tm.P[t], P.term[2], ld, rows, BM) || !make_tmap_u8(&tm.Q[t], Q.term[2], ld, rows, BM)) {
                set_error("cuTensorMapEncodeTiled failed");
                return PSDGB_ERR_CUDA;
            }
            continue;
        }
        void* pb = (t < TERMS) ? P.term[t] : P.term[0];
        void* qb = (t < TERMS) ? Q.term[t] : Q.term[0];
        if (!make_tmap(&tm.P[t], pb, ld, rows, BF16, BM) || !make_tmap(&tm.Q[t], qb, ld, rows, BF16, BM)) {
            set_error("cuTensorMapEncodeTiled failed");
            return PSDGB_ERR_CUDA;
        }
    }
    if (num_tiles <= 0) return PSDGB_OK;
    int g = grid > 0 ? grid : sm_budget(ds);
    if (g > num_tiles) g = static_cast<int>(num_tiles);
    kern<<<static_cast<unsigned>(g), 64 + 32 * EW, Cfg::SMEM_BYTES, s>>>(tm, ep, gw, static_cast<int>(num_tiles),
                                                                    ds->d_error);
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    return PSDGB_OK;
}

template <int TERMS, int NPROD, bool BF16, bool FP8 = false>
psdgb_status launch_acc(DeviceState* ds, int acc_mode, const SplitMat& P, const SplitMat& Q, int64_t ld,
                        int64_t rows, const EpiParams& ep, const GroupWork& gw, int64_t num_tiles, int grid,
                        cudaStream_t s) {
    switch (acc_mode) {
        case ACC_4X1:
            return launch_tc<TERMS, NPROD, BF16, 4, 1, 4, FP8>(ds, P, Q, ld, rows, ep, gw, num_tiles, grid, s);
        case ACC_2X2:
            return launch_tc<TERMS, NPROD, BF16, 2, 2, 4, FP8>(ds, P, Q, ld, rows, ep, gw, num_tiles, grid, s);
        case ACC_1X4:
            // Short-K tiles (block-diagonal batches, small matrices) are
            // epilogue-bound: twice the epilogue warps, each on half the columns.
            if (g_group_epi_warps == 8) {
                // the final reconstruction on its own instantiation, staged
                if constexpr (!FP8) {
                    if (ep.kind == EPI_FINAL)
                        return launch_tc<TERMS, NPROD, BF16, 1, 4, 8, false, true>(ds, P, Q, ld, rows, ep, gw,
                                                                                   num_tiles, grid, s);
                }
                return launch_tc<TERMS, NPROD, BF16, 1, 4, 8, FP8>(ds, P, Q, ld, rows, ep, gw, num_tiles, grid, s);
            }
            return launch_tc<TERMS, NPROD, BF16, 1, 4, 4, FP8>(ds, P, Q, ld, rows, ep, gw, num_tiles, grid, s);
        default: break;
    }
    set_error("gemm_tc: unknown accumulator mode");
    return PSDGB_ERR_INVALID_ARGUMENT;
}

}  // namespace

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

bool make_tmap(CUtensorMap* tm, void* base, int64_t ld, int64_t rows, bool bf16, int box_rows, int box_cols) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(ld), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 2};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(box_cols), static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r =
        fn(tm, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, base, dims, strides, box,
           estr, CU_TENSOR_MAP_INTERLEAVE_NONE, box_cols == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

bool make_tmap_u8(CUtensorMap* tm, void* base, int64_t ld, int64_t rows, int box_rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(ld), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld)};
    const cuuint32_t box[2] = {128u, static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(tm, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, base, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

bool make_tmap_f32(CUtensorMap* tm, const void* base, int64_t ld, int64_t rows, int64_t cols, int box_rows,
                   int box_cols) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(cols), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ld) * 4};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(box_cols), static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

psdgb_status gemm_tc_group(DeviceState* ds, int precision, int acc_mode, const SplitMat& P, const SplitMat& Q,
                           int64_t ld, int64_t rows, const EpiParams& ep, const GroupWork& gw, int64_t num_tiles,
                           int grid, cudaStream_t s) {
    switch (precision) {
        case PSDGB_PREC_FP16: return launch_acc<1, 1, false>(ds, acc_mode, P, Q, ld, rows, ep, gw, num_tiles, grid, s);
        case PSDGB_PREC_FP8:
            return launch_acc<1, 1, false, true>(ds, acc_mode, P, Q, ld, rows, ep, gw, num_tiles, grid, s);
        case PSDGB_PREC_BF16: return launch_acc<1, 1, true>(ds, acc_mode, P, Q, ld, rows, ep, gw, num_tiles, grid, s);
        case PSDGB_PREC_FP16X3:
            return launch_acc<2, 3, false>(ds, acc_mode, P, Q, ld, rows, ep, gw, num_tiles, grid, s);
        case PSDGB_PREC_BF16X3:
            return launch_acc<2, 3, true>(ds, acc_mode, P, Q, ld, rows, ep, gw, num_tiles, grid, s);
        case PSDGB_PREC_BF16X6:
            return launch_acc<3, 6, true>(ds, acc_mode, P, Q, ld, rows, ep, gw, num_tiles, grid, s);
        case PSDGB_PREC_BF16X9:
            return launch_acc<3, 9, true>(ds, acc_mode, P, Q, ld, rows, ep, gw, num_tiles, grid, s);
        default: break;
    }
    set_error("gemm_tc: unknown precision");
    return PSDGB_ERR_INVALID_ARGUMENT;
}

// One matrix: the implicit tile list of all lower tiles of an np x np operand.
psdgb_status gemm_tc(DeviceState* ds, int precision, const SplitMat& P, const SplitMat& Q, int64_t np,
                     const EpiParams& ep, cudaStream_t s) {
    const int64_t nt = np / BM;
    EpiParams e = ep;
    e.ld = static_cast<int>(np);
    // The E4M3 products run on 128 x 128 tiles only; three-term products also
    // run on 256 x 256 pair tiles, not on 128 x 256 single-CTA tiles (whose
    // stages would not fit twice in shared memory).
    const bool fp8 = precision == PSDGB_PREC_FP8;
    const bool three_terms = precision == PSDGB_PREC_BF16X6 || precision == PSDGB_PREC_BF16X9;
    int shape = g_tile_shape;
    if (shape < 0) shape = (!fp8 && np >= 2048) ? TILE_PAIR_256X256 : TILE_128X128;
    if (nt >= 2 && shape == TILE_PAIR_256X128 && !fp8)
        return gemm_tc_pair(ds, precision, auto_acc_mode(precision, np), P, Q, np, e, s);
    if (nt >= 2 && shape == TILE_WIDE_128X256 && !three_terms && !fp8)
        return gemm_tc_wide(ds, precision, P, Q, np, e, s);
    if (nt >= 2 && shape == TILE_PAIR_256X256 && !fp8) return gemm_tc_pairwide(ds, precision, P, Q, np, e, s);
    GroupWork gw{nullptr, nullptr, g_tile_group_rows};
    return gemm_tc_group(ds, precision, auto_acc_mode(precision, np), P, Q, np, np, e, gw, nt * (nt + 1) / 2, 0, s);
}

int g_single_acc_mode = -1;
int g_tile_group_rows = 8;
int g_group_epi_warps = 8;

// Accumulator configuration: the accuracy of one tensor-core FP32 accumulator
// degrades with the number of K blocks it sums (n = 8192: 4.3e-5 rel. error
// with one, 2.1e-5 with two, 1.1e-5 with four, for every split precision), so
// long FP32-class products deal K over four accumulators; short ones, and the
// one-term precisions (whose error is their operand rounding), double-buffer
// the accumulators instead so the epilogue overlaps the next tile (+4-10 %).
int auto_acc_mode(int precision, int64_t np) {
    if (g_single_acc_mode >= 0) return g_single_acc_mode;
    if (precision == PSDGB_PREC_FP16 || precision == PSDGB_PREC_BF16 || precision == PSDGB_PREC_FP8) return ACC_1X4;
    if (np <= 2048) return ACC_1X4;
    if (np <= 4096) return ACC_2X2;
    return ACC_4X1;
}

}  // namespace psdgb
