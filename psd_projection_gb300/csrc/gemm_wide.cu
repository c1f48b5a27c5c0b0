// gemm_wide.cu — symmetric filter products of one matrix on 128 x 256 tiles.
//
// The same products as gemm_tc.cu (C = P * Q of two symmetric, commuting
// matrices on the lower triangle, split-precision operand terms, the fused
// epilogue), replacing the reference's cublasSgemm / cublasGemmEx chain
// (src/composite_FP32.cu:103-115,150; src/composite_FP16.cu:118-163,218-227).
// One CTA owns a 128 x 256 tile: P's tile row bi against Q's tile rows 2 bj and
// 2 bj + 1, and one tcgen05.mma per term product and 16-wide K slice is
// 128 x 256 x 16.  Per MMA cycle the tile reads a third less operand data
// from shared memory than a 128 x 128 tile (the A operand serves twice the
// columns), and shared-memory traffic is what bounds the 128 x 128 kernel.
//
// Wide tile (bi, bj) covers columns 2 bj * 128 .. 2 bj * 128 + 255 and exists
// for 2 bj <= bi; for even bi the tile bj = bi / 2 has its right half above the
// diagonal (its epilogue stores nothing there: 1.5 % of the MMA work at
// n = 8192).
//
// Accumulation in K chunks: a 128 x 256 FP32 accumulator takes 256 of the
// 512 TMEM columns, too few for the four interleaved accumulators that long
// FP32-class products need (one tensor-core accumulator summing K = 8192 loses
// accuracy: 4.3e-5 vs 1.1e-5 at n = 8192).  The MMAs therefore accumulate
// CHUNK K blocks at a time into one of two TMEM slots; the epilogue adds each
// finished chunk into FP32 registers (IEEE adds) and frees the slot while the
// MMAs fill the other one, so accuracy matches K / CHUNK separate
// accumulators and the epilogue of a tile overlaps the next tile's MMAs.
// One-term precisions (whose error is their operand rounding) take the whole
// K of a tile as one chunk.
//
// CTA structure (320 threads): warp 0 lane 0 TMA producer, warp 1 lane 0 MMA
// issuer, warps 2-9 epilogue: warp w reads TMEM lane quarter w % 4 (one lane =
// one tile row) and columns 128 * ((w - 2) / 4) .. + 127 of the tile, keeping
// their 128 running sums in registers.  Barriers, bounded waits and the
// abort path are those of gemm_tc.cu.
#include "tc_kernel.cuh"

namespace psdgb {

namespace {

constexpr int TNW = 256;  // tile width

// Pipeline for TERMS operand terms and K blocks of KB elements (64: 128-byte
// rows, 128-byte swizzle; 32: 64-byte rows, 64-byte swizzle).  Smaller blocks
// give more stages in the same shared memory, so more load latency hidden
// (n = 8192, fp16x3: 4 stages of 48 KB run 6 % faster than 2 of 96 KB); 16-wide
// blocks with the 32-byte swizzle measured 35 % slower.
template <int TERMS, int KB>
struct WideCfg {
    static constexpr int A_TILE_BYTES = BM * KB * 2;
    static constexpr int B_TILE_BYTES = TNW * KB * 2;
    static constexpr int STAGE_BYTES = TERMS * (A_TILE_BYTES + B_TILE_BYTES);
    static constexpr int STAGES_FIT = (SMEM_LIMIT - 1024 /*align*/ - 512 /*barriers*/) / STAGE_BYTES;
    static constexpr int STAGES = STAGES_FIT > 12 ? 12 : STAGES_FIT;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 512;
    static_assert(STAGES >= 2, "pipeline depth");
};

struct TmapWideSet {
    CUtensorMap Pa[2];  // P, boxes of 128 rows: the A operand
    CUtensorMap Qa[2];  // Q, 128 rows: A of a dual product's second half
    CUtensorMap Pb[2];  // P, 256 rows: B of a dual product's second half
    CUtensorMap Qb[2];  // Q, 256 rows: the B operand
};

// Wide tiles of an nt x nt grid of 128-blocks: tile row bi holds bj = 0 .. bi / 2.
__host__ __device__ inline int64_t wide_tile_count(int64_t nt) {
    const int64_t m = nt / 2;
    return (nt % 2 == 0) ? m * (m + 1) : (m + 1) * (m + 1);
}
// First tile of tile row bi in row-major order.
__device__ __forceinline__ int64_t wide_row_start(int64_t bi) {
    const int64_t m = bi / 2;
    return (bi % 2 == 0) ? m * (m + 1) : (m + 1) * (m + 1);
}

// Tile t in grouped order: tile rows G at a time, each group walked column by
// column (G = 0: row by row).
__device__ __forceinline__ void wide_decode(int64_t t, int64_t nt, int64_t G, int64_t& bi, int64_t& bj) {
    int64_t m = static_cast<int64_t>((sqrt(4.0 * static_cast<double>(t) + 1.0) - 1.0) * 0.5);
    while ((m + 1) * (m + 2) <= t) ++m;
    while (m * (m + 1) > t) --m;  // rows 2m and 2m + 1 start at m (m + 1) and (m + 1)^2
    if (t < m * (m + 1) + m + 1) {
        bi = 2 * m;
        bj = t - m * (m + 1);
    } else {
        bi = 2 * m + 1;
        bj = t - (m + 1) * (m + 1);
    }
    if (G <= 0) return;
    const int64_t r0 = (bi / G) * G;
    const int64_t r1 = r0 + G < nt ? r0 + G : nt;
    const int64_t h = r1 - r0;
    int64_t u = t - wide_row_start(r0);
    const int64_t full = r0 / 2 + 1;  // columns bj <= r0 / 2 hold all h rows of the group
    if (u < full * h) {
        bi = r0 + u % h;
        bj = u / h;
        return;
    }
    u -= full * h;
    int64_t c = full;  // column c holds rows 2c .. r1 - 1
    while (u >= r1 - 2 * c) {
        u -= r1 - 2 * c;
        ++c;
    }
    bj = c;
    bi = 2 * c + u;
}

constexpr int W_EPI_WARPS = 8;
constexpr int W_THREADS = 64 + 32 * W_EPI_WARPS;
constexpr uint32_t W_TMEM_COLS = 2 * TNW;  // two accumulator slots

template <int KB>
__device__ __forceinline__ uint64_t sdesc_kb(uint32_t saddr) {
    if constexpr (KB == 64)
        return sdesc_kmajor_sw128(saddr);
    else
        return sdesc_kmajor_sw64(saddr);
}

template <int TERMS, int NPROD, bool BF16, int CHUNK, int KB>
__global__ void __launch_bounds__(W_THREADS, 1)
    tc_wide_kernel(const __grid_constant__ TmapWideSet tm, const EpiParams ep, int group_rows, int num_tiles,
                   int* err) {
    using Cfg = WideCfg<TERMS, KB>;
    constexpr int STAGES = Cfg::STAGES;
    constexpr int STAGE_BYTES = Cfg::STAGE_BYTES;
    constexpr int A_TILE_BYTES = Cfg::A_TILE_BYTES;
    constexpr int B_TILE_BYTES = Cfg::B_TILE_BYTES;
    constexpr uint32_t IDESC = idesc_f16(BM, TNW, BF16);

    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw_addr = smem_u32(smem_raw);
    uint8_t* smem = smem_raw + ((1024u - (raw_addr & 1023u)) & 1023u);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
    uint64_t* empty = full + STAGES;
    uint64_t* acc_full = empty + STAGES;
    uint64_t* acc_empty = acc_full + 2;
    uint64_t* drain = acc_empty + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    volatile int* issued_slot = abort_flag + 1;

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int64_t nt = ep.np / BM;
    const int kb_half = ep.np / KB;
    const int kb_total = kb_half * (ep.dual ? 2 : 1);
    const int nchunks = (kb_total + CHUNK - 1) / CHUNK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], W_EPI_WARPS);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        *issued_slot = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, W_TMEM_COLS);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---- TMA producer ----
        for (int t = 0; t < TERMS; ++t) {
            tma_prefetch_desc(&tm.Pa[t]);
            tma_prefetch_desc(&tm.Qb[t]);
        }
        int g = 0;
        bool stop = false;
        for (int tile = blockIdx.x; tile < num_tiles && !stop; tile += gridDim.x) {
            int64_t bi, bj;
            wide_decode(tile, nt, group_rows, bi, bj);
            const int row_a = static_cast<int>(bi * BM);
            const int row_b = static_cast<int>(bj * TNW);
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
                const bool second = kb >= kb_half;  // dual product: Q's rows against P's rows
                const CUtensorMap* ma = second ? tm.Qa : tm.Pa;
                const CUtensorMap* mb = second ? tm.Pb : tm.Qb;
                const int kx = (second ? kb - kb_half : kb) * KB;
                mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
#pragma unroll
                for (int t = 0; t < TERMS; ++t) tma_load_2d(st + t * A_TILE_BYTES, &ma[t], &full[s], kx, row_a);
#pragma unroll
                for (int t = 0; t < TERMS; ++t)
                    tma_load_2d(st + TERMS * A_TILE_BYTES + t * B_TILE_BYTES, &mb[t], &full[s], kx, row_b);
                *issued_slot = g + 1;
            }
        }
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer: chunk after chunk into alternating TMEM slots ----
        int g = 0, gc = 0;
        bool stop = false;
        for (int tile = blockIdx.x; tile < num_tiles && !stop; tile += gridDim.x) {
            for (int c = 0; c < nchunks; ++c, ++gc) {
                const int slot = gc & 1;
                const uint32_t use_ph = static_cast<uint32_t>(gc >> 1) & 1u;
                if (!mbar_wait_bounded(&acc_empty[slot], use_ph ^ 1u)) {
                    record_error(err, abort_flag, DEVERR_MMA_WAIT);
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t acc = tmem + static_cast<uint32_t>(slot * TNW);
                const int kb0 = c * CHUNK;
                const int kb1 = kb0 + CHUNK < kb_total ? kb0 + CHUNK : kb_total;
                for (int kb = kb0; kb < kb1; ++kb, ++g) {
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
#pragma unroll
                    for (int k = 0; k < KB / 16; ++k) {
#pragma unroll
                        for (int pi = 0; pi < NPROD; ++pi) {
                            const uint64_t ad = sdesc_kb<KB>(base + prod_a(pi) * A_TILE_BYTES + k * 32);
                            const uint64_t bd =
                                sdesc_kb<KB>(base + TERMS * A_TILE_BYTES + prod_b(pi) * B_TILE_BYTES + k * 32);
                            umma_f16(acc, ad, bd, IDESC, (kb > kb0 || k != 0 || pi != 0) ? 1u : 0u);
                        }
                    }
                    umma_commit(&empty[s]);
                }
                if (stop) break;
                umma_commit(&acc_full[slot]);
            }
        }
    } else if (warp >= 2) {
        // ---- epilogue: 128 running sums per thread ----
        const int q4 = warp & 3;
        const int half = (warp - 2) >> 2;
        const uint32_t lane_base = tmem + (static_cast<uint32_t>(q4 * 32) << 16) + static_cast<uint32_t>(half * 128);
        int gc = 0;
        bool stop = false;
        for (int tile = blockIdx.x; tile < num_tiles && !stop; tile += gridDim.x) {
            TileInfo ti;
            wide_decode(tile, nt, group_rows, ti.bi, ti.bj);
            ti.blk.row_base = 0;
            ti.blk.np = ep.np;
            ti.blk.n = ep.n;
            ti.blk.col_base = 0;
            ti.blk.x_off = 0;
            ti.blk.up_dev = ep.up_dev;
            float sum[128];
            for (int c = 0; c < nchunks; ++c, ++gc) {
                const int slot = gc & 1;
                const uint32_t ph = static_cast<uint32_t>(gc >> 1) & 1u;
                if (!mbar_wait_warp(&acc_full[slot], ph)) {
                    record_error(err, abort_flag, DEVERR_EPI_WAIT);
                    stop = true;
                    break;
                }
                if (warp_flag(abort_flag)) {
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t taddr = lane_base + static_cast<uint32_t>(slot * TNW);
                if (c == 0) {
#pragma unroll
                    for (int r = 0; r < 4; ++r)
                        tmem_ld_32cols(taddr + 32u * r, *reinterpret_cast<float(*)[32]>(sum + 32 * r));
                } else {
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        float w[32];
                        tmem_ld_32cols(taddr + 32u * r, w);
#pragma unroll
                        for (int j = 0; j < 32; ++j) sum[32 * r + j] += w[j];
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&acc_empty[slot]);
            }
            if (stop) break;
            const int64_t p0 = ti.bi * BM + q4 * 32;
            const int64_t qbase = ti.bj * TNW + half * 128;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int64_t q0 = qbase + 32 * r;
                if (q0 > p0 + 31) continue;  // above the diagonal: owned by the mirror
                // The storage format follows the operand type (ep.fmt is FP16 for
                // FP16 operands, BF16 for BF16 ones): one epilogue per instantiation.
                epilogue_run<BF16 ? FMT_BF16 : FMT_F16>(ep, ti, p0, q0,
                                                        *reinterpret_cast<float(*)[32]>(sum + 32 * r));
            }
        }
    }

    // ---- teardown ----
    tc_fence_before();
    __syncthreads();
    if (*abort_flag) {
        if (warp == 1 && lane == 0) {
            umma_commit(drain);
            if (!mbar_wait_bounded(drain, 0)) atomicCAS(err, 0, DEVERR_DRAIN_WAIT);
        }
        if (warp == 0 && lane == 0) {
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
        tmem_dealloc(tmem, W_TMEM_COLS);
    }
}

template <int TERMS, int NPROD, bool BF16, int CHUNK, int KB>
psdgb_status launch_wide(DeviceState* ds, const SplitMat& P, const SplitMat& Q, int64_t np, const EpiParams& ep,
                         cudaStream_t s) {
    using Cfg = WideCfg<TERMS, KB>;
    auto kern = tc_wide_kernel<TERMS, NPROD, BF16, CHUNK, KB>;
    static bool configured = false;
    if (!configured) {
        PSDGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM_BYTES));
        configured = true;
    }
    TmapWideSet tm;
    for (int t = 0; t < 2; ++t) {
        void* pb = (t < TERMS) ? P.term[t] : P.term[0];
        void* qb = (t < TERMS) ? Q.term[t] : Q.term[0];
        if (!make_tmap(&tm.Pa[t], pb, np, np, BF16, BM, KB) || !make_tmap(&tm.Qa[t], qb, np, np, BF16, BM, KB) ||
            !make_tmap(&tm.Pb[t], pb, np, np, BF16, TNW, KB) || !make_tmap(&tm.Qb[t], qb, np, np, BF16, TNW, KB)) {
            set_error("cuTensorMapEncodeTiled failed");
            return PSDGB_ERR_CUDA;
        }
    }
    const int64_t num_tiles = wide_tile_count(np / BM);
    if (num_tiles <= 0) return PSDGB_OK;
    const int grid = num_tiles < sm_budget(ds) ? static_cast<int>(num_tiles) : sm_budget(ds);
    kern<<<static_cast<unsigned>(grid), W_THREADS, Cfg::SMEM_BYTES, s>>>(tm, ep, g_tile_group_rows,
                                                                      static_cast<int>(num_tiles), ds->d_error);
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    return PSDGB_OK;
}

}  // namespace

// FP32-class two-term precisions accumulate K in chunks of 16 K blocks; one-term precisions take a tile's whole K as one chunk.
// Three-term precisions are not served here.
psdgb_status gemm_tc_wide(DeviceState* ds, int precision, const SplitMat& P, const SplitMat& Q, int64_t np,
                          const EpiParams& ep, cudaStream_t s) {
    constexpr int WHOLE = 1 << 20;
    const bool one_term = precision == PSDGB_PREC_FP16 || precision == PSDGB_PREC_BF16;
    const int kb = g_wide_kblock > 0 ? g_wide_kblock : (one_term ? 64 : 32);
    if (kb == 32) {
        switch (precision) {
            case PSDGB_PREC_FP16: return launch_wide<1, 1, false, WHOLE, 32>(ds, P, Q, np, ep, s);
            case PSDGB_PREC_BF16: return launch_wide<1, 1, true, WHOLE, 32>(ds, P, Q, np, ep, s);
            case PSDGB_PREC_FP16X3: return launch_wide<2, 3, false, 32, 32>(ds, P, Q, np, ep, s);
            case PSDGB_PREC_BF16X3: return launch_wide<2, 3, true, 32, 32>(ds, P, Q, np, ep, s);
            default: break;
        }
    }
    switch (precision) {
        case PSDGB_PREC_FP16: return launch_wide<1, 1, false, WHOLE, 64>(ds, P, Q, np, ep, s);
        case PSDGB_PREC_BF16: return launch_wide<1, 1, true, WHOLE, 64>(ds, P, Q, np, ep, s);
        case PSDGB_PREC_FP16X3: return launch_wide<2, 3, false, 16, 64>(ds, P, Q, np, ep, s);
        case PSDGB_PREC_BF16X3: return launch_wide<2, 3, true, 16, 64>(ds, P, Q, np, ep, s);
        default: break;
    }
    set_error("gemm_tc_wide: precision not served by 128 x 256 tiles");
    return PSDGB_ERR_UNSUPPORTED;
}

int g_wide_kblock = 0;

}  // namespace psdgb
