// gemm_pairwide.cu — symmetric filter products of one matrix on CTA pairs
// with 256 x 256 tiles.
//
// The products, operands and fused epilogue of gemm_wide.cu (C = P * Q of two
// symmetric, commuting matrices on the lower triangle; split-precision operand
// terms; K accumulated in chunks whose partial sums the epilogue adds in FP32
// registers), replacing the reference's cublasSgemm / cublasGemmEx chain
// (src/composite_FP32.cu:103-115,150; src/composite_FP16.cu:118-163,218-227),
// with the CTA-pair mechanics of gemm_tc2.cu: a cluster of two CTAs on the two
// SMs of a pair owns a 256 x 256 tile (P's tile rows 2I, 2I + 1 against Q's
// tile rows 2J, 2J + 1, J <= I).  CTA r loads its 128 rows of P and its 128 of
// Q's 256 rows; one tcgen05.mma.cta_group::2 of 256 x 256 x 16 per term product
// and K slice, issued by the even CTA, feeds both SMs, and each CTA's TMEM
// receives the 128 x 256 accumulator of its tile row.  Per K block an SM loads
// half the operand bytes of a lone 128 x 256 tile, so the ring holds more
// stages in the same shared memory.
//
// Barriers are those of gemm_tc2.cu (full[s] and acc_empty[b] counted on the
// even CTA, empty[s] and acc_full[b] arrived on both by multicast commits);
// the accumulation is that of gemm_wide.cu (two TMEM slots of 256 columns,
// K chunks drained into registers by 8 epilogue warps per CTA).  Every wait is
// bounded; both CTAs meet at a cluster barrier before freeing TMEM or exiting.
//
// The same kernel serves a block-diagonal batch: with a device list of pair
// tiles (block, I, J), the 256 x 256 tile I, J of that block (row I of pair
// tiles is the block's tile rows 2I, 2I + 1, both inside the block), its
// operands in the batch's strided layout and its K extent the block's n.
#include "tc_kernel.cuh"

namespace psdgb {

namespace {

constexpr int PW_N = 256;         // tile width (the MMA's N)
constexpr int PW_EPI_WARPS = 8;   // per CTA
constexpr int PW_THREADS = 64 + 32 * PW_EPI_WARPS;
constexpr uint32_t PW_TMEM_COLS = 2 * PW_N;

template <int TERMS, int KB>
struct PairWideCfg {
    static constexpr int A_TILE_BYTES = BM * KB * 2;  // 128 rows of P
    static constexpr int B_TILE_BYTES = BM * KB * 2;  // this CTA's 128 of Q's 256 rows
    static constexpr int STAGE_BYTES = TERMS * (A_TILE_BYTES + B_TILE_BYTES);
    static constexpr int STAGES_FIT = (SMEM_LIMIT - 1024 - 512) / STAGE_BYTES;
    static constexpr int STAGES = STAGES_FIT > 8 ? 8 : STAGES_FIT;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 512;
    static_assert(STAGES >= 2, "pipeline depth");
};

struct TmapPW {
    CUtensorMap Pa[3];  // P's term planes, boxes of 128 rows (A operand; B of a dual product's second half)
    CUtensorMap Qa[3];  // Q's term planes, 128 rows
};

template <int KB>
__device__ __forceinline__ uint64_t sdesc_pw(uint32_t saddr) {
    if constexpr (KB == 64)
        return sdesc_kmajor_sw128(saddr);
    else
        return sdesc_kmajor_sw64(saddr);
}

// Pair tile pt: from the batch's device list (gw.tiles), or the lower pair
// tiles of the single matrix ep describes, in groups of group_rows pair rows.
struct PwTile {
    int64_t I, J;
    BlockDesc blk;
    int kb_half;  // K blocks of one product half
};
template <int KB, bool GROUP>
__device__ __forceinline__ PwTile pw_tile(const GroupWork& gw, const EpiParams& ep, int pt, int group_rows) {
    PwTile t;
    if constexpr (GROUP) {
        const TileDesc td = gw.tiles[gw.reverse ? gw.reverse - 1 - pt : pt];
        t.I = td.bi;
        t.J = td.bj;
        t.blk = gw.blocks[td.block];
        TileInfo ti;
        ti.blk = t.blk;
        t.kb_half = tile_kblocks<KB>(ep, ti);
    } else {
        const int64_t nsuper = (ep.np / BM + 1) / 2;  // pair rows / columns of 256
        grouped_decode(pt, nsuper, group_rows, t.I, t.J);
        t.blk.row_base = 0;
        t.blk.np = static_cast<int>(ep.np);
        t.blk.n = static_cast<int>(ep.n);
        t.blk.col_base = 0;
        t.blk.x_off = 0;
        t.blk.up_dev = ep.up_dev;
        t.kb_half = static_cast<int>(ep.np / KB);
    }
    return t;
}

template <int TERMS, int NPROD, bool BF16, int CHUNK, int KB, bool GROUP>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(PW_THREADS, 1)
    tc_pairwide_kernel(const __grid_constant__ TmapPW tm, const EpiParams ep, const GroupWork gw, int group_rows,
                       int num_pairs, int* err) {
    using Cfg = PairWideCfg<TERMS, KB>;
    constexpr int STAGES = Cfg::STAGES;
    constexpr int STAGE_BYTES = Cfg::STAGE_BYTES;
    constexpr int A_TILE_BYTES = Cfg::A_TILE_BYTES;
    constexpr int B_TILE_BYTES = Cfg::B_TILE_BYTES;
    constexpr uint32_t IDESC = idesc_f16(2 * BM, PW_N, BF16);

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
    const uint32_t rank = cluster_ctarank();
    const bool leader = rank == 0;
    const int cluster = static_cast<int>(blockIdx.x >> 1), num_clusters = static_cast<int>(gridDim.x >> 1);
    const int dual_mult = ep.dual ? 2 : 1;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 2 * PW_EPI_WARPS);  // every epilogue warp of both CTAs
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        *issued_slot = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc_pair(tmem_slot, PW_TMEM_COLS);
        tmem_relinquish_pair();
    }
    tc_fence_before();
    cluster_sync_all();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t full_leader = mapa_shared(smem_u32(full), 0);
    const uint32_t acc_empty_leader = mapa_shared(smem_u32(acc_empty), 0);

    if (warp == 0 && lane == 0) {
        // ---- TMA producer (both CTAs) ----
        for (int t = 0; t < TERMS; ++t) {
            tma_prefetch_desc(&tm.Pa[t]);
            tma_prefetch_desc(&tm.Qa[t]);
        }
        int g = 0;
        bool stop = false;
        for (int pt = cluster; pt < num_pairs && !stop; pt += num_clusters) {
            const PwTile tl = pw_tile<KB, GROUP>(gw, ep, pt, group_rows);
            const int kb_half = tl.kb_half;
            const int kb_total = kb_half * dual_mult;
            const int row_a = static_cast<int>(tl.blk.row_base + (2 * tl.I + rank) * BM);
            const int row_b = static_cast<int>(tl.blk.row_base + (2 * tl.J + rank) * BM);
            for (int kb = 0; kb < kb_total; ++kb, ++g) {
                const int s = g % STAGES;
                const uint32_t ph = static_cast<uint32_t>(g / STAGES) & 1u;
                if (!mbar_wait_cluster_bounded(&empty[s], ph ^ 1u)) {
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
                const CUtensorMap* mb = second ? tm.Pa : tm.Qa;
                const int kx = tl.blk.col_base + (second ? kb - kb_half : kb) * KB;
                if (leader) mbar_arrive_expect_tx(&full[s], 2 * STAGE_BYTES);
                const uint32_t fb = full_leader + 8u * static_cast<uint32_t>(s);
#pragma unroll
                for (int t = 0; t < TERMS; ++t) tma_load_2d_pair(st + t * A_TILE_BYTES, &ma[t], fb, kx, row_a);
#pragma unroll
                for (int t = 0; t < TERMS; ++t)
                    tma_load_2d_pair(st + TERMS * A_TILE_BYTES + t * B_TILE_BYTES, &mb[t], fb, kx, row_b);
                *issued_slot = g + 1;
            }
        }
    } else if (warp == 1 && lane == 0 && leader) {
        // ---- MMA issuer (even CTA): chunk after chunk into alternating slots ----
        int g = 0, gc = 0;
        bool stop = false;
        for (int pt = cluster; pt < num_pairs && !stop; pt += num_clusters) {
            const int kb_total = pw_tile<KB, GROUP>(gw, ep, pt, group_rows).kb_half * dual_mult;
            const int nchunks = (kb_total + CHUNK - 1) / CHUNK;
            for (int c = 0; c < nchunks; ++c, ++gc) {
                const int slot = gc & 1;
                const uint32_t use_ph = static_cast<uint32_t>(gc >> 1) & 1u;
                if (!mbar_wait_cluster_bounded(&acc_empty[slot], use_ph ^ 1u)) {
                    record_error(err, abort_flag, DEVERR_MMA_WAIT);
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t acc = tmem + static_cast<uint32_t>(slot * PW_N);
                const int kb0 = c * CHUNK;
                const int kb1 = kb0 + CHUNK < kb_total ? kb0 + CHUNK : kb_total;
                for (int kb = kb0; kb < kb1; ++kb, ++g) {
                    const int s = g % STAGES;
                    const uint32_t ph = static_cast<uint32_t>(g / STAGES) & 1u;
                    if (!mbar_wait_cluster_bounded(&full[s], ph)) {
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
                            const uint64_t ad = sdesc_pw<KB>(base + prod_a(pi) * A_TILE_BYTES + k * 32);
                            const uint64_t bd =
                                sdesc_pw<KB>(base + TERMS * A_TILE_BYTES + prod_b(pi) * B_TILE_BYTES + k * 32);
                            umma_f16_pair(acc, ad, bd, IDESC, (kb > kb0 || k != 0 || pi != 0) ? 1u : 0u);
                        }
                    }
                    umma_commit_pair_mc(&empty[s], 0x3);
                }
                if (stop) break;
                umma_commit_pair_mc(&acc_full[slot], 0x3);
            }
        }
    } else if (warp >= 2) {
        // ---- epilogue (both CTAs): 128 running sums per thread ----
        const int q4 = warp & 3;
        const int half = (warp - 2) >> 2;
        const uint32_t lane_base = tmem + (static_cast<uint32_t>(q4 * 32) << 16) + static_cast<uint32_t>(half * 128);
        int gc = 0;
        bool stop = false;
        for (int pt = cluster; pt < num_pairs && !stop; pt += num_clusters) {
            const PwTile tl = pw_tile<KB, GROUP>(gw, ep, pt, group_rows);
            const int kb_total = tl.kb_half * dual_mult;
            const int nchunks = (kb_total + CHUNK - 1) / CHUNK;
            const int64_t J = tl.J;
            TileInfo ti;
            ti.bi = 2 * tl.I + rank;
            ti.bj = J;  // column tiles of 256
            ti.blk = tl.blk;
            float sum[128];
            for (int c = 0; c < nchunks; ++c, ++gc) {
                const int slot = gc & 1;
                const uint32_t ph = static_cast<uint32_t>(gc >> 1) & 1u;
                if (!mbar_wait_cluster_warp(&acc_full[slot], ph)) {
                    record_error(err, abort_flag, DEVERR_EPI_WAIT);
                    stop = true;
                    break;
                }
                if (warp_flag(abort_flag)) {
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t taddr = lane_base + static_cast<uint32_t>(slot * PW_N);
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
                if (lane == 0) mbar_arrive_cluster(acc_empty_leader + 8u * static_cast<uint32_t>(slot));
            }
            if (stop || ti.bi >= ti.blk.np / BM) continue;
            const int64_t p0 = ti.bi * BM + q4 * 32;
            const int64_t qbase = J * PW_N + half * 128;
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
        if (leader && warp == 1 && lane == 0) {
            umma_commit_pair(drain);
            if (!mbar_wait_bounded(drain, 0)) atomicCAS(err, 0, DEVERR_DRAIN_WAIT);
        }
        if (leader && warp == 0 && lane == 0) {
            const int issued = *issued_slot;
            for (int g = issued - STAGES; g < issued; ++g) {
                if (g < 0) continue;
                const int s = g % STAGES;
                const uint32_t ph = static_cast<uint32_t>(g / STAGES) & 1u;
                if (!mbar_wait_cluster_bounded(&full[s], ph)) atomicCAS(err, 0, DEVERR_DRAIN_WAIT);
            }
        }
        __syncthreads();
    }
    tc_fence_before();
    cluster_sync_all();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc_pair(tmem, PW_TMEM_COLS);
    }
}

// ld, rows: the operands' layout (np, np for a single matrix); gw: the
// batch's pair-tile list (null tiles: the single matrix's lower pair tiles).
template <int TERMS, int NPROD, bool BF16, int CHUNK, int KB, bool GROUP>
psdgb_status launch_pairwide(DeviceState* ds, const SplitMat& P, const SplitMat& Q, int64_t ld, int64_t rows,
                             const EpiParams& ep, const GroupWork& gw, int64_t num_pairs, cudaStream_t s) {
    using Cfg = PairWideCfg<TERMS, KB>;
    auto kern = tc_pairwide_kernel<TERMS, NPROD, BF16, CHUNK, KB, GROUP>;
    static int max_clusters = 0;
    if (max_clusters == 0) {
        PSDGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM_BYTES));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(static_cast<unsigned>(2 * (ds->sm_count / 2)), 1, 1);
        cfg.blockDim = dim3(PW_THREADS, 1, 1);
        cfg.dynamicSmemBytes = Cfg::SMEM_BYTES;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        PSDGB_CUDA_TRY(cudaOccupancyMaxActiveClusters(&n, kern, &cfg));
        if (n <= 0) {
            set_error("gemm_pairwide: no CTA pair fits on this device");
            return PSDGB_ERR_UNSUPPORTED;
        }
        max_clusters = n;
    }
    TmapPW tm;
    for (int t = 0; t < 3; ++t) {
        void* pb = (t < TERMS) ? P.term[t] : P.term[0];
        void* qb = (t < TERMS) ? Q.term[t] : Q.term[0];
        if (!make_tmap(&tm.Pa[t], pb, ld, rows, BF16, BM, KB) || !make_tmap(&tm.Qa[t], qb, ld, rows, BF16, BM, KB)) {
            set_error("cuTensorMapEncodeTiled failed");
            return PSDGB_ERR_CUDA;
        }
    }
    if (num_pairs <= 0) return PSDGB_OK;
    int clusters = num_pairs < max_clusters ? static_cast<int>(num_pairs) : max_clusters;
    if (clusters > sm_budget(ds) / 2) clusters = sm_budget(ds) / 2 > 0 ? sm_budget(ds) / 2 : 1;
    kern<<<static_cast<unsigned>(2 * clusters), PW_THREADS, Cfg::SMEM_BYTES, s>>>(
        tm, ep, gw, g_tile_group_rows, static_cast<int>(num_pairs), ds->d_error);
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    return PSDGB_OK;
}

}  // namespace

// One-, two- and three-term precisions.  Three BF16 terms take K blocks of 32
// (64-byte swizzle): 48 KB stages, four of them in shared memory; chunks of
// 32 K blocks (K = 1024) per TMEM slot, as for the others.
namespace {

template <bool GROUP>
psdgb_status pairwide_dispatch(DeviceState* ds, int precision, const SplitMat& P, const SplitMat& Q, int64_t ld,
                               int64_t rows, const EpiParams& ep, const GroupWork& gw, int64_t num_pairs,
                               cudaStream_t s) {
    constexpr int WHOLE = 1 << 20;
    // K blocks of 64 (128-byte swizzle, 3 stages of 64 KB for two terms)
    // measured faster here than blocks of 32 (n = 8192, fp16x3: 1.87 vs 1.81
    // PFLOP/s); PSDGB_TUNE_WIDE_KBLOCK = 32 selects the latter.
    if (g_wide_kblock == 32 && (precision == PSDGB_PREC_FP16X3 || precision == PSDGB_PREC_BF16X3)) {
        if (precision == PSDGB_PREC_FP16X3)
            return launch_pairwide<2, 3, false, 32, 32, GROUP>(ds, P, Q, ld, rows, ep, gw, num_pairs, s);
        return launch_pairwide<2, 3, true, 32, 32, GROUP>(ds, P, Q, ld, rows, ep, gw, num_pairs, s);
    }
    switch (precision) {
        case PSDGB_PREC_FP16: return launch_pairwide<1, 1, false, WHOLE, 64, GROUP>(ds, P, Q, ld, rows, ep, gw, num_pairs, s);
        case PSDGB_PREC_BF16: return launch_pairwide<1, 1, true, WHOLE, 64, GROUP>(ds, P, Q, ld, rows, ep, gw, num_pairs, s);
        case PSDGB_PREC_FP16X3:
            return launch_pairwide<2, 3, false, 16, 64, GROUP>(ds, P, Q, ld, rows, ep, gw, num_pairs, s);
        case PSDGB_PREC_BF16X3:
            return launch_pairwide<2, 3, true, 16, 64, GROUP>(ds, P, Q, ld, rows, ep, gw, num_pairs, s);
        case PSDGB_PREC_BF16X6:
            return launch_pairwide<3, 6, true, 32, 32, GROUP>(ds, P, Q, ld, rows, ep, gw, num_pairs, s);
        case PSDGB_PREC_BF16X9:
            return launch_pairwide<3, 9, true, 32, 32, GROUP>(ds, P, Q, ld, rows, ep, gw, num_pairs, s);
        default: break;
    }
    set_error("gemm_tc_pairwide: precision not served by 256 x 256 pair tiles");
    return PSDGB_ERR_UNSUPPORTED;
}

}  // namespace

psdgb_status gemm_tc_pairwide(DeviceState* ds, int precision, const SplitMat& P, const SplitMat& Q, int64_t np,
                              const EpiParams& ep, cudaStream_t s) {
    const int64_t nsuper = (np / BM + 1) / 2;
    const GroupWork none{nullptr, nullptr, 0};
    return pairwide_dispatch<false>(ds, precision, P, Q, np, np, ep, none, nsuper * (nsuper + 1) / 2, s);
}

bool pairwide_supported(int precision) {
    return precision == PSDGB_PREC_FP16 || precision == PSDGB_PREC_BF16 || precision == PSDGB_PREC_FP16X3 ||
           precision == PSDGB_PREC_BF16X3 || precision == PSDGB_PREC_BF16X6 || precision == PSDGB_PREC_BF16X9;
}

psdgb_status gemm_tc_pairwide_group(DeviceState* ds, int precision, const SplitMat& P, const SplitMat& Q, int64_t ld,
                                    int64_t rows, const EpiParams& ep, const GroupWork& gw, int64_t num_pairs,
                                    cudaStream_t s) {
    return pairwide_dispatch<true>(ds, precision, P, Q, ld, rows, ep, gw, num_pairs, s);
}

}  // namespace psdgb
