// gemm_tc2.cu — symmetric filter products of one matrix on CTA pairs.
//
// The same products as gemm_tc.cu (C = P * Q of two symmetric, commuting
// matrices on the tiles bi >= bj; split-precision operand terms; the fused
// epilogue of epilogue_tile), replacing the reference's cublasSgemm /
// cublasGemmEx chain (src/composite_FP32.cu:103-115,150;
// src/composite_FP16.cu:118-163,218-227; src/composite_FP32_emulated.cu:108-153,210-221).
//
// A cluster of two CTAs on the two SMs of a pair owns a 256 x 128 tile: P's
// tile rows 2I and 2I + 1 against Q's tile row bj.  CTA r loads its 128 rows
// of P (tile row 2I + r) and 64 of Q's 128 rows; one tcgen05.mma.cta_group::2
// per term product and 16-wide K slice, issued by the even CTA, multiplies the
// whole tile, and each CTA's TMEM receives the 128 x 128 accumulator of its own
// tile row.  Per 64-wide K block and operand term an SM reads 24 KB of
// operand tiles from shared memory instead of the 32 KB of a lone 128 x 128
// tile, which is what bounds the single-CTA kernel.
//
// Pair tile I covers columns bj <= 2I + 1; for bj = 2I + 1 the even CTA's tile
// lies above the diagonal and its epilogue stores nothing (1.5 % of the MMA
// work at n = 8192); with an odd tile count the odd CTA of the last pair row
// multiplies zero rows (TMA fills rows past the matrix with zeros) and stores
// nothing.
//
// Synchronisation (barriers at the same offsets in both CTAs):
//   full[s]      even CTA's: its producer expects both CTAs' bytes, both CTAs'
//                TMA loads count their bytes on it;
//   empty[s]     each CTA's: the MMA commit is multicast to both;
//   acc_full[b]  each CTA's: the MMA commit is multicast to both;
//   acc_empty[b] even CTA's: both CTAs' epilogue warps arrive on it.
// Every wait is bounded; a CTA that gives up records a DeviceError and falls
// through to the teardown, where both CTAs meet at a cluster barrier before
// either frees its TMEM or exits, so no CTA leaves while its peer may still
// touch its shared memory.
#include "tc_kernel.cuh"

namespace psdgb {

namespace {

template <int TERMS>
struct PairCfg {
    static constexpr int STAGE_BYTES = TERMS * (TILE_BYTES + HALF_TILE_BYTES);
    static constexpr int STAGES_FIT = (SMEM_LIMIT - 1024 /*align*/ - 512 /*barriers*/) / STAGE_BYTES;
    static constexpr int STAGES = STAGES_FIT > 12 ? 12 : STAGES_FIT;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 512;
    static_assert(STAGES >= 2, "pipeline depth");
};

struct TmapPairSet {
    CUtensorMap Pa[3];  // P, boxes of 128 rows: the A operand
    CUtensorMap Qa[3];  // Q, 128 rows: the A operand of a dual product's second half
    CUtensorMap Pb[3];  // P, 64 rows: the B operand of a dual product's second half
    CUtensorMap Qb[3];  // Q, 64 rows: the B operand
};

// Pair tiles of an nt x nt tile grid: pair row I (tile rows 2I, 2I + 1) holds
// the columns bj = 0 .. min(2I + 1, nt - 1).
__host__ __device__ inline int64_t pair_tile_count(int64_t nt) {
    const int64_t rows = (nt + 1) / 2;
    return (nt % 2 == 0) ? rows * (rows + 1) : (rows - 1) * rows + nt;
}

// Pair tile t in grouped order (as grouped_decode for single tiles): pair rows
// G at a time, each group walked column by column; G = 0 walks row by row.
__device__ __forceinline__ void pair_decode(int64_t t, int64_t nt, int64_t G, int64_t& I, int64_t& bj) {
    const int64_t rows = (nt + 1) / 2;
    int64_t i = static_cast<int64_t>((sqrt(4.0 * static_cast<double>(t) + 1.0) - 1.0) * 0.5);
    while ((i + 1) * (i + 2) <= t) ++i;
    while (i * (i + 1) > t) --i;  // pair row i starts at tile i (i + 1)
    if (G <= 0) {
        I = i;
        bj = t - i * (i + 1);
        return;
    }
    const int64_t r0 = (i / G) * G;
    const int64_t h = (r0 + G < rows ? r0 + G : rows) - r0;
    int64_t u = t - r0 * (r0 + 1);
    if (u < 2 * r0 * h) {  // the full columns left of the group's own triangle
        bj = u / h;
        I = r0 + u % h;
        return;
    }
    u -= 2 * r0 * h;
    int64_t c = 0;  // column 2 r0 + c of the group holds the pair rows r0 + c / 2 .. r0 + h - 1
    while (u >= h - c / 2) {
        u -= h - c / 2;
        ++c;
    }
    bj = 2 * r0 + c;
    I = r0 + c / 2 + u;
}

template <int TERMS, int NPROD, bool BF16, int ACC_SPLIT, int ACC_BUFS>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(THREADS, 1)
    tc_pair_kernel(const __grid_constant__ TmapPairSet tm, const EpiParams ep, int group_rows, int num_pairs,
                   int* err) {
    using Cfg = PairCfg<TERMS>;
    constexpr int STAGES = Cfg::STAGES;
    constexpr int STAGE_BYTES = Cfg::STAGE_BYTES;
    constexpr uint32_t IDESC = idesc_f16(2 * BM, BN, BF16);
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
    const uint32_t rank = cluster_ctarank();
    const bool leader = rank == 0;
    const int cluster = static_cast<int>(blockIdx.x >> 1), num_clusters = static_cast<int>(gridDim.x >> 1);
    const int64_t nt = ep.np / BM;
    const int kb_half = ep.np / BK;
    const int kb_total = kb_half * (ep.dual ? 2 : 1);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < ACC_BUFS; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 2 * EPI_WARPS);  // every epilogue warp of both CTAs
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        *issued_slot = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc_pair(tmem_slot, TMEM_COLS);
        tmem_relinquish_pair();
    }
    tc_fence_before();
    cluster_sync_all();  // both CTAs' barriers exist before either signals the other
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t full_leader = mapa_shared(smem_u32(full), 0);
    const uint32_t acc_empty_leader = mapa_shared(smem_u32(acc_empty), 0);

    if (warp == 0 && lane == 0) {
        // ---- TMA producer (both CTAs) ----
        for (int t = 0; t < TERMS; ++t) {
            tma_prefetch_desc(&tm.Pa[t]);
            tma_prefetch_desc(&tm.Qb[t]);
        }
        int g = 0;
        bool stop = false;
        for (int pt = cluster; pt < num_pairs && !stop; pt += num_clusters) {
            int64_t I, bj;
            pair_decode(pt, nt, group_rows, I, bj);
            const int row_a = static_cast<int>((2 * I + rank) * BM);
            const int row_b = static_cast<int>(bj * BN + rank * (BN / 2));
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
                // Second half of a dual product: Q's rows against P's rows.
                const bool second = kb >= kb_half;
                const CUtensorMap* ma = second ? tm.Qa : tm.Pa;
                const CUtensorMap* mb = second ? tm.Pb : tm.Qb;
                const int kx = (second ? kb - kb_half : kb) * BK;
                if (leader) mbar_arrive_expect_tx(&full[s], 2 * STAGE_BYTES);
                const uint32_t fb = full_leader + 8u * static_cast<uint32_t>(s);
#pragma unroll
                for (int t = 0; t < TERMS; ++t) tma_load_2d_pair(st + t * TILE_BYTES, &ma[t], fb, kx, row_a);
#pragma unroll
                for (int t = 0; t < TERMS; ++t)
                    tma_load_2d_pair(st + TERMS * TILE_BYTES + t * HALF_TILE_BYTES, &mb[t], fb, kx, row_b);
                *issued_slot = g + 1;
            }
        }
    } else if (warp == 1 && lane == 0 && leader) {
        // ---- MMA issuer (even CTA) ----
        int g = 0, it = 0;
        bool stop = false;
        for (int pt = cluster; pt < num_pairs && !stop; pt += num_clusters, ++it) {
            const int buf = it % ACC_BUFS;
            const uint32_t use_ph = static_cast<uint32_t>(it / ACC_BUFS) & 1u;
            if (!mbar_wait_cluster_bounded(&acc_empty[buf], use_ph ^ 1u)) {
                record_error(err, abort_flag, DEVERR_MMA_WAIT);
                break;
            }
            tc_fence_after();
            const uint32_t acc_base = tmem + static_cast<uint32_t>(buf * ACC_SPLIT * BN);
            for (int kb = 0; kb < kb_total; ++kb, ++g) {
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
                const uint32_t acc = acc_base + static_cast<uint32_t>((kb % ACC_SPLIT) * BN);
#pragma unroll
                for (int k = 0; k < BK / 16; ++k) {
#pragma unroll
                    for (int pi = 0; pi < NPROD; ++pi) {
                        const uint64_t ad = sdesc_kmajor_sw128(base + prod_a(pi) * TILE_BYTES + k * 32);
                        const uint64_t bd =
                            sdesc_kmajor_sw128(base + TERMS * TILE_BYTES + prod_b(pi) * HALF_TILE_BYTES + k * 32);
                        umma_f16_pair(acc, ad, bd, IDESC, (kb >= ACC_SPLIT || k != 0 || pi != 0) ? 1u : 0u);
                    }
                }
                umma_commit_pair_mc(&empty[s], 0x3);
            }
            if (stop) break;
            umma_commit_pair_mc(&acc_full[buf], 0x3);
        }
    } else if (warp >= 2) {
        // ---- epilogue (both CTAs, each on its own tile row) ----
        const int q4 = warp & 3;
        int it = 0;
        for (int pt = cluster; pt < num_pairs; pt += num_clusters, ++it) {
            int64_t I, bj;
            pair_decode(pt, nt, group_rows, I, bj);
            const int buf = it % ACC_BUFS;
            const uint32_t use_ph = static_cast<uint32_t>(it / ACC_BUFS) & 1u;
            if (!mbar_wait_cluster_warp(&acc_full[buf], use_ph)) {
                record_error(err, abort_flag, DEVERR_EPI_WAIT);
                break;
            }
            if (warp_flag(abort_flag)) break;
            tc_fence_after();
            const int64_t bi = 2 * I + rank;
            if (bi < nt) {
                TileInfo ti;
                ti.bi = bi;
                ti.bj = bj;
                ti.blk.row_base = 0;
                ti.blk.np = ep.np;
                ti.blk.n = ep.n;
                ti.blk.col_base = 0;
                ti.blk.x_off = 0;
                ti.blk.up_dev = ep.up_dev;
                const int64_t p0 = bi * BM + q4 * 32;
                const uint32_t tmem_row =
                    tmem + (static_cast<uint32_t>(q4 * 32) << 16) + static_cast<uint32_t>(buf * ACC_SPLIT * BN);
                const int nacc = kb_total < ACC_SPLIT ? kb_total : ACC_SPLIT;
                epilogue_tile<BF16 ? FMT_BF16 : FMT_F16, ACC_SPLIT>(ep, ti, tmem_row, p0, nacc);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive_cluster(acc_empty_leader + 8u * static_cast<uint32_t>(buf));
        }
    }

    // ---- teardown ----
    tc_fence_before();
    __syncthreads();
    if (*abort_flag) {
        if (leader && warp == 1 && lane == 0) {
            // Wait until every pair MMA issued so far has completed.
            umma_commit_pair(drain);
            if (!mbar_wait_bounded(drain, 0)) atomicCAS(err, 0, DEVERR_DRAIN_WAIT);
        }
        if (leader && warp == 0 && lane == 0) {
            // Wait for both CTAs' loads of the last STAGES issued K blocks.
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
    cluster_sync_all();  // neither CTA frees TMEM or exits while the other may still use it
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc_pair(tmem, TMEM_COLS);
    }
}

template <int TERMS, int NPROD, bool BF16, int ACC_SPLIT, int ACC_BUFS>
psdgb_status launch_pair(DeviceState* ds, const SplitMat& P, const SplitMat& Q, int64_t np, const EpiParams& ep,
                         cudaStream_t s) {
    using Cfg = PairCfg<TERMS>;
    auto kern = tc_pair_kernel<TERMS, NPROD, BF16, ACC_SPLIT, ACC_BUFS>;
    static int max_clusters = 0;  // co-resident clusters, per instantiation and process
    if (max_clusters == 0) {
        PSDGB_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::SMEM_BYTES));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(static_cast<unsigned>(2 * (ds->sm_count / 2)), 1, 1);
        cfg.blockDim = dim3(THREADS, 1, 1);
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
            set_error("gemm_tc2: no CTA pair fits on this device");
            return PSDGB_ERR_UNSUPPORTED;
        }
        max_clusters = n;
    }
    TmapPairSet tm;
    for (int t = 0; t < 3; ++t) {
        void* pb = (t < TERMS) ? P.term[t] : P.term[0];
        void* qb = (t < TERMS) ? Q.term[t] : Q.term[0];
        if (!make_tmap(&tm.Pa[t], pb, np, np, BF16, BM) || !make_tmap(&tm.Qa[t], qb, np, np, BF16, BM) ||
            !make_tmap(&tm.Pb[t], pb, np, np, BF16, BN / 2) || !make_tmap(&tm.Qb[t], qb, np, np, BF16, BN / 2)) {
            set_error("cuTensorMapEncodeTiled failed");
            return PSDGB_ERR_CUDA;
        }
    }
    const int64_t num_pairs = pair_tile_count(np / BM);
    if (num_pairs <= 0) return PSDGB_OK;
    int clusters = num_pairs < max_clusters ? static_cast<int>(num_pairs) : max_clusters;
    if (clusters > sm_budget(ds) / 2) clusters = sm_budget(ds) / 2 > 0 ? sm_budget(ds) / 2 : 1;
    kern<<<static_cast<unsigned>(2 * clusters), THREADS, Cfg::SMEM_BYTES, s>>>(tm, ep, g_tile_group_rows,
                                                                             static_cast<int>(num_pairs), ds->d_error);
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    return PSDGB_OK;
}

template <int TERMS, int NPROD, bool BF16>
psdgb_status launch_pair_acc(DeviceState* ds, int acc_mode, const SplitMat& P, const SplitMat& Q, int64_t np,
                             const EpiParams& ep, cudaStream_t s) {
    switch (acc_mode) {
        case ACC_4X1: return launch_pair<TERMS, NPROD, BF16, 4, 1>(ds, P, Q, np, ep, s);
        case ACC_2X2: return launch_pair<TERMS, NPROD, BF16, 2, 2>(ds, P, Q, np, ep, s);
        case ACC_1X4: return launch_pair<TERMS, NPROD, BF16, 1, 4>(ds, P, Q, np, ep, s);
        default: break;
    }
    set_error("gemm_tc2: unknown accumulator mode");
    return PSDGB_ERR_INVALID_ARGUMENT;
}

}  // namespace

psdgb_status gemm_tc_pair(DeviceState* ds, int precision, int acc_mode, const SplitMat& P, const SplitMat& Q,
                          int64_t np, const EpiParams& ep, cudaStream_t s) {
    switch (precision) {
        case PSDGB_PREC_FP16: return launch_pair_acc<1, 1, false>(ds, acc_mode, P, Q, np, ep, s);
        case PSDGB_PREC_BF16: return launch_pair_acc<1, 1, true>(ds, acc_mode, P, Q, np, ep, s);
        case PSDGB_PREC_FP16X3: return launch_pair_acc<2, 3, false>(ds, acc_mode, P, Q, np, ep, s);
        case PSDGB_PREC_BF16X3: return launch_pair_acc<2, 3, true>(ds, acc_mode, P, Q, np, ep, s);
        case PSDGB_PREC_BF16X6: return launch_pair_acc<3, 6, true>(ds, acc_mode, P, Q, np, ep, s);
        case PSDGB_PREC_BF16X9: return launch_pair_acc<3, 9, true>(ds, acc_mode, P, Q, np, ep, s);
        default: break;
    }
    set_error("gemm_tc2: unknown precision");
    return PSDGB_ERR_INVALID_ARGUMENT;
}

int g_tile_shape = -1;

}  // namespace psdgb
