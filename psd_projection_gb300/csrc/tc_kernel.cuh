// tc_kernel.cuh — pieces shared by the tensor-core product kernels
// (gemm_tc.cu: one CTA per 128 x 128 tile; gemm_tc2.cu: a CTA pair per
// 256 x 128 tile): tile geometry, tile-list decoding, tensor maps and the
// epilogue that turns an FP32 accumulator tile into the next operand.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include "epilogue.cuh"
#include "internal.h"

namespace psdgb {

// Tensor map over a row-major plane of `rows` rows with row stride ld (both
// in elements; the inner extent is ld), boxes of box_cols columns x box_rows
// rows: 64 columns (128-byte rows) with the 128-byte swizzle, 32 columns
// (64-byte rows) with the 64-byte swizzle (gemm_tc.cu).
bool make_tmap(CUtensorMap* tm, void* base, int64_t ld, int64_t rows, bool bf16, int box_rows, int box_cols = 64);
// The same over a one-byte (E4M3) plane: boxes of 128 columns (128-byte rows,
// 128-byte swizzle) x box_rows rows.
bool make_tmap_u8(CUtensorMap* tm, void* base, int64_t ld, int64_t rows, int box_rows);

namespace {

constexpr int BM = 128, BN = 128;
constexpr int EPI_WARPS = 4;                   // one per TMEM lane quarter
constexpr int THREADS = 64 + 32 * EPI_WARPS;  // producer warp, MMA warp, epilogue warps
constexpr int SMEM_LIMIT = 232448;             // 227 KB of dynamic shared memory per CTA

constexpr int BK = 64;                         // K block: 128-byte rows, 128-byte swizzle
constexpr int TILE_BYTES = BM * BK * 2;          // one operand term tile of 128 rows
constexpr int HALF_TILE_BYTES = TILE_BYTES / 2;  // 64 rows: one CTA's half of a pair's B operand

// Single-CTA pipeline: per K block, TERMS term tiles of P (rows bi) and of Q
// (rows bj); the ring takes as many stages as fit beside STAGING bytes of
// epilogue staging (placed after the barriers).
template <int TERMS, int STAGING = 0>
struct TcCfg {
    static constexpr int STAGE_BYTES = 2 * TERMS * TILE_BYTES;
    static constexpr int STAGES_FIT = (SMEM_LIMIT - 1024 /*align*/ - 512 /*barriers*/ - STAGING) / STAGE_BYTES;
    static constexpr int STAGES = STAGES_FIT > 12 ? 12 : STAGES_FIT;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 512 + STAGING;
    static_assert(STAGES >= 2, "pipeline depth");
};

// Bytes of shared memory an epilogue warp stages runs in: two 32 x 32 runs
// of one 16-bit plane each (store_run_full_staged, store_run_diag_staged use
// the first; the step epilogue's FP16 loads both).
constexpr int RUN_STAGE_BYTES = 2 * 32 * 64;

struct TmapSet {
    CUtensorMap P[3];
    CUtensorMap Q[3];
};

// Term product list: product i multiplies term prod_a(i) of P by term
// prod_b(i) of Q.  The first 1 / 3 / 6 / 9 products are the x1 / x3 / x6 / x9
// schemes: (0,0); (0,1), (1,0); (0,2), (2,0), (1,1); (1,2), (2,1), (2,2).
__host__ __device__ constexpr int prod_a(int i) {
    return i == 2 ? 1 : i == 4 ? 2 : i == 5 ? 1 : i == 6 ? 1 : i == 7 ? 2 : i == 8 ? 2 : 0;
}
__host__ __device__ constexpr int prod_b(int i) {
    return i == 1 ? 1 : i == 3 ? 2 : i == 5 ? 1 : i == 6 ? 2 : i == 7 ? 1 : i == 8 ? 2 : 0;
}

__device__ __forceinline__ void tri_decode(int64_t t, int64_t& bi, int64_t& bj) {
    int64_t i = static_cast<int64_t>((sqrt(8.0 * static_cast<double>(t) + 1.0) - 1.0) * 0.5);
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    while (i * (i + 1) / 2 > t) --i;
    bi = i;
    bj = t - i * (i + 1) / 2;
}

// Tile t of the lower triangle of an nt x nt tile grid in grouped order: the
// tile rows are taken G at a time and each group is walked column by column
// (bj outer, the group's rows bi inner), so the tiles that run at the same
// time (one wave = consecutive t) read G row blocks of P and about
// wave / G row blocks of Q instead of a few rows of P and every column of Q.
// Fewer distinct row blocks per wave keep more operand reads in L2.
__device__ __forceinline__ void grouped_decode(int64_t t, int64_t nt, int64_t G, int64_t& bi, int64_t& bj) {
    int64_t i, j;
    tri_decode(t, i, j);  // the row-major triangle order and this one share the groups' index ranges
    const int64_t r0 = (i / G) * G;
    const int64_t h = (r0 + G < nt ? r0 + G : nt) - r0;
    int64_t u = t - r0 * (r0 + 1) / 2;
    if (u < r0 * h) {  // the full columns left of the group's own triangle
        bj = u / h;
        bi = r0 + u % h;
        return;
    }
    u -= r0 * h;
    int64_t c = 0;  // column c of the group's triangle holds h - c tiles
    while (u >= h - c) {
        u -= h - c;
        ++c;
    }
    bj = r0 + c;
    bi = bj + u;
}

struct TileInfo {
    int64_t bi, bj;
    BlockDesc blk;
};

// Tile t of the work list: from the device tables, or (tables == null) the
// lower tiles of one block described by the epilogue parameters.
__device__ __forceinline__ TileInfo tile_info(const GroupWork& gw, const EpiParams& ep, int t) {
    TileInfo ti;
    if (gw.tiles != nullptr) {
        const TileDesc td = gw.tiles[gw.reverse ? gw.reverse - 1 - t : t];
        ti.bi = td.bi;
        ti.bj = td.bj;
        ti.blk = gw.blocks[td.block];
    } else {
        if (gw.group_rows > 0)
            grouped_decode(t, ep.np / BM, gw.group_rows, ti.bi, ti.bj);
        else
            tri_decode(t, ti.bi, ti.bj);
        ti.blk.row_base = 0;
        ti.blk.np = ep.np;
        ti.blk.n = ep.n;
        ti.blk.col_base = 0;
        ti.blk.x_off = 0;
        ti.blk.up_dev = ep.up_dev;
    }
    return ti;
}

// K blocks of one half of a tile's K loop: np / BK, or, where the operands'
// padding is zero (ep.skip_pad), only the blocks that reach into the block's
// n columns (the rest multiply zeros).  Producer, MMA issuer and epilogue
// all use this count.
// KBE: elements per K block (64 16-bit or 128 E4M3 elements: 128 bytes either way).
template <int KBE = BK>
__device__ __forceinline__ int tile_kblocks(const EpiParams& ep, const TileInfo& ti) {
    if (!ep.skip_pad) return ti.blk.np / KBE;
    const int kb = (ti.blk.n + KBE - 1) / KBE;
    return kb < 1 ? 1 : kb;
}

__device__ __forceinline__ void record_error(int* err, volatile int* abort_flag, int code) {
    *abort_flag = 1;
    atomicCAS(err, 0, code);
}

// ---- epilogue helpers ------------------------------------------------------

// Store a 32 x 32 run of the warp (lane = local row p0 + lane, columns
// q0..q0+31, every element strictly below the diagonal) and its mirror, one
// term plane at a time: the plane's 32 terms are computed once (the
// arithmetic of split_store, so both give the same bits) and written to the
// row as 16-byte vectors (four per 16-bit plane, two for the E4M3 plane) and
// to the mirror (rows q0..q0+31, column p0 + lane) element by element, which
// the warp's 32 lanes coalesce into contiguous 64-byte stores.  One plane's
// terms at a time keeps 16 words live.  (Transposing the mirror through
// shared memory to write it as vectors measured 2-3 % slower.)
template <int FMT>
__device__ __forceinline__ void store_run_full(const SplitMat& m, int64_t ld, int64_t rb, int64_t cb, int64_t p0,
                                               int64_t q0, const float (&v)[32]) {
    constexpr int NT = FMT == FMT_BF16 ? 3 : 2;  // 16-bit planes
    const int64_t p = p0 + (threadIdx.x & 31);
    const size_t row_idx = static_cast<size_t>(rb + p) * ld + cb + q0;
    const size_t mir_idx = static_cast<size_t>(rb + q0) * ld + cb + p;
    if (FMT == FMT_F16Q8) {
        uint32_t q[8];  // word j / 4: the E4M3 bytes of elements j .. j + 3, lowest first
#pragma unroll
        for (int j = 0; j < 32; j += 4) {
            const __nv_fp8x2_storage_t lo = __nv_cvt_float2_to_fp8x2(
                make_float2(v[j] * kE4M3Scale, v[j + 1] * kE4M3Scale), __NV_SATFINITE, __NV_E4M3);
            const __nv_fp8x2_storage_t hi = __nv_cvt_float2_to_fp8x2(
                make_float2(v[j + 2] * kE4M3Scale, v[j + 3] * kE4M3Scale), __NV_SATFINITE, __NV_E4M3);
            q[j / 4] = static_cast<uint32_t>(lo) | (static_cast<uint32_t>(hi) << 16);
        }
        uint8_t* plane = static_cast<uint8_t*>(m.term[2]);
        uint4* dst = reinterpret_cast<uint4*>(plane + row_idx);
        dst[0] = make_uint4(q[0], q[1], q[2], q[3]);
        dst[1] = make_uint4(q[4], q[5], q[6], q[7]);
#pragma unroll
        for (int j = 0; j < 32; ++j) plane[mir_idx + static_cast<size_t>(j) * ld] = static_cast<uint8_t>(q[j >> 2] >> ((j & 3) * 8));
    }
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        uint32_t pk[16];  // word j / 2: the terms of elements j (low half) and j + 1
#pragma unroll
        for (int j = 0; j < 32; j += 2) {
            float x0 = v[j], x1 = v[j + 1];
            if (FMT != FMT_BF16) {
                x0 *= kF16Scale;
                x1 *= kF16Scale;
            }
            uint16_t h0 = 0, h1 = 0;
#pragma unroll
            for (int u = 0; u <= t; ++u) {
                if (FMT != FMT_BF16) {
                    const __half a0 = __float2half_rn(x0), a1 = __float2half_rn(x1);
                    h0 = __half_as_ushort(a0);
                    h1 = __half_as_ushort(a1);
                    x0 -= __half2float(a0);
                    x1 -= __half2float(a1);
                } else {
                    const __nv_bfloat16 a0 = __float2bfloat16_rn(x0), a1 = __float2bfloat16_rn(x1);
                    h0 = __bfloat16_as_ushort(a0);
                    h1 = __bfloat16_as_ushort(a1);
                    x0 -= __bfloat162float(a0);
                    x1 -= __bfloat162float(a1);
                }
            }
            pk[j / 2] = static_cast<uint32_t>(h0) | (static_cast<uint32_t>(h1) << 16);
        }
        uint16_t* plane = static_cast<uint16_t*>(m.term[t]);
        uint4* dst = reinterpret_cast<uint4*>(plane + row_idx);
#pragma unroll
        for (int u = 0; u < 4; ++u) dst[u] = make_uint4(pk[4 * u], pk[4 * u + 1], pk[4 * u + 2], pk[4 * u + 3]);
#pragma unroll
        for (int j = 0; j < 32; ++j)
            plane[mir_idx + static_cast<size_t>(j) * ld] = static_cast<uint16_t>(pk[j >> 1] >> ((j & 1) * 16));
    }
}

// Staging layout of a 32 x 32 run of one 16-bit plane: row r at r * 64
// bytes, its 16-byte chunk c at chunk c ^ ((r >> 1) & 3), so that a lane
// writing its own row and 8 lanes reading two rows are both free of bank
// conflicts.
__device__ __forceinline__ uint32_t stage_off(int r, int c) {
    return static_cast<uint32_t>(r * 64 + ((c ^ ((r >> 1) & 3)) << 4));
}

// The staged run to global memory: rows row0 .. row0 + 31 (element index of
// the run's first element, row stride ld), 8 rows x 64 bytes per warp
// instruction (full 32-byte sectors) instead of 32 rows x 16 bytes.
__device__ __forceinline__ void stage_flush(const uint8_t* stage, uint16_t* plane, size_t row0, int64_t ld) {
    const int lane = threadIdx.x & 31;
    const int c = lane & 3;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int r = 8 * j + (lane >> 2);
        const uint4 w = *reinterpret_cast<const uint4*>(stage + stage_off(r, c));
        *reinterpret_cast<uint4*>(plane + row0 + static_cast<size_t>(r) * ld + 8 * c) = w;
    }
}

// Rows row0 .. row0 + 31 (32 elements each, row stride ld) of plane into the
// staging buffer, as cp.async copies of 8 rows x 64 bytes per warp
// instruction; the caller commits and waits.
__device__ __forceinline__ void stage_fetch(const uint16_t* plane, size_t row0, int64_t ld, uint8_t* buf) {
    const int lane = threadIdx.x & 31;
    const int c = lane & 3;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int r = 8 * j + (lane >> 2);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(buf + stage_off(r, c))),
                     "l"(plane + row0 + static_cast<size_t>(r) * ld + 8 * c)
                     : "memory");
    }
}
__device__ __forceinline__ void stage_fetch_wait() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
    __syncwarp();
}

// The FP16-pair values of a run of matrix M (rows of row0, stride ld) for
// this lane's row: both planes fetched coalesced through the staging buffer,
// then lo + hi times 2^-12 (load_run8's arithmetic).
__device__ __forceinline__ void stage_values_f16(const SplitMat& M, size_t row0, int64_t ld, uint8_t* stage,
                                                 float (&out)[32]) {
    const int lane = threadIdx.x & 31;
    stage_fetch(static_cast<const uint16_t*>(M.term[0]), row0, ld, stage);
    stage_fetch(static_cast<const uint16_t*>(M.term[1]), row0, ld, stage + 32 * 64);
    stage_fetch_wait();
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const uint4 h = *reinterpret_cast<const uint4*>(stage + stage_off(lane, u));
        const uint4 l = *reinterpret_cast<const uint4*>(stage + 32 * 64 + stage_off(lane, u));
        const uint32_t hw[4] = {h.x, h.y, h.z, h.w}, lw[4] = {l.x, l.y, l.z, l.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float l0 = __half2float(__ushort_as_half(static_cast<uint16_t>(lw[e] & 0xFFFFu)));
            const float l1 = __half2float(__ushort_as_half(static_cast<uint16_t>(lw[e] >> 16)));
            const float h0 = __half2float(__ushort_as_half(static_cast<uint16_t>(hw[e] & 0xFFFFu)));
            const float h1 = __half2float(__ushort_as_half(static_cast<uint16_t>(hw[e] >> 16)));
            out[8 * u + 2 * e] = ((0.f + l0) + h0) * kF16Unscale;
            out[8 * u + 2 * e + 1] = ((0.f + l1) + h1) * kF16Unscale;
        }
    }
    __syncwarp();
}

// The final reconstruction of a run through the staging buffer, one half of
// 16 columns at a time: X's run rows fetched into shared memory with
// cp.async (8 bytes a lane, 16 lanes a row), each lane's o = (X + up acc) / 2
// for its row, the rows written back as 128-byte row segments (the staged
// value of element j of row r at double r * 16 + (j ^ (r & 15))); the mirror
// goes out from each lane's own slots as 256-byte segments.  Same elements
// (q <= p < n) and arithmetic as the direct path.
__device__ __forceinline__ void final_run_staged(const EpiParams& ep, const TileInfo& ti, int64_t p0_, int64_t q0_,
                                                 const float (&v)[32], float acc_scale, uint8_t* stage) {
    // block-local row and column indices in 32 bits, element offsets in 64
    const int lane = threadIdx.x & 31;
    const int n = ti.blk.n, p0 = static_cast<int>(p0_), q0 = static_cast<int>(q0_);
    if (p0 >= n) return;  // no row of the block (warp-uniform)
    const double up = ti.blk.up_dev ? ep.up * *ti.blk.up_dev : ep.up;
    double* out = ep.out64 + ti.blk.x_off;
    const double* x = ep.x64 + ti.blk.x_off;
    double* sd = reinterpret_cast<double*>(stage);
    const int p = p0 + lane;
    const int rsub = lane >> 4, j16 = lane & 15;  // fetch / flush mapping: rows 2 i + rsub, column j16
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int qh = q0 + 16 * h;
        if (qh >= n) break;  // warp-uniform
        const int q = qh + j16;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int r = 2 * i + rsub, pr = p0 + r;
            if (q <= pr && pr < n && q < n)
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(sd + r * 16 + (j16 ^ (r & 15)))),
                             "l"(x + static_cast<int64_t>(pr) * n + q)
                             : "memory");
        }
        asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            double* slot = sd + lane * 16 + (j ^ (lane & 15));
            if (qh + j <= p && p < n && qh + j < n)
                *slot = 0.5 * (*slot + up * static_cast<double>(acc_scale * v[16 * h + j]));
        }
        __syncwarp();
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const int r = 2 * i + rsub, pr = p0 + r;
            if (q <= pr && pr < n && q < n) out[static_cast<int64_t>(pr) * n + q] = sd[r * 16 + (j16 ^ (r & 15))];
        }
        // mirror: row qh + j, column p, for qh + j < p (the lane's own slots)
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int qj = qh + j;
            if (qj < p && p < n && qj < n) out[static_cast<int64_t>(qj) * n + p] = sd[lane * 16 + (j ^ (lane & 15))];
        }
        __syncwarp();
    }
}

// The plane-t terms of the run's 32 values, two per word (element j in the
// low half of word j / 2): the arithmetic of split_store.
template <int FMT>
__device__ __forceinline__ void split_plane(const float (&v)[32], int t, uint32_t (&pk)[16]) {
#pragma unroll
    for (int j = 0; j < 32; j += 2) {
        float x0 = v[j], x1 = v[j + 1];
        if (FMT != FMT_BF16) {
            x0 *= kF16Scale;
            x1 *= kF16Scale;
        }
        uint16_t h0 = 0, h1 = 0;
#pragma unroll
        for (int u = 0; u <= t; ++u) {
            if (FMT != FMT_BF16) {
                const __half a0 = __float2half_rn(x0), a1 = __float2half_rn(x1);
                h0 = __half_as_ushort(a0);
                h1 = __half_as_ushort(a1);
                x0 -= __half2float(a0);
                x1 -= __half2float(a1);
            } else {
                const __nv_bfloat16 a0 = __float2bfloat16_rn(x0), a1 = __float2bfloat16_rn(x1);
                h0 = __bfloat16_as_ushort(a0);
                h1 = __bfloat16_as_ushort(a1);
                x0 -= __bfloat162float(a0);
                x1 -= __bfloat162float(a1);
            }
        }
        pk[j / 2] = static_cast<uint32_t>(h0) | (static_cast<uint32_t>(h1) << 16);
    }
}

// store_run_full with the rows and the mirror through the warp's staging
// buffer (stage, RUN_STAGE_BYTES): each lane writes its row's 64 bytes there
// (then its column of the mirror, one 2-byte element per row), and the warp
// writes whole row segments.  FP16 and BF16 formats.
template <int FMT>
__device__ __forceinline__ void store_run_full_staged(const SplitMat& m, int64_t ld, int64_t rb, int64_t cb,
                                                      int64_t p0, int64_t q0, const float (&v)[32], uint8_t* stage) {
    constexpr int NT = FMT == FMT_BF16 ? 3 : 2;
    const int lane = threadIdx.x & 31;
    const size_t row0 = static_cast<size_t>(rb + p0) * ld + cb + q0;
    const size_t mir0 = static_cast<size_t>(rb + q0) * ld + cb + p0;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        uint32_t pk[16];
        split_plane<FMT>(v, t, pk);
        uint16_t* plane = static_cast<uint16_t*>(m.term[t]);
#pragma unroll
        for (int u = 0; u < 4; ++u)
            *reinterpret_cast<uint4*>(stage + stage_off(lane, u)) = make_uint4(pk[4 * u], pk[4 * u + 1], pk[4 * u + 2], pk[4 * u + 3]);
        __syncwarp();
        stage_flush(stage, plane, row0, ld);
        __syncwarp();
        // mirror: element j of this lane's row goes to row j, column lane
#pragma unroll
        for (int j = 0; j < 32; ++j)
            *reinterpret_cast<uint16_t*>(stage + stage_off(j, lane >> 3) + ((lane & 7) << 1)) =
                static_cast<uint16_t>(pk[j >> 1] >> ((j & 1) * 16));
        __syncwarp();
        stage_flush(stage, plane, mir0, ld);
        __syncwarp();
    }
}

// A run on the diagonal (q0 == p0 + its row offset 0) through the staging
// buffer: every lane stages its whole row, the upper triangle (q > p) is
// replaced by the mirror of the lower one in shared memory, and the whole
// symmetric run goes out as row segments (it is its own mirror).  FP16 and
// BF16 formats.
template <int FMT>
__device__ __forceinline__ void store_run_diag_staged(const SplitMat& m, int64_t ld, int64_t rb, int64_t cb,
                                                      int64_t p0, const float (&v)[32], uint8_t* stage) {
    constexpr int NT = FMT == FMT_BF16 ? 3 : 2;
    const int lane = threadIdx.x & 31;
    const size_t row0 = static_cast<size_t>(rb + p0) * ld + cb + p0;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        uint32_t pk[16];
        split_plane<FMT>(v, t, pk);
#pragma unroll
        for (int u = 0; u < 4; ++u)
            *reinterpret_cast<uint4*>(stage + stage_off(lane, u)) = make_uint4(pk[4 * u], pk[4 * u + 1], pk[4 * u + 2], pk[4 * u + 3]);
        __syncwarp();
        // (lane, j) for j > lane takes (j, lane): a lower element of row j,
        // which no lane writes here.
#pragma unroll 4
        for (int j = 1; j < 32; ++j) {
            if (j > lane) {
                const uint16_t h =
                    *reinterpret_cast<const uint16_t*>(stage + stage_off(j, lane >> 3) + ((lane & 7) << 1));
                *reinterpret_cast<uint16_t*>(stage + stage_off(lane, j >> 3) + ((j & 7) << 1)) = h;
            }
        }
        __syncwarp();
        stage_flush(stage, static_cast<uint16_t*>(m.term[t]), row0, ld);
        __syncwarp();
    }
}

// A run on the diagonal (q0 == p0): element-wise with the p >= q mask.
template <int FMT>
__device__ __forceinline__ void store_run_diag(const SplitMat& m, int64_t ld, int64_t rb, int64_t cb, int64_t p,
                                               int64_t q0, const float (&v)[32]) {
    const size_t row_idx = static_cast<size_t>(rb + p) * ld + cb + q0;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const int64_t q = q0 + j;
        if (p >= q) {
            split_store(m, FMT, row_idx + j, v[j]);
            if (p != q) split_store(m, FMT, static_cast<size_t>(rb + q) * ld + cb + p, v[j]);
        }
    }
}

// Eight consecutive values of a split matrix at element idx (one 16-byte
// vector per term plane), the terms summed from the smallest to the largest
// (FP16 terms: the sum times 2^-12).
template <int FMT>
__device__ __forceinline__ void load_run8(const SplitMat& m, size_t idx, float (&out)[8]) {
    constexpr int NT = FMT == FMT_BF16 ? 3 : 2;  // the F16Q8 format's value is its F16 pair
#pragma unroll
    for (int j = 0; j < 8; ++j) out[j] = 0.f;
#pragma unroll
    for (int t = NT - 1; t >= 0; --t) {
        const uint4 w = *reinterpret_cast<const uint4*>(static_cast<const uint16_t*>(m.term[t]) + idx);
        const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const uint16_t lo = static_cast<uint16_t>(ws[h] & 0xFFFFu), hi = static_cast<uint16_t>(ws[h] >> 16);
            if (FMT != FMT_BF16) {
                out[2 * h] += __half2float(__ushort_as_half(lo));
                out[2 * h + 1] += __half2float(__ushort_as_half(hi));
            } else {
                out[2 * h] += __bfloat162float(__ushort_as_bfloat16(lo));
                out[2 * h + 1] += __bfloat162float(__ushort_as_bfloat16(hi));
            }
        }
    }
    if (FMT != FMT_BF16) {
#pragma unroll
        for (int j = 0; j < 8; ++j) out[j] *= kF16Unscale;
    }
}

// The epilogue of one 32 x 32 run of accumulator values v (lane = row
// p0 + lane, columns q0 .. q0 + 31, q0 <= p0 + 31): the final reconstruction
// in FP64, or the polynomial step / plain store with the operand split, at
// (p, q) and at the mirror (q, p).  FMT is the format the results are stored
// in; E4M3_OPS says the product read the E4M3 plane (F16Q8 storage) rather
// than the 16-bit terms.
//
// stage: the warp's RUN_STAGE_BYTES of shared memory for the staged stores,
// or null for direct stores (the F16Q8 format always stores directly);
// STAGED_LOADS: the FP16 step epilogue also fetches A and A3 through it (two
// 32-value arrays more per thread: for callers with registers to spare);
// STAGED_FINAL: the final reconstruction goes through it too (its own kernel
// instantiation: the staged final's registers would otherwise crowd the
// product epilogues').
template <int FMT, bool E4M3_OPS = false, bool STAGED_LOADS = true, bool STAGED_FINAL = false>
__device__ __forceinline__ void epilogue_run(const EpiParams& ep, const TileInfo& ti, int64_t p0, int64_t q0,
                                             float (&v)[32], uint8_t* stage = nullptr) {
    const int64_t ld = ep.ld;
    const int64_t rb = ti.blk.row_base;
    const int64_t cb = ti.blk.col_base;
    const int64_t p = p0 + (threadIdx.x & 31);
    // FP16 operand terms carry a factor 2^12 each (kF16Scale), E4M3 ones 2^7.
    const float acc_scale = E4M3_OPS ? ep.acc_scale * kE4M3AccUnscale
                            : FMT != FMT_BF16 ? ep.acc_scale * kF16AccUnscale
                                              : ep.acc_scale;
    if (STAGED_FINAL && ep.kind == EPI_FINAL && stage != nullptr) {
        final_run_staged(ep, ti, p0, q0, v, acc_scale, stage);
        return;
    }
    if (ep.kind == EPI_FINAL) {
        const int64_t n = ti.blk.n;
        if (p >= n) return;
        const double up = ti.blk.up_dev ? ep.up * *ti.blk.up_dev : ep.up;
        double* out = ep.out64 + ti.blk.x_off;
        const double* x = ep.x64 + ti.blk.x_off;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const int64_t q = q0 + j;
            if (q <= p && q < n) {
                const double o = 0.5 * (x[p * n + q] + up * static_cast<double>(acc_scale * v[j]));
                out[p * n + q] = o;
                if (q != p) out[q * n + p] = o;
            }
        }
        return;
    }
    if (ep.kind == EPI_FINAL32) {  // FP32 input and output (single matrices only)
        const int64_t n = ti.blk.n;
        if (p >= n) return;
        const double up = ti.blk.up_dev ? ep.up * *ti.blk.up_dev : ep.up;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const int64_t q = q0 + j;
            if (q <= p && q < n) {
                const float o = static_cast<float>(
                    0.5 * (static_cast<double>(ep.x32[p * n + q]) + up * static_cast<double>(acc_scale * v[j])));
                ep.out32[p * n + q] = o;
                if (q != p) ep.out32[q * n + p] = o;
            }
        }
        return;
    }
    if (ep.skip_pad && (p0 >= ti.blk.n || q0 >= ti.blk.n)) return;  // padding run (warp-uniform)
    const size_t idx = static_cast<size_t>(rb + p) * ld + cb + q0;
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] *= acc_scale;
    if (STAGED_LOADS && ep.kind == EPI_STEP && FMT == FMT_F16 && stage != nullptr) {
        // A and A3 fetched coalesced through the staging buffer (same values
        // and arithmetic as load_run8)
        const size_t row0 = static_cast<size_t>(rb + p0) * ld + cb + q0;
        float w[32];
        stage_values_f16(ep.A, row0, ld, stage, w);
#pragma unroll
        for (int j = 0; j < 32; ++j) w[j] *= ep.a;
        float a3[32];
        stage_values_f16(ep.A3, row0, ld, stage, a3);
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = fmaf(ep.c, v[j], fmaf(ep.b, a3[j], w[j]));
    } else if (ep.kind == EPI_STEP) {
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            float a[8], a3[8];
            load_run8<FMT>(ep.A, idx + 8 * g, a);
            load_run8<FMT>(ep.A3, idx + 8 * g, a3);
#pragma unroll
            for (int j = 0; j < 8; ++j) v[8 * g + j] = fmaf(ep.c, v[8 * g + j], fmaf(ep.b, a3[j], ep.a * a[j]));
        }
    }
    if (FMT != FMT_F16Q8 && stage != nullptr) {
        if (q0 + 31 < p0)
            store_run_full_staged<FMT>(ep.out, ld, rb, cb, p0, q0, v, stage);
        else
            store_run_diag_staged<FMT>(ep.out, ld, rb, cb, p0, v, stage);
        return;
    }
    if (q0 + 31 < p0)
        store_run_full<FMT>(ep.out, ld, rb, cb, p0, q0, v);
    else
        store_run_diag<FMT>(ep.out, ld, rb, cb, p, q0, v);
}

// Epilogue of one tile for the warp whose first local row is p0 (lane = row
// p0 + lane), reading the accumulators from TMEM, columns [c_begin, c_end)
// of the tile.  TN is the tile width (the MMA's N): ti.bj counts column tiles
// of TN, and the ACC_SPLIT accumulators of a tile sit TN TMEM columns apart.
template <int FMT, int ACC_SPLIT, int TN = BN, bool E4M3_OPS = false, bool STAGED_FINAL = false>
__device__ void epilogue_tile(const EpiParams& ep, const TileInfo& ti, uint32_t tmem_row, int64_t p0, int nacc,
                              int c_begin = 0, int c_end = TN, uint8_t* stage = nullptr) {
    for (int c0 = c_begin; c0 < c_end; c0 += 32) {
        float v[32];
        tmem_ld_32cols(tmem_row + static_cast<uint32_t>(c0), v);
#pragma unroll
        for (int a = 1; a < ACC_SPLIT; ++a) {
            if (a < nacc) {
                float w[32];
                tmem_ld_32cols(tmem_row + static_cast<uint32_t>(a * TN + c0), w);
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] += w[j];
            }
        }
        const int64_t q0 = ti.bj * TN + c0;
        if (q0 > p0 + 31) continue;  // whole run above the diagonal: owned by the mirror tile
        epilogue_run<FMT, E4M3_OPS, true, STAGED_FINAL>(ep, ti, p0, q0, v, stage);
    }
}

}  // namespace
}  // namespace psdgb
