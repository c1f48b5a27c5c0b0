// common.cuh — shared device helpers for the psdgb kernels (sm_103a only).
//
// Holds the operand-split arithmetic used by every kernel that writes filter
// operands, the inline-PTX wrappers for mbarrier / TMA / tcgen05, and the
// bounded-wait helpers.  Every spin-wait in this library is bounded by a
// wall-clock limit read from %globaltimer; a wait that gives up records an
// error code in the library's device error word and the kernel returns.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>

namespace psdgb {

// ---------------------------------------------------------------------------
// Storage formats of a filter operand ("split matrix").
//   F32  : one FP32 term (plain SIMT mode).
//   F16  : two FP16 terms, x = hi + lo.
//   BF16 : three BF16 terms, x = b0 + b1 + b2 (Henry, Tang & Heinecke,
//          "Leveraging the bfloat16 AI datatype for higher-precision
//          computations", ARITH 2019).
//   F16Q8: the F16 pair (term planes 0 and 1, the stored value) plus an FP8
//          E4M3 plane (term 2, one byte per element) that the FP8 products
//          read; every store writes all three.
// ---------------------------------------------------------------------------
enum Format : int { FMT_F32 = 0, FMT_F16 = 1, FMT_BF16 = 2, FMT_F16Q8 = 3 };

struct SplitMat {
    void* term[3];   // device pointers, each Np x Np row-major (ld = Np), zero padded
};

// FP16 terms hold the value times 2^12.  Unscaled, the low term of an entry
// below 0.125 in magnitude falls into FP16's subnormal range (below 2^-14),
// where its absolute spacing 2^-24 caps the hi + lo pair at about 17 bits for
// the entries of a scaled n = 8192 iterate (about 0.01).  With the factor the
// low term stays normal for |v| >= 2^-15 and hi + lo carries 22 bits
// (relative error <= 2^-22) for 3e-5 <= |v| < 16 (65504 / 2^12), which
// holds the filter operands (their spectral norm, which bounds every entry,
// is about 1).  The
// factor is a power of two, so scaling and unscaling are exact: a product of
// two FP16-format operands accumulates 2^24 times the true value and its
// epilogue multiplies by 2^-24.
constexpr float kF16Scale = 4096.0f;
constexpr float kF16Unscale = 1.0f / 4096.0f;
constexpr float kF16AccUnscale = 1.0f / 16777216.0f;
// The E4M3 plane holds the value times 2^7: E4M3 is normal from 2^-6 and
// saturates at 448, so entries from 1.2e-4 to 3.5 keep its 4 significant
// bits, which covers the filter operands (|v| <= ~1.01 on the FP16
// schedule).  Conversions saturate (satfinite), never overflow to NaN.  A
// product of two E4M3 operands accumulates 2^14 times the true value.
constexpr float kE4M3Scale = 128.0f;
constexpr float kE4M3AccUnscale = 1.0f / 16384.0f;

__host__ __device__ inline int format_terms(int fmt) { return fmt == FMT_F32 ? 1 : (fmt == FMT_F16 ? 2 : 3); }
// Bytes of one element in term plane t.
__host__ __device__ inline int format_plane_bytes(int fmt, int t) {
    return fmt == FMT_F32 ? 4 : (fmt == FMT_F16Q8 && t == 2 ? 1 : 2);
}
// Bytes of one element summed over the planes.
__host__ __device__ inline int format_bytes(int fmt) {
    int b = 0;
    for (int t = 0; t < format_terms(fmt); ++t) b += format_plane_bytes(fmt, t);
    return b;
}

#if defined(__CUDACC__)
// Read the value a split matrix stores at linear index idx (FP32 sum of terms).
__device__ __forceinline__ float split_load(const SplitMat& m, int fmt, size_t idx) {
    if (fmt == FMT_F32) return static_cast<const float*>(m.term[0])[idx];
    if (fmt == FMT_F16 || fmt == FMT_F16Q8) {
        const __half* h = static_cast<const __half*>(m.term[0]);
        const __half* l = static_cast<const __half*>(m.term[1]);
        return (__half2float(h[idx]) + __half2float(l[idx])) * kF16Unscale;
    }
    const __nv_bfloat16* b0 = static_cast<const __nv_bfloat16*>(m.term[0]);
    const __nv_bfloat16* b1 = static_cast<const __nv_bfloat16*>(m.term[1]);
    const __nv_bfloat16* b2 = static_cast<const __nv_bfloat16*>(m.term[2]);
    return __bfloat162float(b0[idx]) + (__bfloat162float(b1[idx]) + __bfloat162float(b2[idx]));
}

// Split an FP32 value into its terms and store them at linear index idx.
__device__ __forceinline__ void split_store(const SplitMat& m, int fmt, size_t idx, float v) {
    if (fmt == FMT_F32) { static_cast<float*>(m.term[0])[idx] = v; return; }
    if (fmt == FMT_F16 || fmt == FMT_F16Q8) {
        if (fmt == FMT_F16Q8)
            static_cast<__nv_fp8_storage_t*>(m.term[2])[idx] =
                __nv_cvt_float_to_fp8(v * kE4M3Scale, __NV_SATFINITE, __NV_E4M3);
        v *= kF16Scale;
        __half h = __float2half_rn(v);
        __half l = __float2half_rn(v - __half2float(h));
        static_cast<__half*>(m.term[0])[idx] = h;
        static_cast<__half*>(m.term[1])[idx] = l;
        return;
    }
    __nv_bfloat16 b0 = __float2bfloat16_rn(v);
    float r1 = v - __bfloat162float(b0);
    __nv_bfloat16 b1 = __float2bfloat16_rn(r1);
    __nv_bfloat16 b2 = __float2bfloat16_rn(r1 - __bfloat162float(b1));
    static_cast<__nv_bfloat16*>(m.term[0])[idx] = b0;
    static_cast<__nv_bfloat16*>(m.term[1])[idx] = b1;
    static_cast<__nv_bfloat16*>(m.term[2])[idx] = b2;
}

// split_store for 8 consecutive elements (idx a multiple of 8): the same
// arithmetic, one 16-byte store per term plane.
__device__ __forceinline__ void split_store8(const SplitMat& m, int fmt, size_t idx, const float (&v)[8]) {
    if (fmt == FMT_F32) {
        float4* d = reinterpret_cast<float4*>(static_cast<float*>(m.term[0]) + idx);
        d[0] = make_float4(v[0], v[1], v[2], v[3]);
        d[1] = make_float4(v[4], v[5], v[6], v[7]);
        return;
    }
    if (fmt == FMT_F16 || fmt == FMT_F16Q8) {
        if (fmt == FMT_F16Q8) {
            __align__(8) __nv_fp8x2_storage_t q[4];
#pragma unroll
            for (int e = 0; e < 4; ++e)
                q[e] = __nv_cvt_float2_to_fp8x2(make_float2(v[2 * e] * kE4M3Scale, v[2 * e + 1] * kE4M3Scale),
                                                __NV_SATFINITE, __NV_E4M3);
            *reinterpret_cast<uint2*>(static_cast<uint8_t*>(m.term[2]) + idx) = *reinterpret_cast<const uint2*>(q);
        }
        __align__(16) __half h[8];
        __align__(16) __half l[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const float x = v[e] * kF16Scale;
            h[e] = __float2half_rn(x);
            l[e] = __float2half_rn(x - __half2float(h[e]));
        }
        *reinterpret_cast<uint4*>(static_cast<__half*>(m.term[0]) + idx) = *reinterpret_cast<const uint4*>(h);
        *reinterpret_cast<uint4*>(static_cast<__half*>(m.term[1]) + idx) = *reinterpret_cast<const uint4*>(l);
        return;
    }
    __align__(16) __nv_bfloat16 b0[8];
    __align__(16) __nv_bfloat16 b1[8];
    __align__(16) __nv_bfloat16 b2[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        b0[e] = __float2bfloat16_rn(v[e]);
        const float r1 = v[e] - __bfloat162float(b0[e]);
        b1[e] = __float2bfloat16_rn(r1);
        b2[e] = __float2bfloat16_rn(r1 - __bfloat162float(b1[e]));
    }
    *reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(m.term[0]) + idx) = *reinterpret_cast<const uint4*>(b0);
    *reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(m.term[1]) + idx) = *reinterpret_cast<const uint4*>(b1);
    *reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(m.term[2]) + idx) = *reinterpret_cast<const uint4*>(b2);
}

#endif  // __CUDACC__

// ---------------------------------------------------------------------------
// Epilogue of a symmetric product C = P * Q.  Only the elements (p, q) with
// p >= q (row-major view; the upper triangle of the column-major matrix) are
// computed; each is written at (p, q) and mirrored to (q, p).
// ---------------------------------------------------------------------------
enum EpiKind : int {
    EPI_STORE = 0,  // C -> out (split)
    EPI_STEP = 1,   // a*A + b*A3 + c*acc -> out (split); A, A3 read from split matrices
    EPI_FINAL = 2,  // 0.5*(X + up*acc) -> out64 (FP64, n x n, ld n); X read from x64
    EPI_FINAL32 = 3 // the same with X read from x32 and written to out32 (FP32), arithmetic in FP64
};

struct EpiParams {
    int kind;
    int fmt;          // format of the split matrices below
    int np;           // padded dimension (multiple of 128)
    int n;            // true dimension
    float a, b, c;    // EPI_STEP coefficients
    double up;        // EPI_FINAL scale (times *up_dev when up_dev is set)
    const double* up_dev;
    SplitMat out;     // EPI_STORE / EPI_STEP destination (may alias A for EPI_STEP)
    SplitMat A;       // EPI_STEP inputs
    SplitMat A3;
    const double* x64;  // EPI_FINAL input X (n x n)
    double* out64;      // EPI_FINAL output (may alias x64)
    const float* x32;   // EPI_FINAL32 input X (n x n)
    float* out32;       // EPI_FINAL32 output (may alias x32)
    int dual;           // mainloop: accumulate P*Q^T + Q*P^T (K doubled), the symmetric part of the product
    float acc_scale;    // the accumulator is multiplied by this first (0.5 for a dual product)
    int ld;             // row stride of the split-matrix layout (elements); np for a single matrix
    int skip_pad;       // EPI_STORE / EPI_STEP: leave 32 x 32 runs wholly outside the block's n x n
                        // alone (their operand values are zero and stay zero: only set where the
                        // padding of every split matrix is zero, as in the batch layout)
};

// A group of independent blocks sharing one strided operand layout: block b
// occupies layout rows [row_base, row_base + np) and columns [col_base,
// col_base + np) (row stride EpiParams::ld),
// its FP64 n x n matrix starts at element x_off of the packed input, and its
// scale (for the final reconstruction) is *up_dev.
struct BlockDesc {
    int row_base;
    int np;
    int n;
    int col_base;     // first layout column of the block (blocks share row bands)
    long long x_off;
    const double* up_dev;
};

// One 128 x 128 output tile (bi >= bj) of block `block`.
struct TileDesc {
    int block;
    int bi;
    int bj;
    int pad;
};

// The tile list of a grouped product: device tables, or both null for the
// implicit list of every lower tile of the single block EpiParams describes.
struct GroupWork {
    const TileDesc* tiles;
    const BlockDesc* blocks;
    int group_rows;  // implicit list only: tile order in groups of this many tile rows (0: row by row)
    int reverse = 0; // device tables only: nonzero = the list's length, walked from its end
};

// ---------------------------------------------------------------------------
// Error word and bounded waits.
// ---------------------------------------------------------------------------
enum DeviceError : int {
    DEVERR_NONE = 0,
    DEVERR_TMA_WAIT = 1,     // producer gave up waiting for a free stage
    DEVERR_MMA_WAIT = 2,     // MMA warp gave up waiting for loaded operands
    DEVERR_EPI_WAIT = 3,     // epilogue gave up waiting for the accumulator
    DEVERR_DRAIN_WAIT = 4,   // in-flight copies/MMAs did not drain after an abort
    DEVERR_SELFTEST_WAIT = 5, // the self-test's wait on a barrier nothing arrives at gave up (expected)
    DEVERR_SYMV_WAIT = 6      // the Lanczos tile matvec gave up waiting for a tile or a free stage
};

#if defined(__CUDACC__)
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wall-clock limit of a single device-side wait.  Every legitimate wait in
// these kernels lasts microseconds to a few milliseconds.
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- mbarrier -------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Wait for the phase with the given parity to complete; false after limit_ns.
__device__ __forceinline__ bool mbar_wait_limit(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (globaltimer_ns() - t0 > limit_ns) return false;
    }
    return true;
}
// Wait for the phase with the given parity to complete; false after kWaitLimitNs.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    return mbar_wait_limit(bar, parity, kWaitLimitNs);
}
// The same for all 32 lanes of a warp that goes on to warp-collective
// (.sync.aligned) instructions such as tcgen05.ld: each lane polls on its own
// and may leave its loop at another time, so the warp meets again here and
// every lane gets the same outcome (false if any lane ran out of time).
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, uint32_t parity) {
    const bool ok = mbar_wait_bounded(bar, parity);
    return __all_sync(0xffffffffu, ok);
}
// A flag read by every lane of a warp, with one answer for all of them.
__device__ __forceinline__ bool warp_flag(const volatile int* flag) {
    return __any_sync(0xffffffffu, *flag != 0);
}

// ---- TMA ------------------------------------------------------------------
__device__ __forceinline__ void tma_load_2d(void* smem_dst, const void* tmap, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(smem_dst)),
        "l"(tmap), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}
__device__ __forceinline__ void tma_prefetch_desc(const void* tmap) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(tmap) : "memory");
}

// ---- tcgen05 --------------------------------------------------------------
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Allocate ncols TMEM columns (power of two >= 32); one full warp executes it.
__device__ __forceinline__ void tmem_alloc(uint32_t* smem_result, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(smem_result)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, both K-major, kind::f16 (FP16 or BF16 in, FP32 out).
__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The same with E4M3 operands: kind::f8f6f4, K = 32 elements (32 bytes) per MMA.
__device__ __forceinline__ void umma_f8(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on an mbarrier once every tcgen05 op issued so far by this thread completes.
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// Load 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld_32cols(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    __syncwarp();  // .sync.aligned: the whole warp, converged
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
        // The load is asynchronous: its registers hold the values only after
        // the wait, so both sit in one statement (the compiler may otherwise
        // copy or spill the outputs in between).
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- CTA pairs (cluster of two CTAs sharing one tcgen05.mma.cta_group::2) ----
__device__ __forceinline__ uint32_t cluster_ctarank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// Address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t mapa_shared(uint32_t addr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
// Arrive on an mbarrier of any CTA in the cluster (release at cluster scope).
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t cluster_addr) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait on a barrier that other CTAs of the cluster arrive on.
__device__ __forceinline__ bool mbar_wait_cluster_bounded(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait_cluster(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait_cluster(bar, parity)) {
        if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
    }
    return true;
}
// mbar_wait_cluster_bounded for a whole warp (see mbar_wait_warp).
__device__ __forceinline__ bool mbar_wait_cluster_warp(uint64_t* bar, uint32_t parity) {
    const bool ok = mbar_wait_cluster_bounded(bar, parity);
    return __all_sync(0xffffffffu, ok);
}
// TMA load into this CTA's shared memory whose completion is counted on the
// mbarrier at `bar_cluster_addr`, which may be in the peer CTA of the pair.
__device__ __forceinline__ void tma_load_2d_pair(void* smem_dst, const void* tmap, uint32_t bar_cluster_addr, int x,
                                                 int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cta.global.tile.mbarrier::complete_tx::bytes.cta_group::2 [%0], [%1, {%3, "
        "%4}], [%2];" ::"r"(smem_u32(smem_dst)),
        "l"(tmap), "r"(bar_cluster_addr), "r"(x), "r"(y)
        : "memory");
}
// TMEM allocation for a CTA pair: one warp of each CTA executes it.
__device__ __forceinline__ void tmem_alloc_pair(uint32_t* smem_result, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(smem_result)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish_pair() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc_pair(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// D (+)= A * B^T over the pair: A's 256 rows are 128 in each CTA's shared
// memory, B's N rows N/2 in each; D's rows 0-127 land in this CTA's TMEM and
// rows 128-255 in the peer's.  Issued by one thread of the even CTA.
__device__ __forceinline__ void umma_f16_pair(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                              uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// Arrive on the mbarrier at the same offset in every CTA of `cta_mask` once the
// pair MMAs issued so far by this thread complete.
__device__ __forceinline__ void umma_commit_pair_mc(uint64_t* bar, uint16_t cta_mask) {
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
            smem_u32(bar)),
        "h"(cta_mask)
        : "memory");
}
__device__ __forceinline__ void umma_commit_pair(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// Every thread of both CTAs: all prior shared-memory and barrier operations of
// the cluster are visible after it.
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor of a K-major tile written by TMA with
// 128-byte swizzle: rows of 128 bytes, 8-row swizzle atoms 1024 bytes apart.
// Fields (tcgen05 shared memory descriptor): start address >> 4 in bits 0-13,
// leading byte offset >> 4 in bits 16-29 (unused for swizzled K-major),
// stride byte offset >> 4 in bits 32-45, descriptor version 1 in bits 46-47,
// base offset 0 (atoms are 1024-byte aligned), swizzle mode 2 (128B) in bits 61-63.
__device__ __forceinline__ uint64_t sdesc_kmajor_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
    d |= static_cast<uint64_t>(1u) << 16;
    d |= static_cast<uint64_t>(1024u >> 4) << 32;
    d |= static_cast<uint64_t>(1u) << 46;
    d |= static_cast<uint64_t>(2u) << 61;
    return d;
}

// The same for 64-byte rows (K blocks of 32 FP16 / BF16) with the 64-byte
// swizzle: 8-row groups 512 bytes apart, swizzle mode 4.
__device__ __forceinline__ uint64_t sdesc_kmajor_sw64(uint32_t saddr) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
    d |= static_cast<uint64_t>(1u) << 16;
    d |= static_cast<uint64_t>(512u >> 4) << 32;
    d |= static_cast<uint64_t>(1u) << 46;
    d |= static_cast<uint64_t>(4u) << 61;
    return d;
}

#endif  // __CUDACC__

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator
// (bits 4-5 = 1), A/B format in bits 7-9 / 10-12 (0 = FP16, 1 = BF16),
// both operands K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
// (kind::f8f6f4 uses the same fields, format 0 = E4M3 for A and B, so
// idesc_f16(M, N, false) also describes an E4M3 x E4M3 -> FP32 MMA.)
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N, bool bf16) {
    return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) |
           (static_cast<uint32_t>(N >> 3) << 17) | (static_cast<uint32_t>(M >> 4) << 24);
}

}  // namespace psdgb
