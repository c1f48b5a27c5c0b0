// gemm_simt.cu — plain FP32 symmetric product on the CUDA cores.
//
// This is the PSDGB_PREC_FP32_SIMT mode: the same arithmetic as the
// reference's cublasSgemm calls (FP32 operands, FP32 FMA accumulation,
// src/composite_FP32.cu:103,106,115,150), restricted to the lower tiles of
// the row-major view (the upper triangle of the column-major matrix) with the
// mirrored-store epilogue.  It is the numerics baseline the tensor-core
// modes are compared against, not the fast path.
#include "epilogue.cuh"
#include "internal.h"

namespace psdgb {

namespace {

constexpr int BM = 128, BK = 8, THREADS = 256;

__device__ __forceinline__ void tri_decode(int64_t t, int64_t& bi, int64_t& bj) {
    int64_t i = static_cast<int64_t>((sqrt(8.0 * static_cast<double>(t) + 1.0) - 1.0) * 0.5);
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    while (i * (i + 1) / 2 > t) --i;
    bi = i;
    bj = t - i * (i + 1) / 2;
}

// C(p, q) = sum_k P(p, k) Q(q, k) for the 128x128 tile (bi, bj), bi >= bj.
__global__ void __launch_bounds__(THREADS) simt_sym_kernel(const float* __restrict__ P, const float* __restrict__ Q,
                                                           int64_t np, EpiParams ep) {
    __shared__ float As[BK][BM + 4];
    __shared__ float Bs[BK][BM + 4];
    int64_t bi, bj;
    tri_decode(blockIdx.x, bi, bj);
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    const int lrow = tid / 2, lk = (tid % 2) * 4;
    for (int half = 0; half < (ep.dual ? 2 : 1); ++half) {
    // The second half of a dual product multiplies Q's rows bi by P's rows bj.
    const float* Pp = (half ? Q : P) + (bi * BM + lrow) * np + lk;
    const float* Qp = (half ? P : Q) + (bj * BM + lrow) * np + lk;
    for (int64_t k0 = 0; k0 < np; k0 += BK) {
        const float4 a = *reinterpret_cast<const float4*>(Pp + k0);
        const float4 b = *reinterpret_cast<const float4*>(Qp + k0);
        __syncthreads();
        As[lk + 0][lrow] = a.x; As[lk + 1][lrow] = a.y; As[lk + 2][lrow] = a.z; As[lk + 3][lrow] = a.w;
        Bs[lk + 0][lrow] = b.x; Bs[lk + 1][lrow] = b.y; Bs[lk + 2][lrow] = b.z; Bs[lk + 3][lrow] = b.w;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            float av[8], bv[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) av[i] = As[k][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 8; ++j) bv[j] = Bs[k][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
    }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int64_t p = bi * BM + ty + 16 * i;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t q = bj * BM + tx + 16 * j;
            if (p >= q) epi_element(ep, p, q, acc[i][j]);
        }
    }
}

}  // namespace

psdgb_status gemm_simt(DeviceState* ds, const SplitMat& P, const SplitMat& Q, int64_t np, const EpiParams& ep,
                       cudaStream_t s) {
    (void)ds;
    const int64_t nt = np / BM;
    const int64_t tiles = nt * (nt + 1) / 2;
    simt_sym_kernel<<<static_cast<unsigned>(tiles), THREADS, 0, s>>>(static_cast<const float*>(P.term[0]),
                                                                      static_cast<const float*>(Q.term[0]), np, ep);
    count_launch();
    PSDGB_CUDA_TRY(cudaGetLastError());
    return PSDGB_OK;
}

}  // namespace psdgb
