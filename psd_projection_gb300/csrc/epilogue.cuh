// epilogue.cuh — per-element epilogue of the symmetric filter products.
//
// The reference applies the step polynomial with separate cuBLAS passes
// (Sscal, Saxpy and a beta=1 Sgemm, src/composite_FP32.cu:108-115), then
// symmetrises with two Sgeam and an Sscal (src/utils.cu:7-32), and ends with
// add_identity, Sscal, a conversion and another symmetrisation
// (src/composite_FP32.cu:143-156).  Here the product kernels compute one
// triangle and this epilogue writes each value twice (at (p, q) and at the
// mirror (q, p)), so every operand is exactly symmetric and no separate pass
// touches HBM.
#pragma once

#include "common.cuh"

namespace psdgb {

// Value the epilogue produces for product element (p, q) with accumulator acc
// (EPI_STORE / EPI_STEP).
__device__ __forceinline__ float epi_value(const EpiParams& ep, size_t idx, float acc) {
    acc *= ep.acc_scale;
    if (ep.kind == EPI_STEP) {
        const float a = split_load(ep.A, ep.fmt, idx);
        const float a3 = split_load(ep.A3, ep.fmt, idx);
        return fmaf(ep.c, acc, fmaf(ep.b, a3, ep.a * a));
    }
    return acc;
}

// Full per-element epilogue for element (p, q), p >= q, of an np x np product.
__device__ __forceinline__ void epi_element(const EpiParams& ep, int64_t p, int64_t q, float acc) {
    if (ep.kind == EPI_FINAL) {
        if (p < ep.n) {
            const int64_t n = ep.n;
            const double up = ep.up_dev ? ep.up * *ep.up_dev : ep.up;
            const double v = 0.5 * (ep.x64[p * n + q] + up * static_cast<double>(ep.acc_scale * acc));
            ep.out64[p * n + q] = v;
            if (p != q) ep.out64[q * n + p] = v;
        }
        return;
    }
    if (ep.kind == EPI_FINAL32) {
        if (p < ep.n) {
            const int64_t n = ep.n;
            const double up = ep.up_dev ? ep.up * *ep.up_dev : ep.up;
            const float v = static_cast<float>(
                0.5 * (static_cast<double>(ep.x32[p * n + q]) + up * static_cast<double>(ep.acc_scale * acc)));
            ep.out32[p * n + q] = v;
            if (p != q) ep.out32[q * n + p] = v;
        }
        return;
    }
    const size_t i0 = static_cast<size_t>(p) * ep.np + q;
    const float v = epi_value(ep, i0, acc);
    split_store(ep.out, ep.fmt, i0, v);
    if (p != q) split_store(ep.out, ep.fmt, static_cast<size_t>(q) * ep.np + p, v);
}

}  // namespace psdgb
