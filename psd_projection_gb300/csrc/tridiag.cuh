// tridiag.cuh — the largest eigenpair of a small symmetric tridiagonal matrix,
// on the device.
//
// The reference forms the Lanczos tridiagonal T densely and takes the last
// eigenpair of cuSOLVER Dsyevd (src/lanczos.cu:186-240).  Here one warp:
// theta by multisection on the Sturm count over up to four warps (129 split
// points a round, about 8 rounds to full FP64 precision), then the
// eigenvector by inverse iteration in thread 0 (one factorisation, two
// solves).  Divisions are reciprocal multiplies (__drcp_rn), and T is first
// staged in the caller's scratch (shared memory) with e^2 precomputed.
#pragma once

#include "common.cuh"

namespace psdgb {

// Number of eigenvalues of T strictly less than x (signs of the LDL^T
// pivots of T - x I); e2[i] = e[i]^2.
__device__ inline int sturm_count(const double* d, const double* e2, int64_t m, double x, double pivmin) {
    int cnt = 0;
    double q = d[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
    for (int64_t i = 1; i < m; ++i) {
        q = d[i] - x - e2[i - 1] * __drcp_rn(q);
        if (fabs(q) < pivmin) q = -pivmin;
        if (q < 0) ++cnt;
    }
    return cnt;
}

// LU factorisation with partial pivoting of the band of T - shift I (fill-in
// on a second superdiagonal).  work holds 5m doubles: reciprocal pivots,
// first and second superdiagonals, multipliers, row-swap flags.
__device__ inline void tridiag_factor(const double* d, const double* e, int64_t m, double shift, double tiny,
                                      double* work) {
    double* rdd = work;
    double* du = work + m;
    double* du2 = work + 2 * m;
    double* f = work + 3 * m;
    double* sw = work + 4 * m;
    double dcur = d[0] - shift;                  // current pivot candidate (row i)
    double dnext = m > 1 ? d[1] - shift : 0.0;   // diagonal of row i+1
    double ucur = m > 1 ? e[0] : 0.0;            // superdiagonal of row i
    for (int64_t i = 0; i + 1 < m; ++i) {
        const double li = e[i];                  // subdiagonal below the pivot
        const double unext = (i + 2 < m) ? e[i + 1] : 0.0;
        if (fabs(dcur) >= fabs(li)) {
            if (dcur == 0.0) dcur = tiny;
            const double fi = li * __drcp_rn(dcur);
            rdd[i] = __drcp_rn(dcur);
            du[i] = ucur;
            du2[i] = 0.0;
            f[i] = fi;
            sw[i] = 0.0;
            dnext -= fi * ucur;
            ucur = unext;
        } else {  // swap rows i and i+1
            const double fi = dcur * __drcp_rn(li);
            rdd[i] = __drcp_rn(li);
            du[i] = dnext;
            du2[i] = unext;
            f[i] = fi;
            sw[i] = 1.0;
            dnext = ucur - fi * dnext;
            ucur = -fi * unext;
        }
        dcur = dnext;
        dnext = (i + 2 < m) ? d[i + 2] - shift : 0.0;
    }
    if (dcur == 0.0) dcur = tiny;
    rdd[m - 1] = __drcp_rn(dcur);
    du[m - 1] = 0.0;
    du2[m - 1] = 0.0;
}

// Solve (T - shift I) x = b in place with the factors of tridiag_factor.
__device__ inline void tridiag_apply(int64_t m, const double* work, double* b) {
    const double* rdd = work;
    const double* du = work + m;
    const double* du2 = work + 2 * m;
    const double* f = work + 3 * m;
    const double* sw = work + 4 * m;
    for (int64_t i = 0; i + 1 < m; ++i) {
        if (sw[i] != 0.0) {
            const double tb = b[i];
            b[i] = b[i + 1];
            b[i + 1] = tb - f[i] * b[i];
        } else {
            b[i + 1] -= f[i] * b[i];
        }
    }
    b[m - 1] *= rdd[m - 1];
    if (m > 1) b[m - 2] = (b[m - 2] - du[m - 2] * b[m - 1]) * rdd[m - 2];
    for (int64_t i = m - 3; i >= 0; --i) b[i] = (b[i] - du[i] * b[i + 1] - du2[i] * b[i + 2]) * rdd[i];
}

// Whole block (every thread calls it; it synchronises the block): the
// largest eigenvalue theta of T (diag d[0..m), off-diagonal e[0..m-1)),
// m >= 2, returned to every thread, and a unit eigenvector in u (written by
// thread 0; synchronise before reading it).  scratch holds 3m doubles (T is
// staged there with e^2; shared memory where the caller has it), work 5m.
//
// An FP64 warp instruction occupies its scheduler for many cycles on this
// GPU whatever the number of active lanes, so the cost is the count of
// dependent FP64 warp instructions: each round, W = min(4, warps) warps (one
// per scheduler) evaluate one Sturm chain per lane, splitting [lo, hi) at
// 32 W points, and the first split point with every eigenvalue below it is
// found from the warps' ballots.  Every thread computes the split points
// with the same formula, so lo and hi are the same numbers everywhere.
__device__ inline double block_tridiag_top(const double* d_in, const double* e_in, int64_t m, double* u,
                                           double* work, double* scratch) {
    __shared__ unsigned masks[2][4];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int W = min(4, static_cast<int>(blockDim.x >> 5));
    const int P = 32 * W;
    double* d = scratch;
    double* e = scratch + m;
    double* e2 = scratch + 2 * m;
    for (int64_t i = tid; i < m; i += blockDim.x) {
        d[i] = d_in[i];
        const double ei = (i + 1 < m) ? e_in[i] : 0.0;
        e[i] = ei;
        e2[i] = ei * ei;
    }
    __syncthreads();
    double lo = INFINITY, hi = -INFINITY, tnorm = 0.0;
    for (int64_t i = 0; i < m; ++i) {
        const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < m ? fabs(e[i]) : 0.0);
        lo = fmin(lo, d[i] - r);
        hi = fmax(hi, d[i] + r);
        tnorm = fmax(tnorm, fabs(d[i]) + r);
    }
    const double eps = 2.220446049250313e-16;
    const double pivmin = fmax(2.2250738585072014e-308, eps * eps * tnorm * tnorm);
    const double pad = 2.0 * eps * tnorm + pivmin;
    lo -= pad;
    hi += pad;
    // Invariant: count(lo) < m <= count(hi); the largest eigenvalue lies in [lo, hi).
    const double step = 1.0 / static_cast<double>(P + 1);
    for (int it = 0; it < 64; ++it) {
        if (hi - lo <= 2.0 * eps * fmax(fabs(lo), fabs(hi))) break;
        const double w = hi - lo;
        bool above = false;
        if (warp < W) {
            const double x = lo + w * (static_cast<double>(warp * 32 + lane + 1) * step);
            above = (x > lo && x < hi) ? (sturm_count(d, e2, m, x, pivmin) >= m) : (x >= hi);
        }
        const unsigned ballot = __ballot_sync(0xffffffffu, above);
        if (warp < W && lane == 0) masks[it & 1][warp] = ballot;
        __syncthreads();
        int g = P;  // first split point with every eigenvalue below it, P if none
        for (int ww = 0; ww < W; ++ww) {
            const unsigned b = masks[it & 1][ww];
            if (b) {
                g = 32 * ww + __ffs(b) - 1;
                break;
            }
        }
        const double new_hi = (g < P) ? lo + w * (static_cast<double>(g + 1) * step) : hi;
        const double new_lo = (g > 0) ? lo + w * (static_cast<double>(g) * step) : lo;
        if (!(new_hi < hi || new_lo > lo)) break;  // no progress at this precision
        hi = new_hi;
        lo = new_lo;
    }
    const double t = 0.5 * (lo + hi);
    if (tid == 0) {
        // Inverse iteration from a shift within a few ulps of theta: one
        // factorisation of T - shift I, two solves.
        const double tiny = eps * fmax(tnorm, 2.2250738585072014e-308);
        const double shift = t + 4.0 * eps * fmax(tnorm, fabs(t));
        tridiag_factor(d, e, m, shift, tiny, work);
        for (int64_t i = 0; i < m; ++i) u[i] = 1.0;
        for (int iter = 0; iter < 2; ++iter) {
            tridiag_apply(m, work, u);
            double s = 0.0;
            for (int64_t i = 0; i < m; ++i) s += u[i] * u[i];
            s = sqrt(s);
            if (!(s > 0.0) || !isfinite(s)) {
                const double v = 1.0 / sqrt(static_cast<double>(m));
                for (int64_t i = 0; i < m; ++i) u[i] = v;
                break;
            }
            const double rs = 1.0 / s;
            for (int64_t i = 0; i < m; ++i) u[i] *= rs;
        }
    }
    return t;
}

}  // namespace psdgb
