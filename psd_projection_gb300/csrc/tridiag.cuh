// tridiag.cuh — the largest eigenpair of a small symmetric tridiagonal matrix,
// on the device.
//
// The reference forms the Lanczos tridiagonal T densely and takes the last
// eigenpair of cuSOLVER Dsyevd (src/lanczos.cu:186-240).  Here one warp:
// theta by 33-way multisection on the Sturm count (each lane evaluates one
// split point, a ballot picks the sub-interval; about 11 rounds to full FP64
// precision), then the eigenvector by four steps of inverse iteration in lane 0.
// Divisions are reciprocal multiplies (__drcp_rn): FP64 division is a long
// dependent sequence on this part and these loops are latency-bound.
#pragma once

#include "common.cuh"

namespace psdgb {

// Number of eigenvalues of T strictly less than x (Sturm count of the LDL^T
// pivots of T - x I).
__device__ inline int64_t sturm_count(const double* d, const double* e, int64_t m, double x, double pivmin) {
    int64_t cnt = 0;
    double q = d[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
    for (int64_t i = 1; i < m; ++i) {
        q = d[i] - x - (e[i - 1] * e[i - 1]) * __drcp_rn(q);
        if (fabs(q) < pivmin) q = -pivmin;
        if (q < 0) ++cnt;
    }
    return cnt;
}

// Solve (T - shift I) x = b in place by Gaussian elimination with partial
// pivoting on the band (fill-in on a second superdiagonal); work holds 4m doubles.
__device__ inline void tridiag_solve(const double* d, const double* e, int64_t m, double shift, double tiny, double* b,
                              double* work) {
    double* dl = work;
    double* dd = work + m;
    double* du = work + 2 * m;
    double* du2 = work + 3 * m;
    for (int64_t i = 0; i < m; ++i) {
        dd[i] = d[i] - shift;
        dl[i] = (i + 1 < m) ? e[i] : 0.0;
        du[i] = (i + 1 < m) ? e[i] : 0.0;
        du2[i] = 0.0;
    }
    for (int64_t i = 0; i + 1 < m; ++i) {
        if (fabs(dd[i]) >= fabs(dl[i])) {
            if (dd[i] == 0.0) dd[i] = tiny;
            const double f = dl[i] * __drcp_rn(dd[i]);
            dd[i + 1] -= f * du[i];
            b[i + 1] -= f * b[i];
            dl[i] = 0.0;
        } else {  // swap rows i and i+1
            const double f = dd[i] * __drcp_rn(dl[i]);
            dd[i] = dl[i];
            const double t = dd[i + 1];
            dd[i + 1] = du[i] - f * t;
            du[i] = t;
            if (i + 2 < m) {
                du2[i] = du[i + 1];
                du[i + 1] = -f * du2[i];
            }
            const double tb = b[i];
            b[i] = b[i + 1];
            b[i + 1] = tb - f * b[i];
        }
    }
    if (dd[m - 1] == 0.0) dd[m - 1] = tiny;
    b[m - 1] *= __drcp_rn(dd[m - 1]);
    if (m > 1) b[m - 2] = (b[m - 2] - du[m - 2] * b[m - 1]) * __drcp_rn(dd[m - 2]);
    for (int64_t i = m - 3; i >= 0; --i) b[i] = (b[i] - du[i] * b[i + 1] - du2[i] * b[i + 2]) * __drcp_rn(dd[i]);
}

// Whole warp: largest eigenvalue theta of T (diag d[0..m), off-diagonal
// e[0..m-1)), m >= 2, and a unit eigenvector in u (lane 0 writes u and
// returns theta; work holds 4m doubles).  Every lane returns theta.
__device__ inline double warp_tridiag_top(const double* d, const double* e, int64_t m, double* u, double* work) {
    const int lane = threadIdx.x & 31;
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
    for (int it = 0; it < 64; ++it) {
        if (hi - lo <= 2.0 * eps * fmax(fabs(lo), fabs(hi))) break;
        const double x = lo + (hi - lo) * (static_cast<double>(lane + 1) / 33.0);
        const bool above = (x > lo && x < hi) ? (sturm_count(d, e, m, x, pivmin) >= m) : (x >= hi);
        const unsigned mask = __ballot_sync(0xffffffffu, above);
        const int first = mask ? __ffs(mask) - 1 : 32;  // first split point with all eigenvalues below it
        const double new_hi = (first < 32) ? __shfl_sync(0xffffffffu, x, first) : hi;
        const double new_lo = (first > 0) ? __shfl_sync(0xffffffffu, x, first > 0 ? first - 1 : 0) : lo;
        if (!(new_hi < hi || new_lo > lo)) break;  // no progress at this precision
        hi = new_hi;
        lo = new_lo;
    }
    const double t = 0.5 * (lo + hi);
    if (lane == 0) {
        const double tiny = eps * fmax(tnorm, 2.2250738585072014e-308);
        const double shift = t + 4.0 * eps * fmax(tnorm, fabs(t));
        for (int64_t i = 0; i < m; ++i) u[i] = 1.0;
        for (int it = 0; it < 4; ++it) {
            tridiag_solve(d, e, m, shift, tiny, u, work);
            double s = 0.0;
            for (int64_t i = 0; i < m; ++i) s += u[i] * u[i];
            s = sqrt(s);
            if (!(s > 0.0) || !isfinite(s)) {
                for (int64_t i = 0; i < m; ++i) u[i] = 1.0 / sqrt(static_cast<double>(m));
                break;
            }
            for (int64_t i = 0; i < m; ++i) u[i] /= s;
        }
    }
    return t;
}

}  // namespace psdgb
