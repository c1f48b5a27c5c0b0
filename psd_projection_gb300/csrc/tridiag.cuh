// tridiag.cuh — the largest eigenpair of a small symmetric tridiagonal matrix,
// on the device.
//
// The reference forms the Lanczos tridiagonal T densely and takes the last
// eigenpair of cuSOLVER Dsyevd (src/lanczos.cu:186-240).  Here one warp:
// theta by 129-way multisection on the Sturm count (each lane evaluates four
// split points as interleaved recurrences, a ballot picks the sub-interval;
// about 8 rounds to full FP64 precision), then the eigenvector by inverse
// iteration in lane 0 (one factorisation, four solves).  Divisions are
// reciprocal multiplies (__drcp_rn): FP64 arithmetic issues slowly on this
// part and these loops are latency-bound, so T is first staged in the
// caller's scratch (shared memory) with e^2 precomputed.
#pragma once

#include "common.cuh"

namespace psdgb {

// Sturm counts of four shifts at once: cnt[j] = number of eigenvalues of T
// strictly less than x[j] (signs of the LDL^T pivots of T - x[j] I).  The four
// recurrences are independent and interleaved, which hides the latency of the
// FP64 reciprocals; e2[i] = e[i]^2.
__device__ inline void sturm_count4(const double* d, const double* e2, int64_t m, const double (&x)[4],
                                    double pivmin, int (&cnt)[4]) {
    double q[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        q[j] = d[0] - x[j];
        if (fabs(q[j]) < pivmin) q[j] = -pivmin;
        cnt[j] = q[j] < 0 ? 1 : 0;
    }
    for (int64_t i = 1; i < m; ++i) {
        const double di = d[i], ei = e2[i - 1];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            q[j] = di - x[j] - ei * __drcp_rn(q[j]);
            if (fabs(q[j]) < pivmin) q[j] = -pivmin;
            cnt[j] += q[j] < 0 ? 1 : 0;
        }
    }
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

// Whole warp: largest eigenvalue theta of T (diag d[0..m), off-diagonal
// e[0..m-1)), m >= 2, and a unit eigenvector in u (lane 0 writes u; every
// lane returns theta).  scratch holds 3m doubles (d, e, e^2 are staged there;
// shared memory where the caller has it), work 5m.
__device__ inline double warp_tridiag_top(const double* d_in, const double* e_in, int64_t m, double* u, double* work,
                                          double* scratch) {
    const int lane = threadIdx.x & 31;
    double* d = scratch;
    double* e = scratch + m;
    double* e2 = scratch + 2 * m;
    for (int64_t i = lane; i < m; i += 32) {
        d[i] = d_in[i];
        const double ei = (i + 1 < m) ? e_in[i] : 0.0;
        e[i] = ei;
        e2[i] = ei * ei;
    }
    __syncwarp();
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
    // Invariant: count(lo) < m <= count(hi); the largest eigenvalue lies in
    // [lo, hi).  Each round splits [lo, hi) at 128 points (four per lane);
    // every lane computes the split points with the same formula, so the new
    // ends are the same numbers in every lane.
    constexpr double kStep = 1.0 / 129.0;
    for (int it = 0; it < 64; ++it) {
        if (hi - lo <= 2.0 * eps * fmax(fabs(lo), fabs(hi))) break;
        const double w = hi - lo;
        double x[4];
        int cnt[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) x[j] = lo + w * (static_cast<double>(4 * lane + j + 1) * kStep);
        sturm_count4(d, e2, m, x, pivmin, cnt);
        int first_local = 4;
#pragma unroll
        for (int j = 3; j >= 0; --j) {
            const bool above = (x[j] > lo && x[j] < hi) ? (cnt[j] >= m) : (x[j] >= hi);
            if (above) first_local = j;
        }
        const unsigned mask = __ballot_sync(0xffffffffu, first_local < 4);
        int g;  // first split point (0..127) with every eigenvalue below it, 128 if none
        if (mask) {
            const int L = __ffs(mask) - 1;
            g = 4 * L + __shfl_sync(0xffffffffu, first_local, L);
        } else {
            g = 128;
        }
        const double new_hi = (g < 128) ? lo + w * (static_cast<double>(g + 1) * kStep) : hi;
        const double new_lo = (g > 0) ? lo + w * (static_cast<double>(g) * kStep) : lo;
        if (!(new_hi < hi || new_lo > lo)) break;  // no progress at this precision
        hi = new_hi;
        lo = new_lo;
    }
    const double t = 0.5 * (lo + hi);
    if (lane == 0) {
        // Inverse iteration: one factorisation of T - shift I, four solves.
        const double tiny = eps * fmax(tnorm, 2.2250738585072014e-308);
        const double shift = t + 4.0 * eps * fmax(tnorm, fabs(t));
        tridiag_factor(d, e, m, shift, tiny, work);
        for (int64_t i = 0; i < m; ++i) u[i] = 1.0;
        for (int it = 0; it < 4; ++it) {
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
