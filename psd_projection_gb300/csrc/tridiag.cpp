// tridiag.cpp — largest eigenpair of the small Lanczos tridiagonal matrix.
//
// The reference forms T densely and calls cuSOLVER Dsyevd on it
// (src/lanczos.cu:186-240), then takes the last (largest) eigenvalue and its
// eigenvector.  T has at most max_iter rows (20 by default), so it is solved
// on the host: the largest eigenvalue by Sturm-sequence bisection (the count
// of negative pivots of the LDL^T factorisation of T - x I), the eigenvector
// by inverse iteration with a tridiagonal LU with partial pivoting.
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "internal.h"

namespace psdgb {

namespace {

// Number of eigenvalues of T strictly less than x.
int64_t sturm_count(const double* d, const double* e, int64_t m, double x, double pivmin) {
    int64_t cnt = 0;
    double q = d[0] - x;
    if (std::fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
    for (int64_t i = 1; i < m; ++i) {
        q = d[i] - x - e[i - 1] * e[i - 1] / q;
        if (std::fabs(q) < pivmin) q = -pivmin;
        if (q < 0) ++cnt;
    }
    return cnt;
}

// Solve (T - shift I) x = b in place (b -> x) by Gaussian elimination with
// partial pivoting on the tridiagonal band (fill-in on the second superdiagonal).
void tridiag_solve(const double* d, const double* e, int64_t m, double shift, double tiny, std::vector<double>& b) {
    std::vector<double> dl(m, 0.0), dd(m), du(m, 0.0), du2(m, 0.0);
    for (int64_t i = 0; i < m; ++i) dd[i] = d[i] - shift;
    for (int64_t i = 0; i + 1 < m; ++i) { dl[i] = e[i]; du[i] = e[i]; }
    for (int64_t i = 0; i + 1 < m; ++i) {
        if (std::fabs(dd[i]) >= std::fabs(dl[i])) {
            if (dd[i] == 0.0) dd[i] = tiny;
            const double f = dl[i] / dd[i];
            dd[i + 1] -= f * du[i];
            b[i + 1] -= f * b[i];
            dl[i] = 0.0;
        } else {  // swap rows i and i+1
            const double f = dd[i] / dl[i];
            dd[i] = dl[i];
            double t = dd[i + 1];
            dd[i + 1] = du[i] - f * t;
            du[i] = t;
            if (i + 2 < m) {
                du2[i] = du[i + 1];
                du[i + 1] = -f * du2[i];
            }
            std::swap(b[i], b[i + 1]);
            b[i + 1] -= f * b[i];
        }
    }
    if (dd[m - 1] == 0.0) dd[m - 1] = tiny;
    b[m - 1] /= dd[m - 1];
    if (m > 1) b[m - 2] = (b[m - 2] - du[m - 2] * b[m - 1]) / dd[m - 2];
    for (int64_t i = m - 3; i >= 0; --i) b[i] = (b[i] - du[i] * b[i + 1] - du2[i] * b[i + 2]) / dd[i];
}

}  // namespace

void tridiag_largest_eigenpair(const double* d, const double* e, int64_t m, double* theta, double* vec) {
    if (m == 1) {
        *theta = d[0];
        vec[0] = 1.0;
        return;
    }
    // Gershgorin interval.
    double lo = std::numeric_limits<double>::infinity(), hi = -lo, tnorm = 0.0;
    for (int64_t i = 0; i < m; ++i) {
        const double r = (i > 0 ? std::fabs(e[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(e[i]) : 0.0);
        lo = std::min(lo, d[i] - r);
        hi = std::max(hi, d[i] + r);
        tnorm = std::max(tnorm, std::fabs(d[i]) + r);
    }
    const double eps = std::numeric_limits<double>::epsilon();
    const double pivmin = std::max(std::numeric_limits<double>::min(), eps * eps * tnorm * tnorm);
    const double pad = 2.0 * eps * tnorm + pivmin;
    lo -= pad;
    hi += pad;
    // sturm_count(lo) == 0 and sturm_count(hi) == m; the largest eigenvalue is
    // the smallest x with count(x) == m.
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (sturm_count(d, e, m, mid, pivmin) >= m) hi = mid; else lo = mid;
        if (hi - lo <= 2.0 * eps * std::max(std::fabs(lo), std::fabs(hi))) break;
    }
    const double t = 0.5 * (lo + hi);
    *theta = t;
    // Inverse iteration.
    std::vector<double> x(m, 1.0);
    const double tiny = eps * std::max(tnorm, std::numeric_limits<double>::min());
    const double shift = t + 4.0 * eps * std::max(tnorm, std::fabs(t));
    for (int it = 0; it < 4; ++it) {
        tridiag_solve(d, e, m, shift, tiny, x);
        double s = 0.0;
        for (double v : x) s += v * v;
        s = std::sqrt(s);
        if (!(s > 0.0) || !std::isfinite(s)) {
            std::fill(x.begin(), x.end(), 1.0 / std::sqrt(static_cast<double>(m)));
            break;
        }
        for (double& v : x) v /= s;
    }
    for (int64_t i = 0; i < m; ++i) vec[i] = x[i];
}

}  // namespace psdgb
