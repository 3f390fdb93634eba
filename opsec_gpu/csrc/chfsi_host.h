// chfsi_host.h -- the host-side numerics of the iterative eigensolver (chfsi.cu): the extreme
// eigenvalues of the Lanczos tridiagonal, the block size and the Chebyshev degree rule.
// Plain C++, so that CPU tests compile and check this code itself.
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

namespace opsec {
namespace chfsi {

constexpr double kMaxGain = 1e4;  // largest filter gain between the top and the M-th Ritz value

// eigenvalues below x of the symmetric tridiagonal (diagonal a, off-diagonal b): the negative
// terms of the Sturm sequence (LDL^T pivots of T - x I)
inline int sturm_count(const std::vector<double>& a, const std::vector<double>& b, double x) {
    int cnt = 0;
    double q = 1.0;
    for (size_t i = 0; i < a.size(); i++) {
        const double bb = i ? b[i - 1] * b[i - 1] : 0.0;
        q = a[i] - x - (i ? bb / q : 0.0);
        if (q == 0.0) q = -1e-300;
        if (q < 0.0) cnt++;
    }
    return cnt;
}

// k-th smallest eigenvalue (0-based) by bisection inside the Gershgorin interval
inline double tridiag_eig(const std::vector<double>& a, const std::vector<double>& b, int k) {
    double lo = 1e300, hi = -1e300;
    for (size_t i = 0; i < a.size(); i++) {
        const double r = (i ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < a.size() ? std::fabs(b[i]) : 0.0);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
    }
    for (int it = 0; it < 200 && hi - lo > 1e-15 * std::max(std::fabs(lo), std::fabs(hi)); it++) {
        const double mid = 0.5 * (lo + hi);
        if (sturm_count(a, b, mid) > k)
            hi = mid;
        else
            lo = mid;
    }
    return 0.5 * (lo + hi);
}

// T_d(t) for t >= 1 (1 below)
inline double cheb(int d, double t) { return std::cosh(d * std::acosh(std::max(t, 1.0))); }

// block B = M + max(guard, 8), rounded up to a multiple of 32, at most N
inline int block_size(int N, int M, int guard) {
    const int B = std::min(N, M + std::max(guard, 8));
    return std::min(N, (B + 31) / 32 * 32);
}

// The Chebyshev degree of one filter step damping [lo, cut]: the largest d <= dmax whose gain
// T_d(t(hi)) / T_d(t(theta_M)) between the top of the spectrum and the M-th Ritz value stays
// at or below max_gain, t(x) = (x - c) / e mapping [lo, cut] onto [-1, 1]
inline int filter_degree(double lo, double cut, double hi, double theta_m, int dmax, double max_gain) {
    const double e = 0.5 * (cut - lo), c0 = 0.5 * (cut + lo);
    const double tM = (theta_m - c0) / e, th = (hi - c0) / e;
    int degree = 1;
    for (int d = 2; d <= dmax; d++)
        if (cheb(d, th) / std::max(cheb(d, tM), 1.0) <= max_gain) degree = d;
    return degree;
}

}  // namespace chfsi
}  // namespace opsec
