// C entry points over opsec_gpu/csrc/chfsi_host.h for tests/test_chfsi_host.py (compiled there
// with g++; no CUDA).
#include <vector>

#include "../opsec_gpu/csrc/chfsi_host.h"

extern "C" {

double chk_tridiag_eig(int n, const double* a, const double* b, int k) {
    std::vector<double> va(a, a + n), vb(b, b + (n > 0 ? n - 1 : 0));
    return opsec::chfsi::tridiag_eig(va, vb, k);
}

int chk_sturm_count(int n, const double* a, const double* b, double x) {
    std::vector<double> va(a, a + n), vb(b, b + (n > 0 ? n - 1 : 0));
    return opsec::chfsi::sturm_count(va, vb, x);
}

int chk_block_size(int N, int M, int guard) { return opsec::chfsi::block_size(N, M, guard); }

int chk_filter_degree(double lo, double cut, double hi, double theta_m, int dmax, double max_gain) {
    return opsec::chfsi::filter_degree(lo, cut, hi, theta_m, dmax, max_gain);
}

double chk_max_gain() { return opsec::chfsi::kMaxGain; }

}  // extern "C"
