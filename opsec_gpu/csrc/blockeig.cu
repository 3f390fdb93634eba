// Batched symmetric eigensolver for the azimuthal blocks of a full-sky signal matrix.
//
// The KL step (klt.cpp:173-248) needs the top-M eigenpairs of S; the reference gets them from
// ARPACK's implicitly restarted Lanczos on the whole S (ParpackSolver.cpp:111-123).  On a
// full-sky grid S is block diagonal in the azimuthal order m (and the mu parity), so the engine
// solves the blocks: every eigenvalue of every block (the global top-M cut needs them all), but
// eigenvectors only for the block eigenvalues that can survive the cut.
//
//   1. tridiag_kernel: Householder reduction A = Q T Q^T of every block, one cluster of four CTAs
//      per block (the lower triangle stays in L2; each step is a fused pass that applies the
//      previous reflector's rank-2 update and forms the next reflector's product A v).  FP64.
//   2. spectrum_kernel: every eigenvalue of every T by bisection on FP32 Sturm counts of the
//      power-of-two-scaled T (to ~1e-6 of the block norm): enough to decide which block
//      eigenvalues can reach the global cut.
//   3. (host) the candidates: per block, the eigenvalues within a safe margin of the cut.
//   4. vectors_kernel: each candidate's eigenvalue by FP64 bisection from its FP32 bracket, then
//      its eigenvector of T by a twisted factorisation (the stationary top-down and bottom-up
//      LDL^T factorisations of T - lambda I meet at the index where the residual is smallest).
//   5. cluster_kernel: Gram-Schmidt (twice) inside clusters of candidates closer than 1e-6 of the
//      block norm, where separately computed vectors need not be orthogonal.
//   6. backtransform_kernel: x = Q z by the stored reflectors, written as the block's eigenvector
//      column (ascending eigenvalue order, the layout of LAPACK's syevd).
#include <cooperative_groups.h>

#include <cfloat>
#include <cmath>

#include "engine.h"

namespace cg = cooperative_groups;

namespace opsec {
namespace {

constexpr int kCl = 4;            // CTAs per block in the reduction (one thread-block cluster)
constexpr int kTT = 512;          // threads per CTA
constexpr int kTW = kTT / 32;     // warps per CTA
constexpr int kMaxN = 1024;       // largest block the reduction keeps its per-warp rows for

// Deterministic CTA-wide sum: the same inputs give the same bits in every CTA of the cluster.
__device__ double cta_sum(double x, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp] = x;
    __syncthreads();
    if (warp == 0) {
        double y = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
        if (lane == 0) red[32] = y;
    }
    __syncthreads();
    const double r = red[32];
    __syncthreads();
    return r;
}

// Householder reflector of the pivot column c held in col[c..n): d_c = col[c], and
// H = I - tau v v^T with v[c+1] = 1 maps col[c+1..n) onto beta e_{c+1}.  Every CTA of the
// cluster computes it from the same data and gets the same bits.
__device__ void householder(int n, int c, const double* col, double* v, double* tau_out, double* beta_out,
                            double* red) {
    const int t = threadIdx.x;
    double s = 0.0;
    for (int i = c + 2 + t; i < n; i += blockDim.x) s += col[i] * col[i];
    const double s2 = cta_sum(s, red);
    const double x0 = col[c + 1];
    double tau = 0.0, beta = x0, scal = 0.0;
    if (s2 > 0.0) {
        const double nrm = sqrt(x0 * x0 + s2);
        beta = x0 >= 0.0 ? -nrm : nrm;
        tau = (beta - x0) / beta;
        scal = 1.0 / (x0 - beta);
    }
    for (int i = c + 2 + t; i < n; i += blockDim.x) v[i] = col[i] * scal;
    if (t == 0) {
        v[c + 1] = 1.0;
        *tau_out = tau;
        *beta_out = beta;
    }
}

// One fused pass over the columns j in [j0, n) of the lower triangle: a -= v_i w_j + w_i v_j
// (when upd), then the partial products p += A vn into this warp's row of pw (when sym).
__device__ void fused_pass(int n, int j0, double* __restrict__ A, const double* vk, const double* wk,
                           const double* vn, double* pw, bool upd, bool sym, int gwarp, int nwarps) {
    const int lane = threadIdx.x & 31;
    const int L = n - j0;
    for (int q0 = 0; q0 < L; q0 += nwarps) {
        // snake order: the long columns at the front go to alternate ends of the warp list
        const int odd = (q0 / nwarps) & 1;
        const int q = q0 + (odd ? nwarps - 1 - gwarp : gwarp);
        if (q >= L) continue;
        const int j = j0 + q;
        double* col = A + (size_t)j * n;
        const double vkj = upd ? vk[j] : 0.0, wkj = upd ? wk[j] : 0.0, vnj = sym ? vn[j] : 0.0;
        double cacc = 0.0;
        for (int i = j + lane; i < n; i += 32) {
            double a = col[i];
            if (upd) {
                a = fma(-vk[i], wkj, a);
                a = fma(-wk[i], vkj, a);
                col[i] = a;
            }
            if (sym) {
                pw[i] = fma(a, vnj, pw[i]);
                if (i != j) cacc = fma(a, vn[i], cacc);
            }
        }
        if (sym) {
#pragma unroll
            for (int o = 16; o; o >>= 1) cacc += __shfl_xor_sync(0xffffffffu, cacc, o);
            if (lane == 0) pw[j] += cacc;
        }
    }
}

// Householder tridiagonalisation of block b = blockIdx.x / kCl (column-major, lower triangle
// read and updated; n >= 3).  Outputs T (dg, eg), the reflectors V[b][c][i] (v[c+1] = 1) and tau.
__global__ void __cluster_dims__(kCl, 1, 1) __launch_bounds__(kTT, 1)
tridiag_kernel(int n, double* __restrict__ Aall, double* __restrict__ Vall, double* __restrict__ tau,
               double* __restrict__ dg, double* __restrict__ eg) {
    extern __shared__ double sm[];
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int b = blockIdx.x / kCl;
    const int t = threadIdx.x, warp = t >> 5;
    double* A = Aall + (size_t)b * n * n;
    double* V = Vall + (size_t)b * n * n;
    double* vk = sm;
    double* wk = vk + n;
    double* vn = wk + n;
    double* col = vn + n;
    double* buf = col + n;           // [2][n] this CTA's partial A v, read by the whole cluster
    double* pw = buf + 2 * n;        // [kTW][n] per-warp partial rows
    double* red = pw + (size_t)kTW * n;  // 40 doubles
    double* scal = red + 40;         // tau of the next reflector, beta
    double* pw_mine = pw + (size_t)warp * n;
    const int gwarp = rank * kTW + warp, nwarps = kCl * kTW;

    // pivot column 0 and the first reflector
    for (int i = t; i < n; i += kTT) col[i] = A[i];
    __syncthreads();
    householder(n, 0, col, vn, &scal[0], &scal[1], red);
    __syncthreads();
    if (rank == 0) {
        for (int i = 1 + t; i < n; i += kTT) V[i] = vn[i];
        if (t == 0) {
            dg[(size_t)b * n] = col[0];
            eg[(size_t)b * n] = scal[1];
            tau[(size_t)b * n] = scal[0];
        }
    }
    for (int i = 1 + (t & 31); i < n; i += 32) pw_mine[i] = 0.0;
    __syncwarp();
    fused_pass(n, 1, A, vk, wk, vn, pw_mine, false, true, gwarp, nwarps);
    __syncthreads();
    for (int i = 1 + t; i < n; i += kTT) {
        double s = 0.0;
        for (int w = 0; w < kTW; w++) s += pw[(size_t)w * n + i];
        buf[i] = s;  // parity 0
    }
    cluster.sync();

    for (int c = 0; c <= n - 3; c++) {
        const double tc = scal[0];
        // (a) v_c, p_c = A v_c from the four CTAs (fixed order), w_c = y - (tau/2)(y.v) v
        const double* rb[kCl];
#pragma unroll
        for (int r = 0; r < kCl; r++) rb[r] = cluster.map_shared_rank(buf + (size_t)(c & 1) * n, r);
        double part = 0.0;
        for (int i = c + 1 + t; i < n; i += kTT) {
            double p = 0.0;
#pragma unroll
            for (int r = 0; r < kCl; r++) p += rb[r][i];
            const double y = tc * p;
            vk[i] = vn[i];
            wk[i] = y;
            part += y * vn[i];
        }
        const double alpha = 0.5 * tc * cta_sum(part, red);
        for (int i = c + 1 + t; i < n; i += kTT) wk[i] -= alpha * vk[i];
        __syncthreads();
        // (b) pivot column c+1 under the update, the next reflector
        const int c1 = c + 1;
        const double vkc = vk[c1], wkc = wk[c1];
        for (int i = c1 + t; i < n; i += kTT) {
            double a = A[(size_t)c1 * n + i];
            a = fma(-vk[i], wkc, a);
            a = fma(-wk[i], vkc, a);
            col[i] = a;
        }
        __syncthreads();
        householder(n, c1, col, vn, &scal[0], &scal[1], red);
        __syncthreads();
        if (rank == 0) {
            for (int i = c1 + 1 + t; i < n; i += kTT) V[(size_t)c1 * n + i] = vn[i];
            if (t == 0) {
                dg[(size_t)b * n + c1] = col[c1];
                eg[(size_t)b * n + c1] = scal[1];
                tau[(size_t)b * n + c1] = scal[0];
            }
        }
        // (c) columns c+2 .. n-1: update by (v_c, w_c); partial A v_{c+1} for the next step
        const bool sym = c1 <= n - 3;
        if (sym) {
            for (int i = c1 + 1 + (t & 31); i < n; i += 32) pw_mine[i] = 0.0;
            __syncwarp();
        }
        fused_pass(n, c1 + 1, A, vk, wk, vn, pw_mine, true, sym, gwarp, nwarps);
        __syncthreads();
        if (sym) {
            double* bo = buf + (size_t)(c1 & 1) * n;
            for (int i = c1 + 1 + t; i < n; i += kTT) {
                double s = 0.0;
                for (int w = 0; w < kTW; w++) s += pw[(size_t)w * n + i];
                bo[i] = s;
            }
        }
        cluster.sync();
    }
    if (rank == 0 && t == 0) {
        dg[(size_t)b * n + n - 1] = A[(size_t)(n - 1) * n + n - 1];
        eg[(size_t)b * n + n - 1] = 0.0;
        tau[(size_t)b * n + n - 1] = 0.0;
    }
}

// ---------------------------------------------------------------- spectrum (FP32 bisection)
__device__ __forceinline__ int sturm32(int n, const float* d, const float* e2, float s, float pivmin) {
    float q = d[0] - s;
    if (fabsf(q) < pivmin) q = -pivmin;
    int cnt = q < 0.0f;
    for (int i = 1; i < n; i++) {
        q = d[i] - s - e2[i - 1] / q;
        if (fabsf(q) < pivmin) q = -pivmin;
        cnt += q < 0.0f;
    }
    return cnt;
}

// Power-of-two scale of a block (>= its Gershgorin bound), so that scaling is exact.
__device__ double block_scale(int n, const double* d, const double* e, double* red) {
    double m = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double r = fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0);
        m = fmax(m, r);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    double g = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) g = fmax(g, red[w]);
    __syncthreads();
    if (!(g > 0.0)) return 1.0;
    int ex;
    frexp(g, &ex);
    return ldexp(1.0, ex);  // 2^ex > g
}

// Every eigenvalue j (ascending) of block b to ~1e-6 of its scale; grid (nblk, ceil(n/256)).
__global__ void __launch_bounds__(256) spectrum_kernel(int n, const double* __restrict__ dg,
                                                       const double* __restrict__ eg, double* __restrict__ w,
                                                       double* __restrict__ scale_out) {
    __shared__ float d[kMaxN], e2[kMaxN];
    __shared__ double red[32];
    const int b = blockIdx.x;
    const double* db = dg + (size_t)b * n;
    const double* ebk = eg + (size_t)b * n;
    const double sc = block_scale(n, db, ebk, red);
    const double inv = 1.0 / sc;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        d[i] = (float)(db[i] * inv);
        const float ei = (float)(ebk[i] * inv);
        e2[i] = ei * ei;
    }
    __syncthreads();
    if (blockIdx.y == 0 && threadIdx.x == 0) scale_out[b] = sc;
    const int j = blockIdx.y * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const float pivmin = 1e-30f;
    float lo = -1.0f, hi = 1.0f;  // the scaled spectrum lies in (-1, 1)
    for (int it = 0; it < 40 && hi - lo > 2.5e-7f; it++) {
        const float mid = 0.5f * (lo + hi);
        if (sturm32(n, d, e2, mid, pivmin) > j) hi = mid;
        else lo = mid;
    }
    w[(size_t)b * n + j] = 0.5 * ((double)lo + (double)hi) * sc;
}

// ---------------------------------------------------------------- candidate eigenpairs (FP64)
__device__ __forceinline__ int sturm64(int n, const double* d, const double* e2, double s, double pivmin) {
    double q = d[0] - s;
    if (fabs(q) < pivmin) q = -pivmin;
    int cnt = q < 0.0;
    for (int i = 1; i < n; i++) {
        q = d[i] - s - e2[i - 1] / q;
        if (fabs(q) < pivmin) q = -pivmin;
        cnt += q < 0.0;
    }
    return cnt;
}

struct VecArgs {
    int n, nblk, ktot;
    const int* kc;       // [nblk] candidates per block (the top kc[b] eigenvalues)
    const int* koff;     // [nblk] their first column in the [row][ktot] arrays
    const double* dg;    // [nblk][n]
    const double* eg;
    const double* scale; // [nblk] power-of-two scale of each block
    double* w;           // [nblk][n] ascending: approximate in, candidates refined out
    double* Z;           // [n][ktot] eigenvectors of T, then of the block
    double* L;           // [n][ktot] scratch: top-down multipliers
    double* U;           // [n][ktot] scratch: bottom-up multipliers
    double* G;           // [n][ktot] scratch: top-down pivots
    int* status;         // [nblk]: 0, or 1 when a bracket could not be confirmed, 2 when a cluster degenerated
};

// Twisted factorisation of T - s I (scaled T): the stationary top-down pivots G and multipliers
// L, the bottom-up multipliers U, the twist index r where |gamma_r| is least, and the vector
// z with z_r = 1 (rows i < r from L, rows i > r from U), written to column col of Z.
// Returns the Rayleigh quotient correction gamma_r / |z|^2 (z^T (T - s I) z / z^T z) and
// leaves |z|^2 in *nrm2.
__device__ double twisted(int n, const double* d, const double* e, double s, double pivmin, size_t K, int col,
                          double* G, double* L, double* U, double* Z, double* nrm2) {
    double g = d[0] - s;
    if (fabs(g) < pivmin) g = -pivmin;
    for (int i = 0; i + 1 < n; i++) {
        G[i * K + col] = g;
        const double l = e[i] / g;
        L[i * K + col] = l;
        g = d[i + 1] - s - l * e[i];
        if (fabs(g) < pivmin) g = -pivmin;
    }
    G[(size_t)(n - 1) * K + col] = g;
    double h = d[n - 1] - s;
    if (fabs(h) < pivmin) h = -pivmin;
    int r = n - 1;
    double gam_r = g, best = fabs(g);  // gamma_{n-1} = G_{n-1}
    for (int i = n - 1; i >= 1; i--) {
        const double u = e[i - 1] / h;
        U[i * K + col] = u;
        h = d[i - 1] - s - u * e[i - 1];
        if (fabs(h) < pivmin) h = -pivmin;
        // gamma_{i-1} = G_{i-1} + H_{i-1} - (d_{i-1} - s)
        const double gam = G[(size_t)(i - 1) * K + col] + h - (d[i - 1] - s);
        if (fabs(gam) < best) {
            best = fabs(gam);
            gam_r = gam;
            r = i - 1;
        }
    }
    double nrm = 1.0, z = 1.0;
    Z[(size_t)r * K + col] = 1.0;
    for (int i = r - 1; i >= 0; i--) {
        z = -L[i * K + col] * z;
        Z[i * K + col] = z;
        nrm += z * z;
    }
    z = 1.0;
    for (int i = r + 1; i < n; i++) {
        z = -U[i * K + col] * z;
        Z[i * K + col] = z;
        nrm += z * z;
    }
    *nrm2 = nrm;
    return gam_r / nrm;
}

// grid (nblk, ceil(n/32)), 32 threads: candidate c (0 = largest) of block b per thread.
// The FP32 estimate's bracket is confirmed by two FP64 Sturm counts.  An eigenvalue alone in
// its bracket is refined by Rayleigh-quotient iteration on twisted factorisations (cubic
// convergence; the iterate must stay in the bracket); an eigenvalue sharing its bracket is
// bisected to full precision first.  The last twisted factorisation gives the vector.
__global__ void __launch_bounds__(32) vectors_kernel(VecArgs a) {
    __shared__ double d[kMaxN], e[kMaxN], e2[kMaxN];
    const int b = blockIdx.x, n = a.n;
    const int kc = a.kc[b];
    if ((int)blockIdx.y * 32 >= kc) return;
    const double sc = a.scale[b], inv = 1.0 / sc;
    for (int i = threadIdx.x; i < n; i += 32) {
        d[i] = a.dg[(size_t)b * n + i] * inv;
        e[i] = a.eg[(size_t)b * n + i] * inv;
        e2[i] = e[i] * e[i];
    }
    __syncthreads();
    const int c = blockIdx.y * 32 + threadIdx.x;
    if (c >= kc) return;
    const int j = n - 1 - c;  // ascending index
    const int col = a.koff[b] + c;
    const size_t K = (size_t)a.ktot;
    const double pivmin = 1e-290;
    const double x = a.w[(size_t)b * n + j] * inv;
    double del = 64.0 * FLT_EPSILON, lo = x - del, hi = x + del;
    int clo = 0, chi = 0;
    bool ok = false;
    for (int k = 0; k < 8 && !ok; k++) {
        lo = x - del;
        hi = x + del;
        clo = sturm64(n, d, e2, lo, pivmin);
        chi = sturm64(n, d, e2, hi, pivmin);
        ok = clo <= j && chi > j;
        del *= 8.0;
    }
    if (!ok) {
        lo = -1.0;
        hi = 1.0;
        clo = sturm64(n, d, e2, lo, pivmin);
        chi = sturm64(n, d, e2, hi, pivmin);
        if (!(clo <= j && chi > j)) atomicMax(&a.status[b], 1);
    }
    double nrm2 = 1.0, lam = x;
    bool done = false;
    if (chi - clo == 1) {
        // converged when the correction is below 1e-14 of the block scale (T is scaled to norm
        // < 1), or when it stops shrinking at a level below 1e-10 (the rounding floor of gamma)
        double s = fmin(fmax(x, lo), hi), prev = 1.0;
        for (int it = 0; it < 8; it++) {
            const double dl = twisted(n, d, e, s, pivmin, K, col, a.G, a.L, a.U, a.Z, &nrm2);
            const double s1 = s + dl;
            if (!(s1 > lo && s1 < hi)) break;  // left the bracket: bisect instead
            if (fabs(dl) <= 1e-14 || (fabs(dl) <= 1e-10 && fabs(dl) > 0.25 * prev)) {
                lam = s1;
                done = true;
                break;
            }
            prev = fabs(dl);
            s = s1;
        }
    }
    if (!done) {
        for (int it = 0; it < 96; it++) {
            const double mid = 0.5 * (lo + hi);
            if (!(hi - lo > 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + 4.0 * pivmin) || mid <= lo || mid >= hi)
                break;
            if (sturm64(n, d, e2, mid, pivmin) > j) hi = mid;
            else lo = mid;
        }
        lam = 0.5 * (lo + hi);
        twisted(n, d, e, lam, pivmin, K, col, a.G, a.L, a.U, a.Z, &nrm2);
    }
    a.w[(size_t)b * n + j] = lam * sc;
    const double s = 1.0 / sqrt(nrm2);
    if (!isfinite(s) || !(s > 0.0)) atomicMax(&a.status[b], 3);
    for (int i = 0; i < n; i++) a.Z[i * K + col] *= s;
}

// Gram-Schmidt, twice, inside clusters of close candidates of block b (one CTA per block).
__global__ void __launch_bounds__(256) cluster_kernel(VecArgs a, double tol) {
    __shared__ double red[40];
    const int b = blockIdx.x, n = a.n, kc = a.kc[b];
    const size_t K = (size_t)a.ktot;
    const double* wb = a.w + (size_t)b * n;
    const double sc = a.scale[b];
    const int c0 = a.koff[b];
    int start = 0;
    for (int c = 1; c < kc; c++) {
        // wb is ascending: candidate c has index n-1-c
        const bool close = wb[n - c] - wb[n - 1 - c] < tol * sc;
        if (!close) {
            start = c;
            continue;
        }
        for (int pass = 0; pass < 2; pass++) {
            for (int k = start; k < c; k++) {
                double s = 0.0;
                for (int i = threadIdx.x; i < n; i += blockDim.x) s += a.Z[i * K + c0 + k] * a.Z[i * K + c0 + c];
                const double dot = cta_sum(s, red);
                for (int i = threadIdx.x; i < n; i += blockDim.x) a.Z[i * K + c0 + c] -= dot * a.Z[i * K + c0 + k];
                __syncthreads();
            }
            double s = 0.0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) s += a.Z[i * K + c0 + c] * a.Z[i * K + c0 + c];
            const double nrm = sqrt(cta_sum(s, red));
            if (pass == 0 && nrm < 1e-2 && threadIdx.x == 0) atomicMax(&a.status[b], 2);
            const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) a.Z[i * K + c0 + c] *= inv;
            __syncthreads();
        }
    }
}

// x = H_0 H_1 ... H_{n-3} z for G candidates of block b per CTA (grid (nblk, ceil(n/G)), 256
// threads).  The G vectors live in shared memory ([row][G]), each reflector row is staged once
// per CTA, thread t works on vector t % G over the rows t / G + 8 k, and the G dot products are
// summed over the 256 / G row groups in a fixed order.  Writes column n-1-c of the block
// (ascending order, column-major).
constexpr int kBT = 256;
template <int G>
__global__ void __launch_bounds__(kBT) backtransform_kernel(VecArgs a, const double* __restrict__ Vall,
                                                            const double* __restrict__ tau, double* __restrict__ out) {
    extern __shared__ double bsm[];
    constexpr int R = kBT / G;  // row groups
    const int b = blockIdx.x, n = a.n, kc = a.kc[b];
    const int c0 = blockIdx.y * G;
    if (c0 >= kc) return;
    double* z = bsm;                       // [n][G]
    double* v = z + (size_t)n * G;         // [n] reflector row
    double* part = v + n;                  // [R][G]
    double* f = part + R * G;              // [G]
    const int t = threadIdx.x, g = t % G, rg = t / G;
    const size_t K = (size_t)a.ktot;
    const int ng = min(G, kc - c0);
    for (int idx = t; idx < n * G; idx += kBT) {
        const int i = idx / G, gg = idx % G;
        z[idx] = gg < ng ? a.Z[(size_t)i * K + a.koff[b] + c0 + gg] : 0.0;
    }
    const double* V = Vall + (size_t)b * n * n;
    const double* tb = tau + (size_t)b * n;
    for (int c2 = n - 3; c2 >= 0; c2--) {
        const double tc = tb[c2];
        if (tc == 0.0) continue;  // uniform over the CTA
        __syncthreads();          // the previous update is done with v
        for (int i = c2 + 1 + t; i < n; i += kBT) v[i] = V[(size_t)c2 * n + i];
        __syncthreads();
        double s0 = 0.0, s1 = 0.0;
        int i = c2 + 1 + rg;
        for (; i + R < n; i += 2 * R) {
            s0 = fma(v[i], z[(size_t)i * G + g], s0);
            s1 = fma(v[i + R], z[(size_t)(i + R) * G + g], s1);
        }
        if (i < n) s0 = fma(v[i], z[(size_t)i * G + g], s0);
        part[rg * G + g] = s0 + s1;
        __syncthreads();
        if (t < G) {
            double s = 0.0;
            for (int r = 0; r < R; r++) s += part[r * G + t];
            f[t] = tc * s;
        }
        __syncthreads();
        const double fg = f[g];
        for (i = c2 + 1 + rg; i < n; i += R) z[(size_t)i * G + g] = fma(-fg, v[i], z[(size_t)i * G + g]);
    }
    __syncthreads();
    for (int gg = 0; gg < ng; gg++) {
        double* o = out + (size_t)b * n * n + (size_t)(n - 1 - (c0 + gg)) * n;
        for (int i2 = t; i2 < n; i2 += kBT) o[i2] = z[(size_t)i2 * G + gg];
    }
}

}  // namespace

size_t blockeig_tridiag_smem(int n) { return sizeof(double) * ((size_t)(6 + kTW) * n + 48); }

bool blockeig_supported(int n) {
    return n >= 3 && n <= kMaxN && blockeig_tridiag_smem(n) <= (size_t)max_dynamic_smem((const void*)tridiag_kernel);
}

void launch_blockeig_tridiag(int n, int nblk, double* A, double* V, double* tau, double* dg, double* eg,
                             cudaStream_t s, long long* launches) {
    const size_t smem = blockeig_tridiag_smem(n);
    OPSEC_CUDA(cudaFuncSetAttribute(tridiag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    max_dynamic_smem((const void*)tridiag_kernel)));
    tridiag_kernel<<<nblk * kCl, kTT, smem, s>>>(n, A, V, tau, dg, eg);
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;
}

void launch_blockeig_spectrum(int n, int nblk, const double* dg, const double* eg, double* w, double* scale,
                              cudaStream_t s, long long* launches) {
    spectrum_kernel<<<dim3(nblk, (n + 255) / 256), 256, 0, s>>>(n, dg, eg, w, scale);
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;
}

void launch_blockeig_vectors(const BlockEigVectors& p, cudaStream_t s, long long* launches) {
    VecArgs a{p.n, p.nblk, p.ktot, p.kc, p.koff, p.dg, p.eg, p.scale, p.w, p.Z, p.L, p.U, p.G, p.status};
    const dim3 grid(p.nblk, (p.n + 31) / 32);
    if (g_clock) g_clock->begin("blockeig_pairs", s);
    vectors_kernel<<<grid, 32, 0, s>>>(a);
    if (g_clock) g_clock->end(s);
    cluster_kernel<<<p.nblk, 256, 0, s>>>(a, 1e-6);
    if (g_clock) g_clock->begin("blockeig_back", s, 2.0 * p.n * (double)p.n * p.ktot);
    if (p.n <= 512) {
        constexpr int G = 32;
        const size_t smem = sizeof(double) * ((size_t)p.n * G + p.n + kBT + G);
        OPSEC_CUDA(cudaFuncSetAttribute(backtransform_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        max_dynamic_smem((const void*)backtransform_kernel<G>)));
        backtransform_kernel<G><<<dim3(p.nblk, (p.n + G - 1) / G), kBT, smem, s>>>(a, p.V, p.tau, p.out);
    } else {
        constexpr int G = 16;
        const size_t smem = sizeof(double) * ((size_t)p.n * G + p.n + kBT + G);
        OPSEC_CUDA(cudaFuncSetAttribute(backtransform_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        max_dynamic_smem((const void*)backtransform_kernel<G>)));
        backtransform_kernel<G><<<dim3(p.nblk, (p.n + G - 1) / G), kBT, smem, s>>>(a, p.V, p.tau, p.out);
    }
    if (g_clock) g_clock->end(s);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 3;
}

}  // namespace opsec
