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

// grid (nblk, ceil(n/32)), 32 threads: candidate c (0 = largest) of block b per thread.
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
    // FP64 bisection from the FP32 bracket, widened until the Sturm counts confirm it
    const double x = a.w[(size_t)b * n + j] * inv;
    double del = 64.0 * FLT_EPSILON, lo = x - del, hi = x + del;
    bool ok = false;
    for (int k = 0; k < 8 && !ok; k++) {
        lo = x - del;
        hi = x + del;
        ok = sturm64(n, d, e2, lo, pivmin) <= j && sturm64(n, d, e2, hi, pivmin) > j;
        del *= 8.0;
    }
    if (!ok) {
        lo = -1.0;
        hi = 1.0;
        if (!(sturm64(n, d, e2, lo, pivmin) <= j && sturm64(n, d, e2, hi, pivmin) > j)) atomicMax(&a.status[b], 1);
    }
    for (int it = 0; it < 96; it++) {
        const double mid = 0.5 * (lo + hi);
        if (!(hi - lo > 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + 4.0 * pivmin) || mid <= lo || mid >= hi) break;
        if (sturm64(n, d, e2, mid, pivmin) > j) hi = mid;
        else lo = mid;
    }
    const double lam = 0.5 * (lo + hi);
    a.w[(size_t)b * n + j] = lam * sc;
    // twisted factorisation of T - lam I: top-down pivots G and multipliers L, then bottom-up
    double g = d[0] - lam;
    if (fabs(g) < pivmin) g = -pivmin;
    for (int i = 0; i + 1 < n; i++) {
        a.G[i * K + col] = g;
        const double l = e[i] / g;
        a.L[i * K + col] = l;
        g = d[i + 1] - lam - l * e[i];
        if (fabs(g) < pivmin) g = -pivmin;
    }
    a.G[(size_t)(n - 1) * K + col] = g;
    double h = d[n - 1] - lam;
    if (fabs(h) < pivmin) h = -pivmin;
    int r = n - 1;
    double best = fabs(g);  // gamma_{n-1} = G_{n-1}
    for (int i = n - 1; i >= 1; i--) {
        const double u = e[i - 1] / h;
        a.U[i * K + col] = u;
        h = d[i - 1] - lam - u * e[i - 1];
        if (fabs(h) < pivmin) h = -pivmin;
        // gamma_{i-1} = G_{i-1} + H_{i-1} - (d_{i-1} - lam)
        const double gam = a.G[(size_t)(i - 1) * K + col] + h - (d[i - 1] - lam);
        if (fabs(gam) < best) {
            best = fabs(gam);
            r = i - 1;
        }
    }
    // z_r = 1, then outward: z_i = -L_i z_{i+1} above r, z_i = -U_i z_{i-1} below r
    double nrm = 1.0;
    a.Z[(size_t)r * K + col] = 1.0;
    double z = 1.0;
    for (int i = r - 1; i >= 0; i--) {
        z = -a.L[i * K + col] * z;
        a.Z[i * K + col] = z;
        nrm += z * z;
    }
    z = 1.0;
    for (int i = r + 1; i < n; i++) {
        z = -a.U[i * K + col] * z;
        a.Z[i * K + col] = z;
        nrm += z * z;
    }
    const double s = 1.0 / sqrt(nrm);
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

// x = H_0 H_1 ... H_{n-3} z for 32 candidates of block b per CTA (one warp, a lane per
// candidate); the vectors live in shared memory when n <= 512.  Writes column n-1-c of the
// block (ascending order, column-major).
template <bool kShared>
__global__ void __launch_bounds__(32) backtransform_kernel(VecArgs a, const double* __restrict__ Vall,
                                                           const double* __restrict__ tau, double* __restrict__ out) {
    extern __shared__ double zs[];
    const int b = blockIdx.x, n = a.n, kc = a.kc[b];
    if ((int)blockIdx.y * 32 >= kc) return;
    const int c = blockIdx.y * 32 + threadIdx.x;
    const bool act = c < kc;
    const size_t K = (size_t)a.ktot;
    const int col = a.koff[b] + (act ? c : 0);
    double* zg = a.Z + col;  // stride K
    double* z = kShared ? zs + threadIdx.x : zg;
    const size_t st = kShared ? 32 : K;
    if (kShared)
        for (int i = 0; i < n; i++) z[i * st] = act ? zg[i * K] : 0.0;
    const double* V = Vall + (size_t)b * n * n;
    for (int c2 = n - 3; c2 >= 0; c2--) {
        const double tc = tau[(size_t)b * n + c2];
        if (tc == 0.0) continue;
        const double* v = V + (size_t)c2 * n;
        double s0 = z[(size_t)(c2 + 1) * st], s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int i = c2 + 2;
        for (; i + 3 < n; i += 4) {
            s0 = fma(v[i], z[(size_t)i * st], s0);
            s1 = fma(v[i + 1], z[(size_t)(i + 1) * st], s1);
            s2 = fma(v[i + 2], z[(size_t)(i + 2) * st], s2);
            s3 = fma(v[i + 3], z[(size_t)(i + 3) * st], s3);
        }
        for (; i < n; i++) s0 = fma(v[i], z[(size_t)i * st], s0);
        const double f = tc * ((s0 + s1) + (s2 + s3));
        z[(size_t)(c2 + 1) * st] -= f;
        for (i = c2 + 2; i < n; i++) z[(size_t)i * st] = fma(-f, v[i], z[(size_t)i * st]);
    }
    if (!act) return;
    double* o = out + (size_t)b * n * n + (size_t)(n - 1 - c) * n;
    for (int i = 0; i < n; i++) o[i] = z[(size_t)i * st];
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
    vectors_kernel<<<grid, 32, 0, s>>>(a);
    cluster_kernel<<<p.nblk, 256, 0, s>>>(a, 1e-6);
    if (p.n <= 512) {
        const size_t smem = sizeof(double) * 32 * p.n;
        OPSEC_CUDA(cudaFuncSetAttribute(backtransform_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        max_dynamic_smem((const void*)backtransform_kernel<true>)));
        backtransform_kernel<true><<<grid, 32, smem, s>>>(a, p.V, p.tau, p.out);
    } else {
        backtransform_kernel<false><<<grid, 32, 0, s>>>(a, p.V, p.tau, p.out);
    }
    OPSEC_CUDA(cudaGetLastError());
    *launches += 3;
}

}  // namespace opsec
