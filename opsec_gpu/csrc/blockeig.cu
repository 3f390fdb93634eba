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
//      previous reflector's rank-2 update and forms the next reflector's product A v).  It runs
//      in double-FP32 (df64.h) but the reflectors' scalars (FP64, one warp).
//   2. spectrum_kernel: every eigenvalue of every T by bisection on FP32 Sturm counts of the
//      power-of-two-scaled T (to ~1e-6 of the block norm): enough to decide which block
//      eigenvalues can reach the global cut.
//   3. (host) the candidates: per block, the eigenvalues within a safe margin of the cut.
//   4. vectors_kernel: each candidate's eigenvalue from its FP32 bracket (confirmed by two FP64
//      Sturm counts, bisected until it holds this eigenvalue alone) by Rayleigh-quotient
//      iteration on twisted factorisations (the stationary top-down and bottom-up LDL^T
//      factorisations of T - s I meet at the index where the residual is smallest), then its
//      eigenvector of T from the last one.
//   5. cluster_kernel: Gram-Schmidt (twice) inside clusters of candidates closer than 1e-6 of the
//      block norm, where separately computed vectors need not be orthogonal.
//   6. backtransform_kernel: x = Q z by the stored reflectors (double-FP32), written as the
//      block's eigenvector column (ascending eigenvalue order, the layout of LAPACK's syevd).
#include <cooperative_groups.h>

#include <cfloat>
#include <cmath>

#include "df64.h"
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

// Deterministic CTA-wide double-FP32 sum (lane 0's butterfly result of each warp, then warp
// 0's): the same inputs give the same bits in every CTA of the cluster.
__device__ df cta_sum_df(df x, float2* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o; o >>= 1)
        x = df_add(x, df{__shfl_xor_sync(0xffffffffu, x.h, o), __shfl_xor_sync(0xffffffffu, x.l, o)});
    if (lane == 0) red[warp] = df_pack(x);
    __syncthreads();
    if (warp == 0) {
        df y = lane < (int)(blockDim.x >> 5) ? df_unpack(red[lane]) : df{0.f, 0.f};
#pragma unroll
        for (int o = 16; o; o >>= 1)
            y = df_add(y, df{__shfl_xor_sync(0xffffffffu, y.h, o), __shfl_xor_sync(0xffffffffu, y.l, o)});
        if (lane == 0) red[32] = df_pack(y);
    }
    __syncthreads();
    const df r = df_unpack(red[32]);
    __syncthreads();
    return r;
}

// Householder reflector of the pivot column c held in col[c..n) (double-FP32): H = I - tau v v^T
// with v[c+1] = 1 maps col[c+1..n) onto beta e_{c+1}.  The sum of squares and v in double-FP32,
// the scalars in FP64 by warp 0 alone (the FP64 pipe issues at 1/64 of the FP32 rate: once per
// CTA, not in every warp).  sc: tau, beta (FP64); sc2: tau, 1/(x0 - beta) as (hi, lo) pairs.
// Every CTA of the cluster computes it from the same data and gets the same bits.
__device__ void householder_df(int n, int c, const float2* col, float2* v, double* sc, float2* sc2, float2* red) {
    const int t = threadIdx.x;
    df s{0.f, 0.f};
    for (int i = c + 2 + t; i < n; i += blockDim.x) {
        const df x = df_unpack(col[i]);
        s = df_fma(s, x, x);
    }
    const df s2 = cta_sum_df(s, red);
    if (t < 32) {
        const double x0 = df_to(df_unpack(col[c + 1])), s2d = df_to(s2);
        double tau = 0.0, beta = x0, scal = 0.0;
        if (s2d > 0.0) {
            const double nrm = sqrt(x0 * x0 + s2d);
            beta = x0 >= 0.0 ? -nrm : nrm;
            tau = (beta - x0) / beta;
            scal = 1.0 / (x0 - beta);
        }
        if (t == 0) {
            sc[0] = tau;
            sc[1] = beta;
            sc2[0] = df_pack(df_from(tau));
            sc2[1] = df_pack(df_from(scal));
        }
    }
    __syncthreads();
    const df scal = df_unpack(sc2[1]);
    for (int i = c + 2 + t; i < n; i += blockDim.x) v[i] = df_pack(df_mul(df_unpack(col[i]), scal));
    if (t == 0) v[c + 1] = make_float2(1.f, 0.f);
}

// One fused pass over the columns j in [j0, n) of the lower triangle, in double-FP32 (the
// FP64 pipe is the bound otherwise): a -= v_i w_j + w_i v_j (when upd), then the partial
// products p += A vn into this warp's row of pw (when sym).  conv: the column still holds FP64
// values (the first pass), which are read as doubles and written back as (hi, lo) pairs in the
// same 8 bytes.
__device__ void fused_pass(int n, int j0, double* __restrict__ A, const float2* vk, const float2* wk,
                           const float2* vn, float2* pw, bool upd, bool sym, bool conv, int gwarp, int nwarps) {
    const int lane = threadIdx.x & 31;
    const int L = n - j0;
    float2* A2 = reinterpret_cast<float2*>(A);
    for (int q0 = 0; q0 < L; q0 += nwarps) {
        // snake order: the long columns at the front go to alternate ends of the warp list
        const int odd = (q0 / nwarps) & 1;
        const int q = q0 + (odd ? nwarps - 1 - gwarp : gwarp);
        if (q >= L) continue;
        const int j = j0 + q;
        const size_t cj = (size_t)j * n;
        const df vkj = upd ? df_unpack(vk[j]) : df{0.f, 0.f}, wkj = upd ? df_unpack(wk[j]) : df{0.f, 0.f};
        const df vnj = sym ? df_unpack(vn[j]) : df{0.f, 0.f};
        df cacc{0.f, 0.f};
        for (int i = j + lane; i < n; i += 32) {
            df a = conv ? df_from(A[cj + i]) : df_unpack(A2[cj + i]);
            if (upd) {
                a = df_fms(a, df_unpack(vk[i]), wkj);
                a = df_fms(a, df_unpack(wk[i]), vkj);
            }
            if (upd || conv) A2[cj + i] = df_pack(a);
            if (sym) {
                pw[i] = df_pack(df_fma(df_unpack(pw[i]), a, vnj));
                if (i != j) cacc = df_fma(cacc, a, df_unpack(vn[i]));
            }
        }
        if (sym) {
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                const df other{__shfl_xor_sync(0xffffffffu, cacc.h, o), __shfl_xor_sync(0xffffffffu, cacc.l, o)};
                cacc = df_add(cacc, other);
            }
            if (lane == 0) pw[j] = df_pack(df_add(df_unpack(pw[j]), cacc));
        }
    }
}

// this CTA's partial A v for rows [i0, n): the warps' rows summed in a fixed order
__device__ void reduce_warp_rows(int n, int i0, const float2* pw, float2* out) {
    for (int i = i0 + (int)threadIdx.x; i < n; i += kTT) {
        df s{0.f, 0.f};
        for (int w = 0; w < kTW; w++) s = df_add(s, df_unpack(pw[(size_t)w * n + i]));
        out[i] = df_pack(s);
    }
}

// Householder tridiagonalisation of block b = blockIdx.x / kCl (column-major, lower triangle
// read and updated; n >= 3).  Outputs T (dg, eg), the reflectors V[b][c][i] as (hi, lo) float
// pairs (v[c+1] = 1) and tau.  Everything runs in double-FP32 but the reflector's scalars
// (FP64, one warp): the O(n^2) fused pass and the O(n) work of each step (p = A v from the
// cluster, w, the pivot column, v).
__global__ void __cluster_dims__(kCl, 1, 1) __launch_bounds__(kTT, 1)
tridiag_kernel(int n, double* __restrict__ Aall, double* __restrict__ Vall, double* __restrict__ tau,
               double* __restrict__ dg, double* __restrict__ eg) {
    extern __shared__ double sm[];
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int b = blockIdx.x / kCl;
    const int t = threadIdx.x, warp = t >> 5;
    double* A = Aall + (size_t)b * n * n;
    float2* V = reinterpret_cast<float2*>(Vall) + (size_t)b * n * n;
    float2* vk2 = reinterpret_cast<float2*>(sm);  // (hi, lo): v and w of the step being applied,
    float2* wk2 = vk2 + n;                        // the next reflector, the pivot column
    float2* vn2 = wk2 + n;
    float2* col2 = vn2 + n;
    float2* buf = col2 + n;           // [2][n] this CTA's partial A v, read by the whole cluster
    float2* pw = buf + 2 * n;         // [kTW][n] per-warp partial rows
    float2* red = pw + (size_t)kTW * n;  // 40 pairs
    double* sc = reinterpret_cast<double*>(red + 40);  // tau, beta of the next reflector
    float2* sc2 = reinterpret_cast<float2*>(sc + 2);   // tau, 1/(x0 - beta) as pairs
    float2* pw_mine = pw + (size_t)warp * n;
    const int gwarp = rank * kTW + warp, nwarps = kCl * kTW;
    const float2* A2 = reinterpret_cast<const float2*>(A);

    // pivot column 0 and the first reflector
    for (int i = t; i < n; i += kTT) col2[i] = df_pack(df_from(A[i]));
    __syncthreads();
    householder_df(n, 0, col2, vn2, sc, sc2, red);
    __syncthreads();
    if (rank == 0) {
        for (int i = 1 + t; i < n; i += kTT) V[i] = vn2[i];
        if (t == 0) {
            dg[(size_t)b * n] = df_to(df_unpack(col2[0]));
            eg[(size_t)b * n] = sc[1];
            tau[(size_t)b * n] = sc[0];
        }
    }
    for (int i = 1 + (t & 31); i < n; i += 32) pw_mine[i] = make_float2(0.f, 0.f);
    __syncthreads();
    fused_pass(n, 1, A, vk2, wk2, vn2, pw_mine, false, true, true, gwarp, nwarps);
    __syncthreads();
    reduce_warp_rows(n, 1, pw, buf);  // parity 0
    cluster.sync();

    for (int c = 0; c <= n - 3; c++) {
        const df tc = df_unpack(sc2[0]);
        // (a) v_c, p_c = A v_c from the four CTAs (fixed order), w_c = y - (tau/2)(y.v) v
        const float2* rb[kCl];
#pragma unroll
        for (int r = 0; r < kCl; r++) rb[r] = cluster.map_shared_rank(buf + (size_t)(c & 1) * n, r);
        df part{0.f, 0.f};
        for (int i = c + 1 + t; i < n; i += kTT) {
            df p = df_unpack(rb[0][i]);
#pragma unroll
            for (int r = 1; r < kCl; r++) p = df_add(p, df_unpack(rb[r][i]));
            const df y = df_mul(tc, p);
            const float2 v = vn2[i];
            vk2[i] = v;
            wk2[i] = df_pack(y);
            part = df_fma(part, y, df_unpack(v));
        }
        const df yv = cta_sum_df(part, red);
        const df alpha = df_mul(tc, df{0.5f * yv.h, 0.5f * yv.l});
        for (int i = c + 1 + t; i < n; i += kTT)
            wk2[i] = df_pack(df_fms(df_unpack(wk2[i]), alpha, df_unpack(vk2[i])));
        __syncthreads();
        // (b) pivot column c+1 under the update, the next reflector
        const int c1 = c + 1;
        const df vkc = df_unpack(vk2[c1]), wkc = df_unpack(wk2[c1]);
        for (int i = c1 + t; i < n; i += kTT) {
            df a = df_unpack(A2[(size_t)c1 * n + i]);
            a = df_fms(a, df_unpack(vk2[i]), wkc);
            a = df_fms(a, df_unpack(wk2[i]), vkc);
            col2[i] = df_pack(a);
        }
        __syncthreads();
        householder_df(n, c1, col2, vn2, sc, sc2, red);
        __syncthreads();
        if (rank == 0) {
            for (int i = c1 + 1 + t; i < n; i += kTT) V[(size_t)c1 * n + i] = vn2[i];
            if (t == 0) {
                dg[(size_t)b * n + c1] = df_to(df_unpack(col2[c1]));
                eg[(size_t)b * n + c1] = sc[1];
                tau[(size_t)b * n + c1] = sc[0];
            }
        }
        // (c) columns c+2 .. n-1: update by (v_c, w_c); partial A v_{c+1} for the next step
        const bool sym = c1 <= n - 3;
        if (sym)
            for (int i = c1 + 1 + (t & 31); i < n; i += 32) pw_mine[i] = make_float2(0.f, 0.f);
        __syncthreads();
        fused_pass(n, c1 + 1, A, vk2, wk2, vn2, pw_mine, true, sym, false, gwarp, nwarps);
        __syncthreads();
        if (sym) reduce_warp_rows(n, c1 + 1, pw, buf + (size_t)(c1 & 1) * n);
        cluster.sync();
    }
    if (rank == 0 && t == 0) {
        dg[(size_t)b * n + n - 1] = df_to(df_unpack(A2[(size_t)(n - 1) * n + n - 1]));
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

// Twisted factorisation of T - s I (scaled T).  The stationary top-down pivots G_i (with the
// multipliers L_i = e_i / G_i) and the bottom-up pivots H_i (U_i = e_{i-1} / H_i) meet at the
// twist index r where |gamma_r| = |G_r + H_r - (d_r - s)| is least; the vector with z_r = 1
// has z_i = -L_i z_{i+1} above r and z_i = -U_i z_{i-1} below it.  Its squared norm at every
// twist follows from two recurrences, S_{i+1} = L_i^2 (1 + S_i) from the top and
// B_{i-1} = U_i^2 (1 + B_i) from the bottom, so |z|^2 = S_r + 1 + B_r without forming z.
// rq_step: one pass each way; returns the Rayleigh-quotient correction gamma_r / |z|^2.  The
// top-down pass keeps G and S in the scratch columns (they are read back, in an order that
// does not depend on the recurrence, by the bottom-up pass).
__device__ double rq_step(int n, const double* d, const double* e, double s, double pivmin, size_t K,
                          double* __restrict__ Gc, double* __restrict__ Sc, int* r_out) {
    double g = d[0] - s, sn = 0.0;
    if (fabs(g) < pivmin) g = -pivmin;
    for (int i = 0; i + 1 < n; i++) {
        Gc[i * K] = g;
        Sc[i * K] = sn;
        const double l = e[i] / g;
        sn = l * l * (1.0 + sn);
        g = d[i + 1] - s - l * e[i];
        if (fabs(g) < pivmin) g = -pivmin;
    }
    // twist at n-1: gamma = G_{n-1}, |z|^2 = S_{n-1} + 1
    int r = n - 1;
    double gam_r = g, best = fabs(g), nz = sn + 1.0;
    double h = d[n - 1] - s, bn = 0.0;
    if (fabs(h) < pivmin) h = -pivmin;
    double gnext = Gc[(size_t)(n - 2) * K], snext = Sc[(size_t)(n - 2) * K];
    for (int i = n - 1; i >= 1; i--) {
        const double gi = gnext, si = snext;  // G_{i-1}, S_{i-1}
        if (i >= 2) {
            gnext = Gc[(size_t)(i - 2) * K];
            snext = Sc[(size_t)(i - 2) * K];
        }
        const double u = e[i - 1] / h;
        bn = u * u * (1.0 + bn);
        h = d[i - 1] - s - u * e[i - 1];
        if (fabs(h) < pivmin) h = -pivmin;
        const double gam = gi + h - (d[i - 1] - s);
        if (fabs(gam) < best) {
            best = fabs(gam);
            gam_r = gam;
            r = i - 1;
            nz = si + 1.0 + bn;
        }
    }
    *r_out = r;
    return gam_r / nz;
}

// The eigenvector at s with twist r into column Zc (stride K), unnormalised, |z|^2 in *nrm_out;
// Lc, Uc scratch columns.
__device__ void twisted_vector(int n, const double* d, const double* e, double s, double pivmin, int r, size_t K,
                               double* __restrict__ Lc, double* __restrict__ Uc, double* __restrict__ Zc,
                               double* nrm_out) {
    double g = d[0] - s;
    if (fabs(g) < pivmin) g = -pivmin;
    for (int i = 0; i < r; i++) {
        const double l = e[i] / g;
        Lc[i * K] = l;
        g = d[i + 1] - s - l * e[i];
        if (fabs(g) < pivmin) g = -pivmin;
    }
    double h = d[n - 1] - s;
    if (fabs(h) < pivmin) h = -pivmin;
    for (int i = n - 1; i > r; i--) {
        const double u = e[i - 1] / h;
        Uc[i * K] = u;
        h = d[i - 1] - s - u * e[i - 1];
        if (fabs(h) < pivmin) h = -pivmin;
    }
    double nrm = 1.0, z = 1.0;
    Zc[(size_t)r * K] = 1.0;
    for (int i = r - 1; i >= 0; i--) {
        z = -Lc[i * K] * z;
        Zc[i * K] = z;
        nrm += z * z;
    }
    z = 1.0;
    for (int i = r + 1; i < n; i++) {
        z = -Uc[i * K] * z;
        Zc[i * K] = z;
        nrm += z * z;
    }
    *nrm_out = nrm;
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
    double del = 8.0 * FLT_EPSILON, lo = x - del, hi = x + del;
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
    double* Gc = a.G + col;
    double* Sc = a.L + col;
    double lam = x, vs = x;  // the eigenvalue, and the shift whose twist r gives the vector
    int r = n - 1;
    bool done = false;
    // a bracket holding several eigenvalues is bisected until it holds this one alone
    for (int it = 0; it < 60 && chi - clo > 1 && hi - lo > 4.0 * DBL_EPSILON; it++) {
        const double mid = 0.5 * (lo + hi);
        const int cm = sturm64(n, d, e2, mid, pivmin);
        if (cm > j) {
            hi = mid;
            chi = cm;
        } else {
            lo = mid;
            clo = cm;
        }
    }
    if (chi - clo == 1) {
        // converged when the correction is below 1e-14 of the block scale (T is scaled to norm
        // < 1), or when it stops shrinking at a level below 1e-10 (the rounding floor of gamma)
        double s = fmin(fmax(x, lo), hi), prev = 1.0;
        for (int it = 0; it < 8; it++) {
            const double dl = rq_step(n, d, e, s, pivmin, K, Gc, Sc, &r);
            const double s1 = s + dl;
            if (!(s1 > lo && s1 < hi)) break;  // left the bracket: bisect instead
            if (fabs(dl) <= 1e-14 || (fabs(dl) <= 1e-10 && fabs(dl) > 0.25 * prev)) {
                lam = s1;
                vs = s;  // the twist r belongs to s
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
        lam = vs = 0.5 * (lo + hi);
        rq_step(n, d, e, vs, pivmin, K, Gc, Sc, &r);
    }
    double nrm2 = 1.0;
    twisted_vector(n, d, e, vs, pivmin, r, K, a.L + col, a.U + col, a.Z + col, &nrm2);
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
// threads), in double-FP32.  The G vectors live in shared memory ([row][G] (hi, lo) pairs),
// each reflector row is staged once per CTA, thread t works on vector t % G over the rows
// t / G + R k, and the G dot products are summed over the R = 256 / G row groups in a fixed
// order.  Writes column n-1-c of the block in FP64 (ascending order, column-major).
constexpr int kBT = 256;
template <int G>
__global__ void __launch_bounds__(kBT) backtransform_kernel(VecArgs a, const double* __restrict__ Vall,
                                                            const double* __restrict__ tau, double* __restrict__ out) {
    extern __shared__ double bsm[];
    constexpr int R = kBT / G;  // row groups
    const int b = blockIdx.x, n = a.n, kc = a.kc[b];
    const int c0 = blockIdx.y * G;
    if (c0 >= kc) return;
    float2* z = reinterpret_cast<float2*>(bsm);  // [n][G]
    float2* v = z + (size_t)n * G;                // [n] reflector row
    float2* part = v + n;                         // [R][G]
    float2* f = part + R * G;                     // [G]
    float2* tau2 = f + G;                         // [n] tau as (hi, lo) pairs
    const int t = threadIdx.x, g = t % G, rg = t / G;
    const size_t K = (size_t)a.ktot;
    const int ng = min(G, kc - c0);
    for (int idx = t; idx < n * G; idx += kBT) {
        const int i = idx / G, gg = idx % G;
        z[idx] = df_pack(df_from(gg < ng ? a.Z[(size_t)i * K + a.koff[b] + c0 + gg] : 0.0));
    }
    const float2* V = reinterpret_cast<const float2*>(Vall) + (size_t)b * n * n;
    const double* tb = tau + (size_t)b * n;
    for (int i = t; i < n; i += kBT) tau2[i] = df_pack(df_from(tb[i]));
    __syncthreads();
    for (int c2 = n - 3; c2 >= 0; c2--) {
        const float2 tc2 = tau2[c2];
        if (tc2.x == 0.f) continue;  // uniform over the CTA
        __syncthreads();          // the previous update is done with v and f
        for (int i = c2 + 1 + t; i < n; i += kBT) v[i] = V[(size_t)c2 * n + i];
        __syncthreads();
        df s0{0.f, 0.f}, s1{0.f, 0.f};
        int i = c2 + 1 + rg;
        for (; i + R < n; i += 2 * R) {
            s0 = df_fma(s0, df_unpack(v[i]), df_unpack(z[(size_t)i * G + g]));
            s1 = df_fma(s1, df_unpack(v[i + R]), df_unpack(z[(size_t)(i + R) * G + g]));
        }
        if (i < n) s0 = df_fma(s0, df_unpack(v[i]), df_unpack(z[(size_t)i * G + g]));
        part[rg * G + g] = df_pack(df_add(s0, s1));
        __syncthreads();
        if (t < G) {
            df s = df_unpack(part[t]);
            for (int r = 1; r < R; r++) s = df_add(s, df_unpack(part[r * G + t]));
            f[t] = df_pack(df_mul(df_unpack(tc2), s));
        }
        __syncthreads();
        const df fg = df_unpack(f[g]);
        for (i = c2 + 1 + rg; i < n; i += R)
            z[(size_t)i * G + g] = df_pack(df_fms(df_unpack(z[(size_t)i * G + g]), fg, df_unpack(v[i])));
    }
    __syncthreads();
    for (int gg = 0; gg < ng; gg++) {
        double* o = out + (size_t)b * n * n + (size_t)(n - 1 - (c0 + gg)) * n;
        for (int i2 = t; i2 < n; i2 += kBT) o[i2] = df_to(df_unpack(z[(size_t)i2 * G + gg]));
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
    if (p.n <= 256) {  // 16 vectors per CTA above: twice the CTAs, two per SM
        constexpr int G = 32;
        const size_t smem = sizeof(double) * ((size_t)p.n * G + 2 * p.n + kBT + G);
        OPSEC_CUDA(cudaFuncSetAttribute(backtransform_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        max_dynamic_smem((const void*)backtransform_kernel<G>)));
        backtransform_kernel<G><<<dim3(p.nblk, (p.n + G - 1) / G), kBT, smem, s>>>(a, p.V, p.tau, p.out);
    } else {
        constexpr int G = 16;
        const size_t smem = sizeof(double) * ((size_t)p.n * G + 2 * p.n + kBT + G);
        OPSEC_CUDA(cudaFuncSetAttribute(backtransform_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        max_dynamic_smem((const void*)backtransform_kernel<G>)));
        backtransform_kernel<G><<<dim3(p.nblk, (p.n + G - 1) / G), kBT, smem, s>>>(a, p.V, p.tau, p.out);
    }
    if (g_clock) g_clock->end(s);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 3;
}

}  // namespace opsec
