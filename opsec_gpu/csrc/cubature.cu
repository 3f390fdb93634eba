// cubature.cu -- cell-pair integrals Q_t(key) for every xi table at once.
//
// Q_ab = int_{[0,1]^6} xi(|x(u1..3) - y(u4..6)|) d^6u over the two cells of a
// symmetry key (sig.cpp:381-482), by the ng^3 x ng^3 Gauss-Legendre product
// rule.  Cartesian cells map affinely; spherical cells map r through r^3 so
// that the map is volume-uniform (sig.cpp:453-458).
//
// Layout and precision:
//  * a point table holds every Gauss point of every grid cell once, as an
//    FP32 pair (hi, lo) with hi + lo = the FP64 position to ~1e-14, and its
//    FP32 weight: [cell][point][hi, lo] float4s, built by one kernel per
//    build, so the per-key setup is FP32 arithmetic (FP64 runs at 1/64 of
//    the FP32 rate on this part);
//  * one warp integrates one key; a CTA holds G xi tables in shared memory
//    (FP32) and loops its warps over keys.  The second cell's points are
//    shifted to the first cell's middle point (pair-relative coordinates) and
//    staged in the warp's slice of shared memory; each lane keeps its own
//    first-cell point in registers;
//  * exact mode (the default): the separation of a point pair is formed as
//    an FP32 pair by Knuth's two-sum, r^2 as an FP32 pair by FMA two-product
//    and two-sum, and the table index from log2(r^2) = E + log2(T_k) +
//    log2(1 + delta), with E the binary exponent of r^2, T_k = 1 + k/128 from
//    its top 7 mantissa bits and delta < 1/128 from the FP32 pair; in the
//    linear section t = r n1/r1 takes r and n1/r1 as FP32 pairs and the
//    fraction from the FMA residual of the rounded product.  The fraction of
//    the index is then good to ~3e-7 of a grid step at every r, and the error
//    left is that of the FP32 tables (~1e-7 of max|Q| per band);
//  * fast mode: one FP32 separation, sqrt and hardware log2 of the mantissa;
//    the fraction of the index then carries the ~6e-8 relative rounding of r,
//    i.e. a phase error k r 6e-8 in an oscillating band table;
//  * FP32 sums over the ng^3 points of the second cell; FP64 for the outer
//    sum and the warp reduction.
// Periodic boxes wrap each pair difference into [-L/2, L/2) (BoxSurvey.cpp:26-30).
#include <climits>
#include <cmath>
#include <algorithm>
#include <cstring>
#include <string>

#include "engine.h"

namespace opsec {
namespace {

// Table index of a distance r.  Linear section: t = r n1 / r1.  Log section:
// t = n1 + (log2 r - log2 r1) (n2-1) / log2(r2/r1).  log2 is split into the
// binary exponent e of the argument and the log2 of its mantissa, and the
// offset of each exponent, c_e, is precomputed in FP64 as an integer part
// plus an FP32 fraction.  Fast mode takes the exponent of r, exact mode the
// exponent of r^2 (c_e = n1 + (e/2 - log2 r1) (n2-1)/log2(r2/r1)).
constexpr int kMaxExp = 64;
constexpr int kLogBits = 7;
constexpr int kLogN = 1 << kLogBits;
struct Lookup {
    float inv_dr;   // n1 / r1: index in the linear section
    float inv_dr_lo;  // n1 / r1 - inv_dr
    float r1, r1sq;
    float inv_du;   // (n2-1) / log2(r2/r1)
    float cp;       // exact mode: (n2-1) / log2(r2/r1) / (2 ln 2), index per unit of ln(1 + delta)
    int n1;
    int imax;       // n - 2
    int e0;         // smallest exponent held in the offset table
    int ne;         // entries in the offset table
    int ci[kMaxExp];    // integer part of c_e
    float cf[kMaxExp];  // fraction of c_e
    // exact mode, per k < 128: (1/T_k, fraction of z_k, integer part of z_k, 0),
    // z_k = log2(T_k) (n2-1) / log2(r2/r1) / 2
    float4 kt[kLogN];
};

// Smallest separation whose table index is b (the QSpline grid: linear below r1, log above).
__device__ __forceinline__ float bin_edge(const Lookup& lk, int b) {
    return b <= lk.n1 ? (float)b / lk.inv_dr : lk.r1 * exp2f((float)(b - lk.n1) / lk.inv_du);
}

template <int NG>
struct Shape {
    static constexpr int NP = NG * NG * NG;
    // 16 warps per CTA (twice the latency hiding) while the point buffers leave room for tables
    static constexpr int kWarps = NG <= 4 ? 16 : 8;
};

// Row ha of entry tri of the packed upper triangle of an H x H matrix (row ha starts at
// ha H - ha (ha - 1) / 2): the FP32 root of the quadratic (FP64 issues at 1/64 of the FP32
// rate on this part), then exact integer corrections.
__device__ __forceinline__ int tri_row(int H, long long tri) {
    const float H2 = 2.f * (float)H + 1.f;
    int ha = (int)floorf((H2 - sqrtf(fmaxf(H2 * H2 - 8.f * (float)tri, 0.f))) * 0.5f);
    ha = min(max(ha, 0), H - 1);
    while (ha > 0 && (long long)ha * H - (long long)ha * (ha - 1) / 2 > tri) --ha;
    while ((long long)(ha + 1) * H - (long long)(ha + 1) * ha / 2 <= tri) ++ha;
    return ha;
}

__device__ __forceinline__ void decode_key(const KeySpace& ks, long long key, int* c1, int* c2) {
    if (ks.coordsys == 1) {
        int kz = (int)(key % ks.N3);
        long long t = key / ks.N3;
        int ky = (int)(t % ks.N2);
        int kx = (int)(t / ks.N2);
        c1[0] = 0; c1[1] = 0; c1[2] = 0;
        c2[0] = kx; c2[1] = ky; c2[2] = kz;
        return;
    }
    const int df = (int)(key % ks.nf);
    const long long tri = key / ks.nf;
    const int ha = tri_row(ks.H, tri);
    const int hb = ha + (int)(tri - ((long long)ha * ks.H - (long long)ha * (ha - 1) / 2));
    c1[0] = ha / ks.N2; c1[1] = ha % ks.N2; c1[2] = 0;
    c2[0] = hb / ks.N2; c2[1] = hb % ks.N2; c2[2] = df;
}

// Spherical grids whose mu range is symmetric about 0: the reflection
// z -> -z maps arc h = (i, j) to P h = (i, N_mu-1-j) and leaves phi alone, so
// Q(h_a, h_b, df) = Q(P h_a, P h_b, df).  Of the two keys of such an orbit the
// one with the smaller (h_a, h_b) triangle index is integrated; the other is
// copied after the cubature.  Returns the partner key (= key on self-orbits).
__device__ __forceinline__ long long reflect_partner(const KeySpace& ks, long long key) {
    const int df = (int)(key % ks.nf);
    const long long tri = key / ks.nf;
    const int ha = tri_row(ks.H, tri);
    const int hb = ha + (int)(tri - ((long long)ha * ks.H - (long long)ha * (ha - 1) / 2));
    const int pa = (ha / ks.N2) * ks.N2 + (ks.N2 - 1 - ha % ks.N2);
    const int pb = (hb / ks.N2) * ks.N2 + (ks.N2 - 1 - hb % ks.N2);
    const int p1 = min(pa, pb), p2 = max(pa, pb);
    const long long ptri = (long long)p1 * ks.H - (long long)p1 * (p1 - 1) / 2 + (p2 - p1);
    return ptri * ks.nf + df;
}

// Knuth's two-sum: s + e == a + b exactly.  The _rn intrinsics keep the
// compiler from contracting a product that feeds these sums into an FMA.
__device__ __forceinline__ float two_sum(float a, float b, float* e) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    *e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

// (hi, lo) of b - a for FP32 pairs
__device__ __forceinline__ float diff2(float bh, float bl, float ah, float al, float* lo) {
    float e;
    const float s = two_sum(bh, -ah, &e);
    *lo = e + (bl - al);
    return s;
}

__device__ __forceinline__ void index_r2(const Lookup& lk, const int* s_ci, const float* s_cf, const float4* s_kt,
                                         float r2, float r2l, int& i, float& fr);

// Table index (i, fr) of one point pair in exact mode: separation and r^2
// as FP32 pairs, log2(r^2) split as E + log2(T_k) + log2(1 + delta).
__device__ __forceinline__ void exact_index(const Lookup& lk, const int* s_ci, const float* s_cf, const float4* s_kt,
                                            float4 B, float4 Bl, float ax, float alx, float ay, float aly, float az,
                                            float alz, bool periodic, float Lh, float Ll, float hL, int& i,
                                            float& fr) {
    float lx, ly, lz;
    float dx = diff2(B.x, Bl.x, ax, alx, &lx);
    float dy = diff2(B.y, Bl.y, ay, aly, &ly);
    float dz = diff2(B.z, Bl.z, az, alz, &lz);
    if (periodic) {
        // |d| in [L/2, L]: d -+ L is exact in FP32 (Sterbenz)
        const float wx = (float)((dx < -hL) - (dx >= hL));
        const float wy = (float)((dy < -hL) - (dy >= hL));
        const float wz = (float)((dz < -hL) - (dz >= hL));
        dx = fmaf(wx, Lh, dx); lx = fmaf(wx, Ll, lx);
        dy = fmaf(wy, Lh, dy); ly = fmaf(wy, Ll, ly);
        dz = fmaf(wz, Lh, dz); lz = fmaf(wz, Ll, lz);
    }
    // r^2 = hi + lo: exact squares by FMA, exact sums by two-sum
    const float px = __fmul_rn(dx, dx), py = __fmul_rn(dy, dy), pz = __fmul_rn(dz, dz);
    float e1, e2;
    const float h1 = two_sum(px, py, &e1);
    const float r2 = two_sum(h1, pz, &e2);
    float r2l = fmaf(dx, dx, -px) + fmaf(dy, dy, -py) + fmaf(dz, dz, -pz) + (e1 + e2);
    r2l = fmaf(2.f * dx, lx, fmaf(2.f * dy, ly, fmaf(2.f * dz, lz, r2l)));
    index_r2(lk, s_ci, s_cf, s_kt, r2, r2l, i, fr);
}

// Table index (i, fr) of a separation given as r^2 = r2 + r2l (an FP32 pair).
__device__ __forceinline__ void index_r2(const Lookup& lk, const int* s_ci, const float* s_cf, const float4* s_kt,
                                         float r2, float r2l, int& i, float& fr) {
    if (r2 < lk.r1sq) {
        // t = r n1 / r1 with r = rh + rl and n1 / r1 = inv_dr + inv_dr_lo; the
        // fraction is formed from the exact residual of the rounded product
        const float rh = sqrtf(r2);
        const float rl = rh > 0.f ? __fdividef(fmaf(-rh, rh, r2) + r2l, 2.f * rh) : 0.f;
        const float t = rh * lk.inv_dr;
        i = (int)t;
        fr = fmaf(rh, lk.inv_dr, -(float)i) + fmaf(rh, lk.inv_dr_lo, rl * lk.inv_dr);
    } else {
        const int bits = __float_as_int(r2);
        const int eb = bits >> 23;  // biased exponent; r2 > 0 here
        const int e = min(max(eb - 127 - lk.e0, 0), lk.ne - 1);
        const int k = (bits >> (23 - kLogBits)) & (kLogN - 1);
        const float Rk = __int_as_float(bits & ~((1 << (23 - kLogBits)) - 1));
        const float4 kt = s_kt[k];
        const float inv_pow = __int_as_float((254 - eb) << 23);  // 2^-(eb-127)
        const float delta = ((r2 - Rk) + r2l) * (kt.x * inv_pow);
        // ln(1 + delta), |delta| < 1/128: the series to delta^4 is good to 3e-12
        const float ln1p = delta * fmaf(-delta, fmaf(-delta, fmaf(-delta, 0.25f, 1.f / 3.f), 0.5f), 1.f);
        const float y = fmaf(ln1p, lk.cp, s_cf[e] + kt.y);
        const float yi = floorf(y);
        i = s_ci[e] + __float_as_int(kt.z) + (int)yi;
        fr = y - yi;
        if (i < lk.n1) {
            i = lk.n1;
            fr = 0.f;
        }
    }
    if (i > lk.imax) {
        i = lk.imax;
        fr = 1.0f;
    }
}

// Gauss points of every cell: [cell][p] -> hi (x, y, z, w), lo (x, y, z, 0).
__global__ void point_table_kernel(CubatureArgs a, int ng, long long ncell) {
    const int np = ng * ng * ng;
    const long long n = ncell * np;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long cell = t / np;
        const int p = (int)(t % np);
        const int c2 = (int)(cell % a.ks.N3);
        const int c1 = (int)((cell / a.ks.N3) % a.ks.N2);
        const int c0 = (int)(cell / ((long long)a.ks.N3 * a.ks.N2));
        const int i = p / (ng * ng), j = (p / ng) % ng, l = p % ng;
        const double w = a.w[i] * a.w[j] * a.w[l];
        double x[3];
        if (a.coordsys == 1) {
            x[0] = a.node1[c0 * ng + i];
            x[1] = a.node2[c1 * ng + j];
            x[2] = a.node3[c2 * ng + l];
        } else {
            const double r = a.node1[c0 * ng + i];
            const double mu = a.node2[c1 * ng + j];
            const double rs = r * a.snode2[c1 * ng + j];
            x[0] = rs * a.cphi[c2 * ng + l];
            x[1] = rs * a.sphi[c2 * ng + l];
            x[2] = r * mu;
        }
        float h[3], lo[3];
        for (int d = 0; d < 3; d++) {
            h[d] = (float)x[d];
            lo[d] = (float)(x[d] - (double)h[d]);
        }
        a.pts[2 * t] = make_float4(h[0], h[1], h[2], (float)w);
        a.pts[2 * t + 1] = make_float4(lo[0], lo[1], lo[2], 0.f);
    }
}

// Q of the keys skipped by the reflection symmetry, from their partners.
__global__ void reflect_fill_kernel(KeySpace ks, int ntab, double* Q) {
    for (long long key = blockIdx.x * (long long)blockDim.x + threadIdx.x; key < ks.nkeys;
         key += (long long)gridDim.x * blockDim.x) {
        const long long p = reflect_partner(ks, key);
        if (p < key)
            for (int t = 0; t < ntab; t++) Q[(size_t)t * ks.nkeys + key] = Q[(size_t)t * ks.nkeys + p];
    }
}

__device__ __forceinline__ long long cell_id(const KeySpace& ks, const int* c) {
    return ((long long)c[0] * ks.N2 + c[1]) * ks.N3 + c[2];
}

template <int NG, int G, bool EXACT>
__global__ void __launch_bounds__(Shape<NG>::kWarps * 32, 1)
    cubature_kernel(CubatureArgs a, int tab0, int ngrp, Lookup lk) {
    constexpr int NP = Shape<NG>::NP;
    constexpr int kWarps = Shape<NG>::kWarps;
    constexpr int NB = EXACT ? 2 : 1;  // staged float4s per second-cell point
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nx = a.xl.n();
    float4* pts = reinterpret_cast<float4*>(smem_raw);           // [kWarps][NB][NP]
    float* tab = reinterpret_cast<float*>(pts + kWarps * NB * NP);  // [ngrp][nx]

    for (int i = threadIdx.x; i < ngrp * nx; i += blockDim.x) tab[i] = a.tab32[(size_t)tab0 * nx + i];
    __shared__ int s_ci[kMaxExp];
    __shared__ float s_cf[kMaxExp];
    __shared__ float4 s_kt[EXACT ? kLogN : 1];
    for (int i = threadIdx.x; i < lk.ne; i += blockDim.x) {
        s_ci[i] = lk.ci[i];
        s_cf[i] = lk.cf[i];
    }
    if (EXACT)
        for (int i = threadIdx.x; i < kLogN; i += blockDim.x) s_kt[i] = lk.kt[i];
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* P2 = pts + warp * NB * NP;   // hi (x, y, z, w)
    float4* P2l = P2 + (NB - 1) * NP;    // lo (x, y, z, 0), exact mode
    const bool periodic = (a.coordsys == 1 && a.L > 0);
    const float Lh = (float)a.L, Ll = (float)(a.L - (double)Lh), hL = 0.5f * Lh;

    const long long nwork = a.list ? (long long)*a.list_count : a.ks.nkeys;
    for (long long j = (long long)blockIdx.x * kWarps + warp; j < nwork; j += (long long)gridDim.x * kWarps) {
        const long long key = a.list ? (long long)a.list[j] : j;
        if (!a.list && a.ks.coordsys == 2 && a.ks.mu_reflect && reflect_partner(a.ks, key) < key) continue;
        if (!a.list && a.skip && a.skip[key]) continue;
        int c1[3], c2[3];
        decode_key(a.ks, key, c1, c2);
        const float4* G1 = a.pts + 2 * NP * cell_id(a.ks, c1);
        const float4* G2 = a.pts + 2 * NP * cell_id(a.ks, c2);
        const float4 Oh = G1[2 * (NP / 2)], Ol = G1[2 * (NP / 2) + 1];  // origin: middle point of cell 1
        for (int q = lane; q < NP; q += 32) {
            const float4 Bh = G2[2 * q], Bl = G2[2 * q + 1];
            float lx, ly, lz;
            const float sx = diff2(Bh.x, Bl.x, Oh.x, Ol.x, &lx);
            const float sy = diff2(Bh.y, Bl.y, Oh.y, Ol.y, &ly);
            const float sz = diff2(Bh.z, Bl.z, Oh.z, Ol.z, &lz);
            if (EXACT) {
                P2[q] = make_float4(sx, sy, sz, Bh.w);
                P2l[q] = make_float4(lx, ly, lz, 0.f);
            } else {
                P2[q] = make_float4(sx + lx, sy + ly, sz + lz, Bh.w);
            }
        }
        __syncwarp();

        double tot[G];
#pragma unroll
        for (int t = 0; t < G; t++) tot[t] = 0.0;
        for (int p = lane; p < NP; p += 32) {
            const float4 Ah = G1[2 * p], Al = G1[2 * p + 1];
            float alx, aly, alz;
            const float ax = diff2(Ah.x, Al.x, Oh.x, Ol.x, &alx);
            const float ay = diff2(Ah.y, Al.y, Oh.y, Ol.y, &aly);
            const float az = diff2(Ah.z, Al.z, Oh.z, Ol.z, &alz);
            float acc[G];
#pragma unroll
            for (int t = 0; t < G; t++) acc[t] = 0.f;
#pragma unroll 4
            for (int q = 0; q < NP; q++) {
                const float4 B = P2[q];
                int i;
                float fr;
                if (EXACT) {
                    exact_index(lk, s_ci, s_cf, s_kt, B, P2l[q], ax, alx, ay, aly, az, alz, periodic, Lh, Ll, hL, i,
                                fr);
                } else {
                    float dx = B.x - ax, dy = B.y - ay, dz = B.z - az;
                    if (periodic) {
                        dx += Lh * (float)((dx < -hL) - (dx >= hL));
                        dy += Lh * (float)((dy < -hL) - (dy >= hL));
                        dz += Lh * (float)((dz < -hL) - (dz >= hL));
                    }
                    const float r = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
                    if (r < lk.r1) {
                        const float t = r * lk.inv_dr;
                        i = (int)t;
                        fr = t - (float)i;
                    } else {
                        const int bits = __float_as_int(r);
                        const int e = min(max((bits >> 23) - 127 - lk.e0, 0), lk.ne - 1);
                        const float lm = __log2f(__int_as_float((bits & 0x007FFFFF) | 0x3F800000));  // log2 of mantissa
                        const float y = fmaf(lm, lk.inv_du, s_cf[e]);
                        const float yi = floorf(y);
                        i = s_ci[e] + (int)yi;
                        fr = y - yi;
                        if (i < lk.n1) {
                            i = lk.n1;
                            fr = 0.f;
                        }
                    }
                }
                if (i > lk.imax) {
                    i = lk.imax;
                    fr = 1.0f;
                }
#pragma unroll
                for (int t = 0; t < G; t++) {
                    if (t < ngrp) {
                        const float y0 = tab[t * nx + i];
                        const float y1 = tab[t * nx + i + 1];
                        acc[t] = fmaf(B.w, fmaf(fr, y1 - y0, y0), acc[t]);
                    }
                }
            }
#pragma unroll
            for (int t = 0; t < G; t++) tot[t] += (double)Ah.w * (double)acc[t];
        }
#pragma unroll
        for (int t = 0; t < G; t++) {
            double v = tot[t];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0 && t < ngrp) a.Q[(size_t)(tab0 + t) * a.ks.nkeys + key] = v;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- window path (exact mode)
// Q_t(key) = sum_pairs w_p w_q [(1-fr) T_t[i] + fr T_t[i+1]] = sum_bins T_t[bin] h_key[bin]:
// one pass over the point pairs of a key scatters the interpolation weights
// into a histogram h over the key's window of table bins, then one dot product
// per table.  The pair geometry is computed once for all tables.  A key's
// window follows from the bounding spheres of its two cells; keys are
// bucketed by window start so a CTA's batch of keys shares one shared-memory
// tile of every table.  Keys with windows wider than a tile allows (near and
// self pairs) go to the table-group kernel in list mode.
struct WinPlan {
    int Wkey;     // histogram bins per warp: one pass covers Wkey - 1 bins of a key's window
    int Wmax;     // widest key window on the window path (npass_max passes)
    int flush;    // Cartesian window kernel: second-cell points per loop chunk (0: all)
    int dot64;    // compensated dot products for every key (1) or only where windows cancel strongly (0)
    float qinv;   // coarse fixed-point units per unit of pair weight (2^k / largest pair weight)
    float qfrac;  // fraction units per coarse unit (2^fbits)
    int fbits;
    float qfine;  // pair weight per unit of the 64-bit histogram (2^-fbits / qinv)
    int nbucket;  // nx + 1: bucket nx holds the near keys
    int2* win;        // [nkeys]: (bucket, width); bucket -1 = key copied by the reflection fill
    int* order;       // [2 nkeys]: far keys, then near keys (incl. windows too wide for the far kernels)
    int* count;       // [nbucket + 1]
    int* cursor;      // [nbucket + 1]
    int keyorder;     // far and near keys each in ascending key order (1) or by window start (0)
    int4* tiles;      // key order: per tile of kPartTile keys, the counts of the three classes, then
                      // the tile's first slot in order[] for each
    int* nfar;        // far keys
    int* nnear;       // near keys incl. overflows (list length from order + nfar)
    int* violations;  // pairs that fell outside their key's window (must stay 0)
    float4* cen;      // per cell: bounding-sphere centre and radius
    float* tabT;      // [nx][ntab]: the FP32 tables transposed, bin-major
    // spherical grids (see cubature_far_sph_kernel)
    float4* arc;      // [H][ng^2]: rho hi, rho lo, z hi, z lo of node pair P = i_r ng + i_mu
    float* wrm;       // [ng^2]: w_r w_mu of node pair P
    float4* sph;      // [nf][ng(ng+1)/2]: sin^2(theta/2) hi, lo, phi-node weight (x2 off the diagonal), 0
    int logkeys;      // one-pass keys in the log section take the specialised loop
    float4* arcbox;   // [H]: rho min, rho max, z min, z max over the arc's node pairs (rounded outward)
    float2* sphbox;   // [nf]: min and max of sin^2(theta/2) over the canonical phi-node pairs (outward)
};

// Tables of the spherical window kernel, from the cubature nodes (FP64 products,
// split into FP32 pairs).  Canonical phi-node pairs (l_p, l_q), l_p + l_q <= ng-1,
// in the order l_p, then l_q.
__global__ void sph_tables_kernel(CubatureArgs a, WinPlan w) {
    const int ng = a.ng, ng2 = ng * ng, nc = ng * (ng + 1) / 2;
    const long long narc = (long long)a.ks.H * ng2;
    const long long nsph = (long long)a.ks.nf * nc;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < narc + ng2 + nsph;
         e += (long long)gridDim.x * blockDim.x) {
        if (e < narc) {
            const int h = (int)(e / ng2), P = (int)(e % ng2);
            const int d1 = h / a.ks.N2, d2 = h % a.ks.N2, ir = P / ng, im = P % ng;
            const double r = a.node1[d1 * ng + ir];
            const double rho = r * a.snode2[d2 * ng + im], z = r * a.node2[d2 * ng + im];
            const float rh = (float)rho, zh = (float)z;
            w.arc[e] = make_float4(rh, (float)(rho - (double)rh), zh, (float)(z - (double)zh));
        } else if (e < narc + ng2) {
            const int P = (int)(e - narc);
            w.wrm[P] = (float)(a.w[P / ng] * a.w[P % ng]);
        } else {
            const long long t = e - narc - ng2;
            const int df = (int)(t / nc);
            int c = (int)(t % nc), lp = 0;
            while (c >= ng - lp) {
                c -= ng - lp;
                ++lp;
            }
            const int lq = c;
            // chord of the two phi nodes' unit vectors: |e_q - e_p| = 2 sin(theta / 2)
            const double dc = a.cphi[df * ng + lq] - a.cphi[lp], ds = a.sphi[df * ng + lq] - a.sphi[lp];
            const double s2 = 0.25 * (dc * dc + ds * ds);
            const float sh = (float)s2;
            const double wphi = a.w[lp] * a.w[lq] * (lp + lq < ng - 1 ? 2.0 : 1.0);
            w.sph[t] = make_float4(sh, (float)(s2 - (double)sh), (float)wphi, 0.f);
        }
    }
}

// Ranges of the spherical kernel's pair terms: per arc, the (rho, z) box of its node pairs;
// per azimuthal offset, the range of sin^2(theta/2) over its canonical phi-node pairs (FP64
// from the FP32 pairs).  key_window_kernel bounds r^2 = (rho_P - rho_Q)^2 + (z_P - z_Q)^2 +
// 4 rho_P rho_Q sin^2(theta/2) of a key's pairs by them.
__global__ void sph_box_kernel(CubatureArgs a, WinPlan w) {
    const int ng2 = a.ng * a.ng, nc = a.ng * (a.ng + 1) / 2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)a.ks.H + a.ks.nf;
         e += (long long)gridDim.x * blockDim.x) {
        if (e < a.ks.H) {
            double b[4] = {INFINITY, -INFINITY, INFINITY, -INFINITY};
            for (int P = 0; P < ng2; P++) {
                const float4 v = w.arc[e * ng2 + P];
                const double rho = (double)v.x + v.y, z = (double)v.z + v.w;
                b[0] = fmin(b[0], rho);
                b[1] = fmax(b[1], rho);
                b[2] = fmin(b[2], z);
                b[3] = fmax(b[3], z);
            }
            w.arcbox[e] = make_float4(__double2float_rd(b[0]), __double2float_ru(b[1]), __double2float_rd(b[2]),
                                      __double2float_ru(b[3]));
        } else {
            const long long df = e - a.ks.H;
            double lo = INFINITY, hi = -INFINITY;
            for (int c = 0; c < nc; c++) {
                const float4 v = w.sph[df * nc + c];
                const double s2 = (double)v.x + v.y;
                lo = fmin(lo, s2);
                hi = fmax(hi, s2);
            }
            w.sphbox[df] = make_float2(__double2float_rd(lo), __double2float_ru(hi));
        }
    }
}

// The tables bin-major, so that the lanes of a warp (one table each) read one
// bin of every table with one coalesced load.
__global__ void transpose_tables_kernel(const float* tab32, int ntab, int nx, float* tabT) {
    const long long n = (long long)ntab * nx;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(e / ntab), t = (int)(e % ntab);
        tabT[e] = tab32[(size_t)t * nx + b];
    }
}

// bounding sphere of each cell from its Gauss points (FP64), radius inflated by a margin
__global__ void cell_sphere_kernel(const float4* pts, int np, long long ncell, float4* cen) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
         c += (long long)gridDim.x * blockDim.x) {
        const float4* P = pts + 2 * np * c;
        double m[3] = {0, 0, 0};
        for (int p = 0; p < np; p++) {
            m[0] += (double)P[2 * p].x + P[2 * p + 1].x;
            m[1] += (double)P[2 * p].y + P[2 * p + 1].y;
            m[2] += (double)P[2 * p].z + P[2 * p + 1].z;
        }
        for (int d = 0; d < 3; d++) m[d] /= np;
        double r = 0;
        for (int p = 0; p < np; p++) {
            const double dx = (double)P[2 * p].x + P[2 * p + 1].x - m[0];
            const double dy = (double)P[2 * p].y + P[2 * p + 1].y - m[1];
            const double dz = (double)P[2 * p].z + P[2 * p + 1].z - m[2];
            r = fmax(r, sqrt(dx * dx + dy * dy + dz * dz));
        }
        cen[c] = make_float4((float)m[0], (float)m[1], (float)m[2], (float)(r * (1.0 + 1e-5) + 1e-3));
    }
}

// table bin of a distance (the QSpline grid) in FP32: the index the pair kernels compute to
// ~1e-3 of a bin (the windows carry a bin of margin below and three above)
// (per_oct: bins per octave of r in the log section, (n2 - 1) / log2(r2 / r1))
__device__ __forceinline__ int bin_floor(const XiLayout& xl, float per_oct, float r) {
    const float r1 = (float)xl.r1;
    if (r < r1) return (int)floorf(r * ((float)xl.n1 / r1));
    if (r >= (float)xl.r2) return xl.n() - 1;
    return xl.n1 + (int)floorf(log2f(r / r1) * per_oct);
}

__global__ void key_window_kernel(CubatureArgs a, WinPlan w) {
    const bool periodic = (a.coordsys == 1 && a.L > 0);
    const int nx = a.xl.n();
    const float per_oct = (float)((a.xl.n2 - 1) / log2(a.xl.r2 / a.xl.r1));
    for (long long key = blockIdx.x * (long long)blockDim.x + threadIdx.x; key < a.ks.nkeys;
         key += (long long)gridDim.x * blockDim.x) {
        if ((a.ks.coordsys == 2 && a.ks.mu_reflect && reflect_partner(a.ks, key) < key) || (a.skip && a.skip[key])) {
            w.win[key] = make_int2(-1, 0);
            continue;
        }
        int c1[3], c2[3];
        decode_key(a.ks, key, c1, c2);
        // FP32 (FP64 issues at 1/64 of the FP32 rate here), every bound widened by 1e-5 of
        // itself: far beyond the FP32 rounding of these few operations
        const float4 A = w.cen[cell_id(a.ks, c1)], B = w.cen[cell_id(a.ks, c2)];
        float d[3] = {B.x - A.x, B.y - A.y, B.z - A.z};
        const float R = A.w + B.w;
        bool near = false;
        if (periodic) {
            const float L = (float)a.L;
            for (int k = 0; k < 3; k++) {
                d[k] -= L * floorf(d[k] / L + 0.5f);
                if (fabsf(d[k]) + R >= 0.5f * L * (1.f - 1e-5f)) near = true;  // pair differences may wrap differently
            }
        }
        const float dist = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        float rlo = fmaxf(dist - R, 0.f) * (1.f - 1e-5f), rhi = (dist + R) * (1.f + 1e-5f);
        if (w.arcbox) {
            // spherical grids: the bounding spheres of cells long in phi are loose; bound r^2
            // term by term from the arcs' (rho, z) boxes and the offset's sin^2 range, and keep
            // the tighter of the two bounds (both hold for every node pair of the key)
            const float4 ba = w.arcbox[c1[0] * a.ks.N2 + c1[1]];
            const float4 bb = w.arcbox[c2[0] * a.ks.N2 + c2[1]];
            const float2 s2 = w.sphbox[c2[2]];
            const float grho = fmaxf(0.f, fmaxf(bb.x - ba.y, ba.x - bb.y));
            const float gz = fmaxf(0.f, fmaxf(bb.z - ba.w, ba.z - bb.w));
            const float drho = fmaxf(bb.y - ba.x, ba.y - bb.x);
            const float dz = fmaxf(bb.w - ba.z, ba.w - bb.z);
            const float r2lo = grho * grho + gz * gz + 4.f * ba.x * bb.x * s2.x;
            const float r2hi = drho * drho + dz * dz + 4.f * ba.y * bb.y * s2.y;
            rlo = fmaxf(rlo, sqrtf(r2lo) * (1.f - 1e-5f));
            rhi = fminf(rhi, sqrtf(r2hi) * (1.f + 1e-5f));
        }
        const int blo = max(bin_floor(a.xl, per_oct, rlo) - 1, 0);
        const int bhi = min(bin_floor(a.xl, per_oct, rhi) + 3, nx);
        const int width = bhi - blo;
        const int bucket = (near || width > w.Wmax) ? nx : blo;
        w.win[key] = make_int2(bucket, width);
        if (!w.keyorder) atomicAdd(&w.count[bucket], 1);
    }
}

// exclusive scan of the bucket counts (one block)
__global__ void bucket_scan_kernel(WinPlan w) {
    __shared__ int part[1024];
    const int n = w.nbucket;
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per, b1 = min(n, b0 + per);
    int s = 0;
    for (int b = b0; b < b1; b++) s += w.count[b];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int t = 0; t < (int)blockDim.x; t++) {
            const int v = part[t];
            part[t] = run;
            run += v;
        }
    }
    __syncthreads();
    int run = part[threadIdx.x];
    for (int b = b0; b < b1; b++) {
        w.cursor[b] = run;
        run += w.count[b];
    }
    if (threadIdx.x == 0) {
        *w.nfar = 0;
        for (int b = 0; b < n - 1; b++) *w.nfar += w.count[b];
        *w.nnear = w.count[n - 1];
    }
}

__global__ void bucket_scatter_kernel(long long nkeys, WinPlan w) {
    for (long long key = blockIdx.x * (long long)blockDim.x + threadIdx.x; key < nkeys;
         key += (long long)gridDim.x * blockDim.x) {
        const int b = w.win[key].x;
        if (b < 0) continue;
        w.order[atomicAdd(&w.cursor[b], 1)] = (int)key;
    }
}

// Key order: a stable partition of the keys into three classes, each in ascending key order:
// far keys that the spherical kernel's log-section loop takes (one pass, window above the
// linear section), the other far keys, the near keys.  Consecutive warps of the far kernels
// then integrate consecutive keys (mostly the same arc pair at consecutive azimuthal
// offsets, or neighbouring Cartesian offsets), so the Q values they write for one table fall
// into the same 32-byte sectors, which L2 merges before they reach DRAM (in window-start order
// every Q value was an isolated 8-byte write to its own sector), and the warps of an SM run
// the same loop at the same time.  Three launches: per-tile class counts, a scan over the
// tiles, a scatter in key order.
constexpr int kPartTile = 1024;  // keys per tile
constexpr int kPartThreads = 256;

// 0: reflected or skipped key, 1: far, log-section loop, 2: other far, 3: near.  n1log: the
// window start above which one-pass keys take the log-section loop (INT_MAX: none).
__device__ __forceinline__ int part_class(const WinPlan& w, long long key, int n1log) {
    const int2 wn = w.win[key];
    if (wn.x < 0) return 0;
    if (wn.x == w.nbucket - 1) return 3;
    const int S = w.Wkey - 1;
    return (wn.y - 1 <= S && wn.x > n1log) ? 1 : 2;
}

__global__ void __launch_bounds__(kPartThreads) part_count_kernel(long long nkeys, WinPlan w, int n1log) {
    __shared__ int s_n[3][kPartThreads / 32];
    const long long k0 = (long long)blockIdx.x * kPartTile;
    int n[3] = {0, 0, 0};
    for (int t = threadIdx.x; t < kPartTile && k0 + t < nkeys; t += kPartThreads) {
        const int c = part_class(w, k0 + t, n1log);
        if (c > 0) ++n[c - 1];
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int c = 0; c < 3; c++) n[c] += __shfl_xor_sync(0xffffffffu, n[c], o);
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 3; c++) s_n[c][threadIdx.x >> 5] = n[c];
    __syncthreads();
    if (threadIdx.x == 0) {
        int4 v = make_int4(0, 0, 0, 0);
        for (int i = 0; i < kPartThreads / 32; i++) {
            v.x += s_n[0][i];
            v.y += s_n[1][i];
            v.z += s_n[2][i];
        }
        w.tiles[blockIdx.x] = v;
    }
}

// exclusive scan of the tile counts (one block) into the tiles' first slots in order[]: class 1
// from 0, class 2 after all of class 1, class 3 (near keys) after all far keys
__global__ void part_scan_kernel(int ntiles, WinPlan w) {
    __shared__ int4 part[1024];
    const int per = (ntiles + blockDim.x - 1) / blockDim.x;
    const int t0 = threadIdx.x * per, t1 = min(ntiles, t0 + per);
    int4 sum = make_int4(0, 0, 0, 0);
    for (int t = t0; t < t1; t++) {
        const int4 v = w.tiles[t];
        sum.x += v.x;
        sum.y += v.y;
        sum.z += v.z;
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        int4 run = make_int4(0, 0, 0, 0);
        for (int i = 0; i < (int)blockDim.x; i++) {
            const int4 v = part[i];
            part[i] = run;
            run.x += v.x;
            run.y += v.y;
            run.z += v.z;
        }
        *w.nfar = run.x + run.y;
        *w.nnear = run.z;
        part[0].w = run.x;  // class 1 total, read below (after the barrier)
    }
    __syncthreads();
    const int n1 = part[0].w, nfar = *w.nfar;
    int4 run = part[threadIdx.x];
    for (int t = t0; t < t1; t++) {
        const int4 v = w.tiles[t];
        w.tiles[t] = make_int4(run.x, n1 + run.y, nfar + run.z, 0);
        run.x += v.x;
        run.y += v.y;
        run.z += v.z;
    }
}

// each thread classifies kPartTile / kPartThreads consecutive keys; a block-wide scan of the
// per-thread counts gives every key its slot
__global__ void __launch_bounds__(kPartThreads) part_scatter_kernel(long long nkeys, WinPlan w, int n1log) {
    constexpr int kPer = kPartTile / kPartThreads;
    constexpr int kW = kPartThreads / 32;
    __shared__ int s_n[3][kW];
    const long long k0 = (long long)blockIdx.x * kPartTile + (long long)threadIdx.x * kPer;
    int cls[kPer];
    int cnt[3] = {0, 0, 0};
#pragma unroll
    for (int u = 0; u < kPer; u++) {
        cls[u] = k0 + u < nkeys ? part_class(w, k0 + u, n1log) : 0;
        for (int c = 0; c < 3; c++) cnt[c] += cls[u] == c + 1;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc[3] = {cnt[0], cnt[1], cnt[2]};  // inclusive scans over the warp
    for (int o = 1; o < 32; o <<= 1)
        for (int c = 0; c < 3; c++) {
            const int v = __shfl_up_sync(0xffffffffu, inc[c], o);
            if (lane >= o) inc[c] += v;
        }
    if (lane == 31)
        for (int c = 0; c < 3; c++) s_n[c][warp] = inc[c];
    __syncthreads();
    const int4 base = w.tiles[blockIdx.x];
    int slot[3] = {base.x, base.y, base.z};
    for (int c = 0; c < 3; c++) {
        for (int i = 0; i < warp; i++) slot[c] += s_n[c][i];
        slot[c] += inc[c] - cnt[c];
    }
#pragma unroll
    for (int u = 0; u < kPer; u++)
        if (cls[u] > 0) w.order[slot[cls[u] - 1]++] = (int)(k0 + u);
}

// Histogram bins hold sum w_p w_q (1-fr) and sum w_p w_q fr, in fixed point:
// each contribution is scaled so that the largest pair weight is 2^k coarse
// units (k = 18 for 4^3 x 4^3 points), rounded once in FP32 (the product),
// split into its nearest integer and the rest in 2^-k units, and added with
// two native 32-bit integer shared-memory atomics; neither partial sum can
// overflow within a pass, at whose end the dot products combine them into the
// 64-bit value.  The sums are exact and independent of the order of the atomics.
// Each warp keeps two copies of its histogram, one per half-warp, interleaved
// (copy c of bin b at word 2b + c): the lanes' bins collide in shared-memory
// banks, and the copies cut the wavefronts per atomic from 3.6 to 2.7 (a model
// of the 32k-cell shell's bins; no extra memory: the 64-bit staging histogram
// is gone).
// (64-bit integer shared atomics instead: cubature 90 ms against 66 ms at 32k
// cells.)
// (FP32 shared-memory atomics were slower -- the counters showed them retried
// -- and their rounding grows with the partial sum: a bin summed in FP32 over
// a whole key carries rounding relative to its positive sum into the strongly
// cancelling dot product with an oscillating band table, 2.2e-6 of max|S| on
// the 4x4x4 box without flushes.  21 bits without the fraction gave 1.5e-6 on
// the same box.)  The dot products (window_dots) read the bin-major tables
// from L1/L2, so the tables take no shared memory and two 16-warp CTAs fit on
// an SM.

// 1.5 * 2^23: an FP32 sum with it that lands in [2^23, 2^24), where the FP32 values are the
// integers, is the integer rounding of the other addend, read from the sum's bits (FMA/ALU
// pipes, no conversion instruction)
constexpr float kMagic = 12582912.f;
constexpr int kMagicBits = 0x4B400000;

// Add x (in units of the coarse quantum, |x| < 2^21) to bin b of the fixed-point partial
// histogram: its nearest integer a into hqa, x - a (exact, |x - a| <= 1/2) in units of 1/frac
// (a power of two), rounded to nearest, into hqb (both native integer shared atomics, exact
// and order-independent).  a frac + rn((x - a) frac) is the nearest integer to x frac whatever
// the integer a, so the sums are those of any other integer split.
__device__ __forceinline__ void add_fixed(int* hqa, int* hqb, int b, float x, float frac) {
    const float s = __fadd_rn(x, kMagic);
    const float f = __fsub_rn(x, __fsub_rn(s, kMagic));
    atomicAdd(&hqa[b], __float_as_int(s) - kMagicBits);
    atomicAdd(&hqb[b], __float_as_int(fmaf(f, frac, kMagic)) - kMagicBits);
}

// Table index (i, fr) of r^2 = r2 + r2l when r^2 >= r1^2 is known (every pair of a key whose
// window starts above the linear section): index_r2's log branch with the same operations
// and roundings, its exponent clamp and 2^-E folded into a table indexed by the biased
// exponent, s_ce[eb] = (2^(127-eb), fraction of c_e, integer part of c_e - kMagicBits, 0),
// the mantissa table split into (1/T_k, fraction of z_k) pairs and the integer parts of z_k
// (8 + 2 bytes per entry instead of 16: the lanes' random entries cost fewer shared-memory
// wavefronts), and floor(y) from an FP32 addition rounded down.
__device__ __forceinline__ void index_log(const Lookup& lk, const float4* s_ce, const float2* s_kt2,
                                          const unsigned short* s_kz, float r2, float r2l, int& i, float& fr) {
    const unsigned u = __float_as_uint(r2) >> (23 - kLogBits);  // exponent and top mantissa bits
    const float4 ce = s_ce[(u >> kLogBits) & 255];
    const int k = u & (kLogN - 1);
    const float2 kt = s_kt2[k];
    const float Rk = __uint_as_float(u << (23 - kLogBits));
    const float delta = ((r2 - Rk) + r2l) * (kt.x * ce.x);
    const float ln1p = delta * fmaf(-delta, fmaf(-delta, fmaf(-delta, 0.25f, 1.f / 3.f), 0.5f), 1.f);
    const float y = fmaf(ln1p, lk.cp, ce.y + kt.y);
    const float s = __fadd_rd(y, kMagic);  // kMagic + floor(y), |y| < 2^22
    i = __float_as_int(ce.z) + (int)s_kz[k] + __float_as_int(s);
    fr = __fsub_rn(y, __fsub_rn(s, kMagic));
    if (i > lk.imax) {
        i = lk.imax;
        fr = 1.0f;
    }
}

// Clear bins [0, n) of both copies.  Warp-wide.
__device__ __forceinline__ void clear_fixed(int* hqa, int* hqb, int n, int lane) {
    for (int j = lane; j < 2 * n; j += 32) {
        hqa[j] = 0;
        hqb[j] = 0;
    }
    __syncwarp();
}

constexpr int kMaxPasses = 8;  // passes over the point pairs for windows wider than one histogram
constexpr int kDotChunk = 16;  // bins summed in FP32 per compensated addition in the window dot products

// Dot products of one pass's histogram (bins s0 .. s0 + segw - 1 of the key's window)
// with every table, added into Q.  Two work items per table, alternate chunks of kDotChunk
// bins, spread over the lanes (table t: items 2t and 2t+1 on neighbouring lanes, combined by
// one shuffle).  Far keys: FP32 within a chunk, the chunk sums added by two-sum into an FP32
// pair (as exact as FP64 additions of them, without the FP64 pipe).  Keys whose window
// reaches the linear section of the table or needs several passes (self and adjacent
// cells, whose integrals cancel strongly over several periods of a band table) and every
// key with `dot64`: compensated FP32 -- exact products by FMA, two-sum accumulation, the bin
// values as FP32 high + low parts -- about FP64 accuracy.  The bin values replace the partial
// sums in place: hp[b] is word b of hqa, hl[b] word b of hqb.  Warp-wide.
__device__ __forceinline__ void window_dots(const CubatureArgs& a, const WinPlan& w, int* hqa, int* hqb, int key,
                                            int wx, int s0, int segw, int pass, bool precise, int lane) {
    const int ntab = a.ntab;
    float* hp = reinterpret_cast<float*>(hqa);
    float* hl = reinterpret_cast<float*>(hqb);
    // bin b's two copies are words 2b, 2b+1, and its value goes to word b: the 32 bins of a
    // sweep read words [64k, 64k + 64) and write [32k, 32k + 32), whose inputs earlier sweeps
    // (or this one, before the barrier) have read
    for (int b0 = 0; b0 < segw; b0 += 32) {
        const int b = b0 + lane;
        long long v = 0;
        if (b < segw)
            v = (((long long)hqa[2 * b] + hqa[2 * b + 1]) << w.fbits) + (long long)hqb[2 * b] + hqb[2 * b + 1];
        __syncwarp();
        if (b < segw) {
            if (precise) {
                const double x = (double)v * (double)w.qfine;
                const float hi = (float)x;
                hp[b] = hi;
                hl[b] = (float)(x - (double)hi);
            } else {
                hp[b] = (float)v * w.qfine;
            }
        }
    }
    __syncwarp();
    for (int base = 0; base < 2 * ntab; base += 32) {
        const int it = base + lane;
        const int t = it >> 1, h = it & 1;
        double acc = 0.0;
        if (it < 2 * ntab) {
            const float* tr = w.tabT + (size_t)(wx + s0) * ntab + t;
            if (precise) {
                float sh = 0.f, sl = 0.f;
                for (int b0 = kDotChunk * h; b0 < segw; b0 += 2 * kDotChunk)
                    for (int b = b0; b < min(b0 + kDotChunk, segw); b++) {
                        const float tv = tr[(size_t)b * ntab], v = hp[b];
                        const float p = tv * v;
                        float e;
                        sh = two_sum(sh, p, &e);
                        sl += e + fmaf(tv, v, -p) + tv * hl[b];
                    }
                acc = (double)sh + (double)sl;
            } else {
                float sh = 0.f, sl = 0.f;
                for (int b0 = kDotChunk * h; b0 < segw; b0 += 2 * kDotChunk) {
                    float pt = 0.f;
                    if (b0 + kDotChunk <= segw) {
                        // a whole chunk: the histogram values four at a time (one broadcast
                        // 16-byte shared load; hp is 16-byte aligned, Wkey a multiple of 4)
                        const float* trb = tr + (size_t)b0 * ntab;
#pragma unroll
                        for (int u = 0; u < kDotChunk; u += 4) {
                            const float4 hv = *reinterpret_cast<const float4*>(hp + b0 + u);
                            pt = fmaf(trb[0], hv.x, pt);
                            pt = fmaf(trb[ntab], hv.y, pt);
                            pt = fmaf(trb[2 * ntab], hv.z, pt);
                            pt = fmaf(trb[3 * ntab], hv.w, pt);
                            trb += 4 * ntab;
                        }
                    } else {
                        for (int b = b0; b < segw; b++) pt = fmaf(tr[(size_t)b * ntab], hp[b], pt);
                    }
                    float e;
                    sh = two_sum(sh, pt, &e);
                    sl += e;
                }
                acc = (double)sh + (double)sl;
            }
        }
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        if (it < 2 * ntab && h == 0) {
            double* q = a.Q + (size_t)t * a.ks.nkeys + key;
            *q = pass == 0 ? acc : *q + acc;
        }
    }
    __syncwarp();
}


template <int NG>
struct FarShape {
    static constexpr int NP = NG * NG * NG;
    static constexpr int kWarps = 16;
};

template <int NG>
__global__ void __launch_bounds__(FarShape<NG>::kWarps * 32, 2)
    cubature_far_kernel(CubatureArgs a, Lookup lk, WinPlan w) {
    constexpr int NP = FarShape<NG>::NP;
    constexpr int NG2 = NG * NG;
    constexpr int kWarps = FarShape<NG>::kWarps;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4* pts = reinterpret_cast<float4*>(smem_raw);                  // [kWarps][2][NP]
    int* pa = reinterpret_cast<int*>(pts + kWarps * 2 * NP);  // [kWarps][Wkey][2]: partial sums, integer part
    int* pb = pa + 2 * kWarps * w.Wkey;                       // [kWarps][Wkey][2]: partial sums, fraction
    __shared__ int s_ci[kMaxExp];
    __shared__ float s_cf[kMaxExp];
    __shared__ float4 s_kt[kLogN];
    for (int i = threadIdx.x; i < lk.ne; i += blockDim.x) {
        s_ci[i] = lk.ci[i];
        s_cf[i] = lk.cf[i];
    }
    for (int i = threadIdx.x; i < kLogN; i += blockDim.x) s_kt[i] = lk.kt[i];
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* P2 = pts + warp * 2 * NP;
    float4* P2l = P2 + NP;
    int* hqa = pa + 2 * warp * w.Wkey;
    int* hqb = pb + 2 * warp * w.Wkey;
    const int cpy = lane >> 4;  // this lane's histogram copy
    const bool periodic = (a.coordsys == 1 && a.L > 0);
    const float Lh = (float)a.L, Ll = (float)(a.L - (double)Lh), hL = 0.5f * Lh;
    const int nfar = *w.nfar;
    // consecutive warps take consecutive keys of the order (see part_scatter_kernel)
    for (int kk = blockIdx.x * kWarps + warp; kk < nfar; kk += gridDim.x * kWarps) {
        const int key = w.order[kk];
        const int2 wn = w.win[key];
        const int wl = wn.y;
        int c1[3], c2[3];
        decode_key(a.ks, key, c1, c2);
        const float4* G1 = a.pts + 2 * NP * cell_id(a.ks, c1);
        const float4* G2 = a.pts + 2 * NP * cell_id(a.ks, c2);
        const float4 Oh = G1[2 * (NP / 2)], Ol = G1[2 * (NP / 2) + 1];
        // second-cell points in the order (innermost node l, other nodes): P2[l NG^2 + ij]
        for (int qq = lane; qq < NP; qq += 32) {
            const int q = (qq % NG2) * NG + qq / NG2;
            const float4 Bh = G2[2 * q], Bl = G2[2 * q + 1];
            float lx, ly, lz;
            const float sx = diff2(Bh.x, Bl.x, Oh.x, Ol.x, &lx);
            const float sy = diff2(Bh.y, Bl.y, Oh.y, Ol.y, &ly);
            const float sz = diff2(Bh.z, Bl.z, Oh.z, Ol.z, &lz);
            P2[qq] = make_float4(sx, sy, sz, Bh.w);
            P2l[qq] = make_float4(lx, ly, lz, 0.f);
        }
        __syncwarp();
        int bad = 0;
        // A window wider than the histogram takes several passes over the point pairs, pass s
        // keeping the pairs whose lower bin lies in [s S, s S + S), S = Wkey - 1 (the upper
        // bin of such a pair is at most s S + S); the dot products of the passes are summed.
        const int S = w.Wkey - 1;
        const int npass = (wl - 1 + S - 1) / S;
        for (int pass = 0; pass < npass; pass++) {
            const int s0 = pass * S;
            const int segw = min(S, wl - 1 - s0) + 1;  // bins s0 .. s0 + segw - 1 of the window
            // With several passes a pair whose plain FP32 r^2 lies well outside the
            // separations of this pass's bins skips the exact arithmetic: margins of 1e-4
            // relative plus 0.01 in r cover the rounding of the plain r^2 and of the bin
            // edges.  The first pass has no lower bound and the last no upper bound, so
            // pairs outside the whole window still reach the clamp and the violation count.
            const bool filt = npass > 1 && !periodic;
            float f_lo = 0.f, f_hi = INFINITY;
            if (filt) {
                if (pass > 0) {
                    const float r = bin_edge(lk, wn.x + s0) * (1.f - 1e-4f) - 0.01f;
                    f_lo = r > 0.f ? r * r : 0.f;
                }
                if (pass < npass - 1) {
                    const float r = bin_edge(lk, wn.x + s0 + S) * (1.f + 1e-4f) + 0.01f;
                    f_hi = r * r;
                }
            }
            clear_fixed(hqa, hqb, segw, lane);
            // Mirror symmetry of the innermost axis (phi on spherical grids, z on Cartesian
            // ones): the Gauss nodes are symmetric about each cell's centre, so the pair of
            // innermost nodes (l_p, l_q) and (NG-1-l_q, NG-1-l_p) have the same separation
            // along it, the same other coordinates and the same weight.  Only pairs with
            // l_p + l_q <= NG-1 are evaluated, those with l_p + l_q < NG-1 at twice the
            // weight: 10 of every 16 node pairs for NG = 4.  The lanes take the first-cell
            // points in the order (l, other nodes), so the lanes of one iteration share
            // their smallest l_p and the second-cell loop stops at l_q = NG-1-l_p(min).
            // Every lane runs the same trip counts: the flushes below are warp-wide.
            for (int p0 = 0; p0 < NP; p0 += 32) {
                const int pp = p0 + lane;
                const bool act = pp < NP;
                const int lp = pp / NG2;
                const int p = (pp % NG2) * NG + lp;
                const float4 Ah = act ? G1[2 * p] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 Al = act ? G1[2 * p + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
                float alx, aly, alz;
                const float ax = diff2(Ah.x, Al.x, Oh.x, Ol.x, &alx);
                const float ay = diff2(Ah.y, Al.y, Oh.y, Ol.y, &aly);
                const float az = diff2(Ah.z, Al.z, Oh.z, Ol.z, &alz);
                const int qend = (NG - p0 / NG2) * NG2;  // second-cell points with l_q <= NG-1-l_p(min)
                const int nfl = w.flush > 0 ? w.flush : NP;
                for (int q0 = 0; q0 < qend; q0 += nfl) {
                    if (act) {
#pragma unroll 4
                        for (int q = q0; q < q0 + nfl && q < qend; q++) {
                            const int lsum = lp + q / NG2;
                            if (lsum > NG - 1) continue;  // the mirror image of an evaluated pair
                            const float4 B = P2[q];
                            if (filt) {
                                const float dx = B.x - ax, dy = B.y - ay, dz = B.z - az;
                                const float r2a = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                                if (r2a < f_lo || r2a >= f_hi) continue;
                            }
                            int i;
                            float fr;
                            exact_index(lk, s_ci, s_cf, s_kt, B, P2l[q], ax, alx, ay, aly, az, alz, periodic, Lh, Ll, hL,
                                        i, fr);
                            int bi = i - wn.x;
                            const bool out = bi < 0 || bi > wl - 2;  // outside the window: cannot happen for a sound window
                            bi = min(max(bi, 0), wl - 2) - s0;
                            if (bi >= 0 && bi < S) {
                                bad += out;
                                const float ww = (lsum < NG - 1 ? 2.f : 1.f) * Ah.w * B.w;
                                const float wq = ww * w.qinv;  // fixed point: the largest pair weight -> 2^k units
                                add_fixed(hqa, hqb, 2 * bi + cpy, fmaf(-wq, fr, wq), w.qfrac);
                                add_fixed(hqa, hqb, 2 * bi + 2 + cpy, wq * fr, w.qfrac);
                            }
                        }
                    }
                }
            }
            __syncwarp();
            window_dots(a, w, hqa, hqb, key, wn.x, s0, segw, pass,
                        w.dot64 || npass > 1 || wn.x < lk.n1, lane);
        }
        if (bad) atomicAdd(w.violations, bad);
    }
}

// Spherical grids.  A point of node pair P = (i_r, i_mu) and phi node l sits at
// rho = r sqrt(1 - mu^2), z = r mu, angle phi_l, so for the pair (P of arc h_a,
// l_p) and (Q of arc h_b, l_q)
//   r^2 = (rho_P - rho_Q)^2 + (z_P - z_Q)^2 + 4 rho_P rho_Q sin^2(theta / 2),
// theta the angle between the two phi nodes (cells df apart): three
// non-negative terms, no cancellation.  The first two and 4 rho_P rho_Q are FP32
// pairs formed once per (P, Q) -- one lane each -- and every canonical
// phi-node pair then costs one FP32-pair product and a two-sum; the mirror
// symmetry of the phi nodes is in the table of sin^2(theta / 2) (10 canonical
// pairs of 16 for ng = 4, weighted 2 below the diagonal).  Histograms, flushes,
// passes and dot products as in cubature_far_kernel.
template <int NG>
__global__ void __launch_bounds__(FarShape<NG>::kWarps * 32, 2)
    cubature_far_sph_kernel(CubatureArgs a, Lookup lk, WinPlan w) {
    constexpr int NG2 = NG * NG;
    constexpr int NC = NG * (NG + 1) / 2;
    constexpr int kWarps = FarShape<NG>::kWarps;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4* sphw = reinterpret_cast<float4*>(smem_raw);        // [kWarps][NC]: the key's phi-node pairs
    int* pa = reinterpret_cast<int*>(sphw + kWarps * NC);  // [kWarps][Wkey][2]: partial sums, integer part
    int* pb = pa + 2 * kWarps * w.Wkey;                    // [kWarps][Wkey][2]: partial sums, fraction
    __shared__ int s_ci[kMaxExp];
    __shared__ float s_cf[kMaxExp];
    __shared__ float4 s_kt[kLogN];
    __shared__ float s_wrm[NG2];
    __shared__ float4 s_ce[256];  // index_log's exponent table
    __shared__ float2 s_kt2[kLogN];          // index_log: 1/T_k, fraction of z_k
    __shared__ unsigned short s_kz[kLogN];   // index_log: integer part of z_k
    for (int i = threadIdx.x; i < lk.ne; i += blockDim.x) {
        s_ci[i] = lk.ci[i];
        s_cf[i] = lk.cf[i];
    }
    for (int i = threadIdx.x; i < kLogN; i += blockDim.x) {
        const float4 kt = lk.kt[i];
        s_kt[i] = kt;
        s_kt2[i] = make_float2(kt.x, kt.y);
        s_kz[i] = (unsigned short)__float_as_int(kt.z);  // < 2^16: checked on the host
    }
    for (int i = threadIdx.x; i < NG2; i += blockDim.x) s_wrm[i] = w.wrm[i];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        const int e = min(max(i - 127 - lk.e0, 0), lk.ne - 1);
        s_ce[i] = make_float4(__uint_as_float((unsigned)(254 - i) << 23), lk.cf[e],
                              __int_as_float(lk.ci[e] - kMagicBits), 0.f);
    }
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* SP = sphw + warp * NC;
    int* hqa = pa + 2 * warp * w.Wkey;
    int* hqb = pb + 2 * warp * w.Wkey;
    const int cpy = lane >> 4;  // this lane's histogram copy
    const int nfar = *w.nfar;
    for (int kk = blockIdx.x * kWarps + warp; kk < nfar; kk += gridDim.x * kWarps) {
        const int key = w.order[kk];
        const int2 wn = w.win[key];
        const int wl = wn.y;
        int c1[3], c2[3];
        decode_key(a.ks, key, c1, c2);
        const int ha = c1[0] * a.ks.N2 + c1[1], hb = c2[0] * a.ks.N2 + c2[1], df = c2[2];
        for (int c = lane; c < NC; c += 32) SP[c] = w.sph[(size_t)df * NC + c];
        const float4* AA = w.arc + (size_t)ha * NG2;
        const float4* AB = w.arc + (size_t)hb * NG2;
        __syncwarp();
        int bad = 0;
        const int S = w.Wkey - 1;
        const int npass = (wl - 1 + S - 1) / S;
        for (int pass = 0; pass < npass; pass++) {
            const int s0 = pass * S;
            const int segw = min(S, wl - 1 - s0) + 1;
            const bool filt = npass > 1;
            float f_lo = 0.f, f_hi = INFINITY;
            if (filt) {
                if (pass > 0) {
                    const float r = bin_edge(lk, wn.x + s0) * (1.f - 1e-4f) - 0.01f;
                    f_lo = r > 0.f ? r * r : 0.f;
                }
                if (pass < npass - 1) {
                    const float r = bin_edge(lk, wn.x + s0 + S) * (1.f + 1e-4f) + 0.01f;
                    f_hi = r * r;
                }
            }
            clear_fixed(hqa, hqb, segw, lane);
            // One pass whose window starts above the linear section of the table (most far
            // keys): every pair has r^2 >= r1^2 and its bin is in the histogram, so the loop
            // below needs neither the linear branch nor the pass filter.
            const bool logkeys = w.logkeys && npass == 1 && wn.x > lk.n1;
            // lanes take the (P, Q) node pairs; every lane runs the same trip counts
            for (int c0 = 0; c0 < NG2 * NG2; c0 += 32) {
                const int c = c0 + lane;
                if (c < NG2 * NG2) {
                    const int P = c / NG2, Q = c % NG2;
                    const float4 A = AA[P], B = AB[Q];
                    float rl, zl;
                    const float dr = diff2(B.x, B.y, A.x, A.y, &rl);
                    const float dz = diff2(B.z, B.w, A.z, A.w, &zl);
                    // D = dr^2 + dz^2 and B4 = 4 rho_P rho_Q as FP32 pairs
                    const float pr = __fmul_rn(dr, dr), pz = __fmul_rn(dz, dz);
                    float e1;
                    const float Dh = two_sum(pr, pz, &e1);
                    const float Dl = fmaf(dr, dr, -pr) + fmaf(dz, dz, -pz) + e1 + fmaf(2.f * dr, rl, 2.f * dz * zl);
                    const float t0 = __fmul_rn(A.x, B.x);
                    const float B4h = 4.f * t0;
                    const float B4l = 4.f * (fmaf(A.x, B.x, -t0) + fmaf(A.x, B.y, A.y * B.x));
                    const float wpq = s_wrm[P] * s_wrm[Q];
                    if (logkeys) {
#pragma unroll 2
                        for (int j = 0; j < NC; j++) {
                            const float4 sp = SP[j];
                            const float t = __fmul_rn(B4h, sp.x);
                            const float tl = fmaf(B4h, sp.x, -t) + fmaf(B4h, sp.y, B4l * sp.x);
                            float e;
                            const float r2 = two_sum(Dh, t, &e);
                            const float r2l = e + Dl + tl;
                            int i;
                            float fr;
                            index_log(lk, s_ce, s_kt2, s_kz, r2, r2l, i, fr);
                            int bi = i - wn.x;
                            if ((unsigned)bi > (unsigned)(wl - 2)) {  // outside the window: cannot happen for a sound window
                                ++bad;
                                bi = min(max(bi, 0), wl - 2);
                            }
                            const float ww = wpq * sp.z;
                            const float wq = ww * w.qinv;
                            add_fixed(hqa, hqb, 2 * bi + cpy, fmaf(-wq, fr, wq), w.qfrac);
                            add_fixed(hqa, hqb, 2 * bi + 2 + cpy, wq * fr, w.qfrac);
                        }
                        continue;
                    }
#pragma unroll 2
                    for (int j = 0; j < NC; j++) {
                        const float4 sp = SP[j];
                        if (filt) {
                            const float r2a = fmaf(B4h, sp.x, Dh);
                            if (r2a < f_lo || r2a >= f_hi) continue;
                        }
                        const float t = __fmul_rn(B4h, sp.x);
                        const float tl = fmaf(B4h, sp.x, -t) + fmaf(B4h, sp.y, B4l * sp.x);
                        float e;
                        const float r2 = two_sum(Dh, t, &e);
                        const float r2l = e + Dl + tl;
                        int i;
                        float fr;
                        index_r2(lk, s_ci, s_cf, s_kt, r2, r2l, i, fr);
                        int bi = i - wn.x;
                        const bool out = bi < 0 || bi > wl - 2;  // outside the window: cannot happen for a sound window
                        bi = min(max(bi, 0), wl - 2) - s0;
                        if (bi >= 0 && bi < S) {
                            bad += out;
                            const float ww = wpq * sp.z;
                            const float wq = ww * w.qinv;  // fixed point: the largest pair weight -> 2^k units
                            add_fixed(hqa, hqb, 2 * bi + cpy, fmaf(-wq, fr, wq), w.qfrac);
                            add_fixed(hqa, hqb, 2 * bi + 2 + cpy, wq * fr, w.qfrac);
                        }
                    }
                }
            }
            __syncwarp();
            window_dots(a, w, hqa, hqb, key, wn.x, s0, segw, pass,
                        w.dot64 || npass > 1 || wn.x < lk.n1, lane);
        }
        if (bad) atomicAdd(w.violations, bad);
    }
}

// keys the cubature integrates (the others are copied by the reflection fill)
double canonical_keys(const KeySpace& ks) {
    if (!(ks.coordsys == 2 && ks.mu_reflect)) return (double)ks.nkeys;
    long long n = 0;
    for (int ha = 0; ha < ks.H; ha++)
        for (int hb = ha; hb < ks.H; hb++) {
            const int pa = (ha / ks.N2) * ks.N2 + (ks.N2 - 1 - ha % ks.N2);
            const int pb = (hb / ks.N2) * ks.N2 + (ks.N2 - 1 - hb % ks.N2);
            const int p1 = std::min(pa, pb), p2 = std::max(pa, pb);
            if (p1 > ha || (p1 == ha && p2 >= hb)) ++n;
        }
    return (double)n * ks.nf;
}

double cubature_lookups(const CubatureArgs& a) { return canonical_keys(a.ks) * a.np * a.np * a.ntab; }

template <int NG, bool EXACT>
size_t smem_points() {
    return sizeof(float4) * Shape<NG>::kWarps * (EXACT ? 2 : 1) * Shape<NG>::NP;
}

template <int NG, int G, bool EXACT>
void run(const CubatureArgs& a, int tab0, int ngrp, const Lookup& lk, cudaStream_t s) {
    constexpr int kWarps = Shape<NG>::kWarps;
    constexpr int NP = Shape<NG>::NP;
    const size_t smem = smem_points<NG, EXACT>() + sizeof(float) * (size_t)ngrp * a.xl.n();
    auto k = cubature_kernel<NG, G, EXACT>;
    OPSEC_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem((const void*)k)));
    int dev = 0, nsm = 0, occ = 0;
    OPSEC_CUDA(cudaGetDevice(&dev));
    OPSEC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    OPSEC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kWarps * 32, smem));
    if (occ < 1) fail(OPSEC_ERR_CUDA, "cubature kernel does not fit on an SM");
    long long want = a.list ? (long long)nsm * occ : (a.ks.nkeys + kWarps - 1) / kWarps;
    long long grid = (long long)nsm * occ;
    if (want < grid) grid = want;
    if (g_clock && !a.list) g_clock->begin("cubature", s, canonical_keys(a.ks) * NP * NP * ngrp);
    k<<<(unsigned)grid, kWarps * 32, smem, s>>>(a, tab0, ngrp, lk);
    OPSEC_CUDA(cudaGetLastError());
    if (g_clock && !a.list) g_clock->end(s);
}

template <int NG, bool EXACT>
void run_groups(const CubatureArgs& a, const Lookup& lk, cudaStream_t s, long long* launches) {
    const size_t budget = 222 * 1024 - smem_points<NG, EXACT>();
    int gmax = (int)(budget / (sizeof(float) * a.xl.n()));
    if (gmax > 16) gmax = 16;
    if (gmax < 1) fail(OPSEC_ERR_CONFIG, "xi table too long for shared memory");
    const int ngroups = (a.ntab + gmax - 1) / gmax;
    const int per = (a.ntab + ngroups - 1) / ngroups;
    for (int t0 = 0; t0 < a.ntab; t0 += per) {
        const int g = (a.ntab - t0 < per) ? a.ntab - t0 : per;
        if (g <= 1)
            run<NG, 1, EXACT>(a, t0, g, lk, s);
        else if (g <= 4)
            run<NG, 4, EXACT>(a, t0, g, lk, s);
        else if (g <= 8)
            run<NG, 8, EXACT>(a, t0, g, lk, s);
        else if (g <= 12)
            run<NG, 12, EXACT>(a, t0, g, lk, s);
        else
            run<NG, 16, EXACT>(a, t0, g, lk, s);
        ++*launches;
    }
}

template <int NG>
void run_mode(const CubatureArgs& a, const Lookup& lk, cudaStream_t s, long long* launches) {
    if (a.exact)
        run_groups<NG, true>(a, lk, s, launches);
    else
        run_groups<NG, false>(a, lk, s, launches);
}

}  // namespace

size_t cubature_point_count(const KeySpace& ks, int ng) {
    return (size_t)ks.N1 * ks.N2 * ks.N3 * ng * ng * ng;
}

namespace {
// scratch layout of the window path
struct WinLayout {
    size_t win, order, count, cursor, scal, cen, tabT, arc, wrm, sph, arcbox, sphbox, tiles, total;
};
WinLayout win_layout(const KeySpace& ks, int nx, int ntab, int ng) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t ncell = (size_t)ks.N1 * ks.N2 * ks.N3;
    WinLayout L;
    L.win = 0;
    L.order = L.win + al(sizeof(int2) * ks.nkeys);
    L.count = L.order + al(sizeof(int) * 2 * ks.nkeys);
    L.cursor = L.count + al(sizeof(int) * (nx + 2));
    L.scal = L.cursor + al(sizeof(int) * (nx + 2));
    L.cen = L.scal + 256;
    L.tabT = L.cen + al(sizeof(float4) * ncell);
    L.arc = L.tabT + al(sizeof(float) * (size_t)nx * ntab);
    const bool sph = ks.coordsys == 2;
    L.wrm = L.arc + (sph ? al(sizeof(float4) * (size_t)ks.H * ng * ng) : 0);
    L.sph = L.wrm + (sph ? al(sizeof(float) * (size_t)ng * ng) : 0);
    L.arcbox = L.sph + (sph ? al(sizeof(float4) * (size_t)ks.nf * (ng * (ng + 1) / 2)) : 0);
    L.sphbox = L.arcbox + (sph ? al(sizeof(float4) * (size_t)ks.H) : 0);
    L.tiles = L.sphbox + (sph ? al(sizeof(float2) * (size_t)ks.nf) : 0);
    L.total = L.tiles + al(sizeof(int4) * (size_t)((ks.nkeys + kPartTile - 1) / kPartTile));
    return L;
}

template <int NG>
size_t far_smem(const WinPlan& w, bool sph) {
    const size_t pts = sph ? sizeof(float4) * (NG * (NG + 1) / 2) : sizeof(float4) * 2 * FarShape<NG>::NP;
    return FarShape<NG>::kWarps * (pts + 4 * sizeof(int) * w.Wkey);
}

// Far keys by windows, near keys by table groups in list mode.  Returns false (nothing
// launched) when the per-warp histograms of the widest window do not fit in shared memory.
template <int NG>
bool run_window(const CubatureArgs& a, const Lookup& lk, cudaStream_t s, long long* launches) {
    constexpr int kWarps = FarShape<NG>::kWarps;
    const int nx = a.xl.n();
    WinPlan w{};
    // Cartesian grids also keep the second cell's points per warp: narrower histograms so
    // that two CTAs still fit on an SM
    w.Wkey = std::min(a.coordsys == 2 ? a.win_key : std::min(a.win_key, 256), nx) & ~3;  // 16-byte rows
    w.Wmax = std::min(kMaxPasses * (w.Wkey - 1) + 1, nx);
    w.flush = a.win_flush;
    w.dot64 = a.win_dot64;
    w.logkeys = a.win_logkeys;
    {
        int zmax = 0;  // index_log keeps the integer parts of z_k in 16 bits
        for (int k = 0; k < kLogN; k++) {
            int zi = 0;
            std::memcpy(&zi, &lk.kt[k].z, sizeof zi);
            zmax = std::max(zmax, zi);
        }
        if (zmax > 65535) w.logkeys = 0;
    }
    w.keyorder = a.win_keyorder;
    const bool sph = a.coordsys == 2;
    {
        // Fixed-point partial histograms, summed over a whole pass: at most `pairs`
        // contributions reach one bin (every evaluated pair of a key), each at most the
        // largest pair weight (mirror factor 2 included).  With that weight at 2^k coarse
        // units and fractions in 2^-k of a unit, both partial sums stay below 2^30; the
        // quantum is 2^-2k of the largest weight (2^-36 for 4^3 x 4^3 points).
        constexpr int NP = FarShape<NG>::NP, NC = NG * (NG + 1) / 2;
        const double pairs = sph ? (double)NG * NG * NG * NG * NC : (double)NP * NP;
        const int k = std::min(21, 30 - (int)std::ceil(std::log2(pairs)));
        const double wwmax = 2.0 * std::pow(a.wmax, 6) * (1.0 + 1e-6);
        w.qinv = (float)(std::ldexp(1.0, k) / wwmax);
        w.fbits = k;
        w.qfrac = (float)std::ldexp(1.0, k);
        w.qfine = (float)(wwmax / std::ldexp(1.0, 2 * k));
    }
    const void* kfn = sph ? (const void*)cubature_far_sph_kernel<NG> : (const void*)cubature_far_kernel<NG>;
    if (w.Wkey < 8 || far_smem<NG>(w, sph) > (size_t)max_dynamic_smem(kfn)) return false;
    w.nbucket = nx + 1;
    const WinLayout L = win_layout(a.ks, nx, a.ntab, a.ng);
    if (!a.work || a.work_bytes < L.total) fail(OPSEC_ERR_ARG, "cubature scratch too small");
    unsigned char* base = static_cast<unsigned char*>(a.work);
    w.win = reinterpret_cast<int2*>(base + L.win);
    w.order = reinterpret_cast<int*>(base + L.order);
    w.count = reinterpret_cast<int*>(base + L.count);
    w.cursor = reinterpret_cast<int*>(base + L.cursor);
    w.tiles = reinterpret_cast<int4*>(base + L.tiles);
    int* scal = reinterpret_cast<int*>(base + L.scal);
    w.nfar = scal;
    w.nnear = scal + 1;
    w.violations = scal + 2;
    w.cen = reinterpret_cast<float4*>(base + L.cen);
    w.tabT = reinterpret_cast<float*>(base + L.tabT);
    if (sph) {
        w.arc = reinterpret_cast<float4*>(base + L.arc);
        w.wrm = reinterpret_cast<float*>(base + L.wrm);
        w.sph = reinterpret_cast<float4*>(base + L.sph);
        w.arcbox = reinterpret_cast<float4*>(base + L.arcbox);
        w.sphbox = reinterpret_cast<float2*>(base + L.sphbox);
    }
    OPSEC_CUDA(cudaMemsetAsync(w.count, 0, sizeof(int) * (nx + 2), s));
    OPSEC_CUDA(cudaMemsetAsync(scal, 0, 256, s));
    const long long ncell = (long long)a.ks.N1 * a.ks.N2 * a.ks.N3;
    auto blocks = [](long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 65536); };
    cell_sphere_kernel<<<blocks(ncell), 256, 0, s>>>(a.pts, a.np, ncell, w.cen);
    OPSEC_CUDA(cudaGetLastError());
    if (sph) {
        const long long n = (long long)a.ks.H * a.ng * a.ng + a.ng * a.ng + (long long)a.ks.nf * (a.ng * (a.ng + 1) / 2);
        sph_tables_kernel<<<blocks(n), 256, 0, s>>>(a, w);
        OPSEC_CUDA(cudaGetLastError());
        sph_box_kernel<<<blocks((long long)a.ks.H + a.ks.nf), 256, 0, s>>>(a, w);
        OPSEC_CUDA(cudaGetLastError());
        *launches += 2;
    }
    key_window_kernel<<<blocks(a.ks.nkeys), 256, 0, s>>>(a, w);
    OPSEC_CUDA(cudaGetLastError());
    if (w.keyorder) {
        const long long ntiles = (a.ks.nkeys + kPartTile - 1) / kPartTile;
        if (ntiles > INT_MAX) fail(OPSEC_ERR_CONFIG, "cubature: too many keys");
        const int n1log = sph && w.logkeys ? lk.n1 : INT_MAX;
        part_count_kernel<<<(unsigned)ntiles, kPartThreads, 0, s>>>(a.ks.nkeys, w, n1log);
        OPSEC_CUDA(cudaGetLastError());
        part_scan_kernel<<<1, 1024, 0, s>>>((int)ntiles, w);
        OPSEC_CUDA(cudaGetLastError());
        part_scatter_kernel<<<(unsigned)ntiles, kPartThreads, 0, s>>>(a.ks.nkeys, w, n1log);
        OPSEC_CUDA(cudaGetLastError());
        ++*launches;
    } else {
        bucket_scan_kernel<<<1, 1024, 0, s>>>(w);
        OPSEC_CUDA(cudaGetLastError());
        bucket_scatter_kernel<<<blocks(a.ks.nkeys), 256, 0, s>>>(a.ks.nkeys, w);
        OPSEC_CUDA(cudaGetLastError());
    }
    transpose_tables_kernel<<<blocks((long long)a.ntab * nx), 256, 0, s>>>(a.tab32, a.ntab, nx, w.tabT);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 5;
    int h_nfar = 0;
    OPSEC_CUDA(cudaMemcpyAsync(&h_nfar, w.nfar, sizeof(int), cudaMemcpyDeviceToHost, s));
    OPSEC_CUDA(cudaStreamSynchronize(s));
    // far keys
    const size_t smem = far_smem<NG>(w, sph);
    auto k = sph ? cubature_far_sph_kernel<NG> : cubature_far_kernel<NG>;
    OPSEC_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem((const void*)k)));
    int dev = 0, nsm = 0, occ = 0;
    OPSEC_CUDA(cudaGetDevice(&dev));
    OPSEC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    OPSEC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kWarps * 32, smem));
    if (occ < 1) fail(OPSEC_ERR_CUDA, "cubature window kernel does not fit on an SM");
    const long long grid =
        std::max<long long>(1, std::min<long long>((long long)nsm * occ, ((long long)h_nfar + kWarps - 1) / kWarps));
    if (h_nfar > 0) {
        constexpr int NP = FarShape<NG>::NP;
        if (g_clock) g_clock->begin("cubature_far", s, (double)h_nfar * NP * NP);  // point pairs
        k<<<(unsigned)grid, kWarps * 32, smem, s>>>(a, lk, w);
        OPSEC_CUDA(cudaGetLastError());
        if (g_clock) g_clock->end(s);
        ++*launches;
    }
    // near keys: the table-group kernel over the list
    CubatureArgs an = a;
    an.list = w.order + h_nfar;
    an.list_count = w.nnear;
    run_groups<NG, true>(an, lk, s, launches);
    int viol = 0;
    OPSEC_CUDA(cudaMemcpyAsync(&viol, w.violations, sizeof(int), cudaMemcpyDeviceToHost, s));
    OPSEC_CUDA(cudaStreamSynchronize(s));
    if (viol != 0) fail(OPSEC_ERR_NUMERIC, "cubature: " + std::to_string(viol) + " point pairs outside their key window");
    return true;
}
}  // namespace

size_t cubature_work_bytes(const KeySpace& ks, int nx, int ntab, int ng) { return win_layout(ks, nx, ntab, ng).total; }

void launch_cubature(const CubatureArgs& a, cudaStream_t s, long long* launches) {
    // point table: every Gauss point of every cell, once
    {
        const long long ncell = (long long)a.ks.N1 * a.ks.N2 * a.ks.N3;
        const long long n = ncell * a.np;
        const int threads = 256;
        long long blocks = (n + threads - 1) / threads;
        if (blocks > 65536) blocks = 65536;
        point_table_kernel<<<(unsigned)blocks, threads, 0, s>>>(a, a.ng, ncell);
        OPSEC_CUDA(cudaGetLastError());
        ++*launches;
    }
    Lookup lk{};
    const double inv_du = (a.xl.n2 - 1) / std::log2(a.xl.r2 / a.xl.r1);
    lk.inv_dr = (float)(a.xl.n1 / a.xl.r1);
    lk.inv_dr_lo = (float)(a.xl.n1 / a.xl.r1 - (double)lk.inv_dr);
    lk.r1 = (float)a.xl.r1;
    lk.r1sq = (float)(a.xl.r1 * a.xl.r1);
    lk.inv_du = (float)inv_du;
    lk.cp = (float)(0.5 * inv_du / std::log(2.0));
    lk.n1 = a.xl.n1;
    lk.imax = a.xl.n() - 2;
    // exponents of r (fast) or r^2 (exact) over [r1, r2], one spare below and above
    const double lo = a.exact ? a.xl.r1 * a.xl.r1 : a.xl.r1;
    const double hi = a.exact ? a.xl.r2 * a.xl.r2 : a.xl.r2;
    const double scale = a.exact ? 0.5 : 1.0;  // log2 r = scale * log2(argument)
    int e_lo = 0, e_hi = 0;
    std::frexp(lo, &e_lo);  // lo = f 2^e_lo, f in [0.5,1): binary exponent of lo is e_lo - 1
    std::frexp(hi, &e_hi);
    lk.e0 = e_lo - 2;
    lk.ne = e_hi - e_lo + 3;
    if (lk.ne > kMaxExp) fail(OPSEC_ERR_CONFIG, "xi table spans too many octaves of r");
    for (int k = 0; k < lk.ne; k++) {
        const double c = a.xl.n1 + (scale * (lk.e0 + k) - std::log2(a.xl.r1)) * inv_du;
        const double ci = std::floor(c);
        lk.ci[k] = (int)ci;
        lk.cf[k] = (float)(c - ci);
    }
    for (int k = 0; k < kLogN; k++) {
        const double T = 1.0 + (double)k / kLogN;
        const double z = 0.5 * std::log2(T) * inv_du;
        const double zi = std::floor(z);
        int zi_bits = (int)zi;
        float zi_f;
        std::memcpy(&zi_f, &zi_bits, sizeof zi_f);
        lk.kt[k] = make_float4((float)(1.0 / T), (float)(z - zi), zi_f, 0.f);
    }
    // exact mode: far keys through the window path when it applies
    bool done = false;
    if (a.exact && a.window && a.work) {
        if (g_clock) g_clock->begin("cubature", s, cubature_lookups(a));
        switch (a.ng) {
        case 1: done = run_window<1>(a, lk, s, launches); break;
        case 2: done = run_window<2>(a, lk, s, launches); break;
        case 3: done = run_window<3>(a, lk, s, launches); break;
        case 4: done = run_window<4>(a, lk, s, launches); break;
        case 5: done = run_window<5>(a, lk, s, launches); break;
        case 6: done = run_window<6>(a, lk, s, launches); break;
        default: fail(OPSEC_ERR_CONFIG, "sig.gauss must be between 1 and 6");
        }
        if (g_clock) g_clock->end(s);
    }
    if (!done) switch (a.ng) {
    case 1: run_mode<1>(a, lk, s, launches); break;
    case 2: run_mode<2>(a, lk, s, launches); break;
    case 3: run_mode<3>(a, lk, s, launches); break;
    case 4: run_mode<4>(a, lk, s, launches); break;
    case 5: run_mode<5>(a, lk, s, launches); break;
    case 6: run_mode<6>(a, lk, s, launches); break;
    default: fail(OPSEC_ERR_CONFIG, "sig.gauss must be between 1 and 6");
    }
    if (a.ks.coordsys == 2 && a.ks.mu_reflect) {
        long long blocks = (a.ks.nkeys + 255) / 256;
        if (blocks > 65536) blocks = 65536;
        reflect_fill_kernel<<<(unsigned)blocks, 256, 0, s>>>(a.ks, a.ntab, a.Q);
        OPSEC_CUDA(cudaGetLastError());
        ++*launches;
    }
}

}  // namespace opsec
