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
#include <cmath>
#include <cstring>

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

template <int NG>
struct Shape {
    static constexpr int NP = NG * NG * NG;
    // 16 warps per CTA (twice the latency hiding) while the point buffers leave room for tables
    static constexpr int kWarps = NG <= 4 ? 16 : 8;
};

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
    // rows of the upper triangle: row ha starts at ha*H - ha(ha-1)/2
    const double H2 = 2.0 * ks.H + 1.0;
    int ha = (int)floor((H2 - sqrt(H2 * H2 - 8.0 * (double)tri)) * 0.5);
    if (ha < 0) ha = 0;
    while (ha > 0 && (long long)ha * ks.H - (long long)ha * (ha - 1) / 2 > tri) --ha;
    while ((long long)(ha + 1) * ks.H - (long long)(ha + 1) * ha / 2 <= tri) ++ha;
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
    const double H2 = 2.0 * ks.H + 1.0;
    int ha = (int)floor((H2 - sqrt(H2 * H2 - 8.0 * (double)tri)) * 0.5);
    if (ha < 0) ha = 0;
    while (ha > 0 && (long long)ha * ks.H - (long long)ha * (ha - 1) / 2 > tri) --ha;
    while ((long long)(ha + 1) * ks.H - (long long)(ha + 1) * ha / 2 <= tri) ++ha;
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

    for (long long key = (long long)blockIdx.x * kWarps + warp; key < a.ks.nkeys;
         key += (long long)gridDim.x * kWarps) {
        if (a.ks.coordsys == 2 && a.ks.mu_reflect && reflect_partner(a.ks, key) < key) continue;  // copied later
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
                    const float4 Bl = P2l[q];
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
                        const float ln1p =
                            delta * fmaf(-delta, fmaf(-delta, fmaf(-delta, 0.25f, 1.f / 3.f), 0.5f), 1.f);
                        const float y = fmaf(ln1p, lk.cp, s_cf[e] + kt.y);
                        const float yi = floorf(y);
                        i = s_ci[e] + __float_as_int(kt.z) + (int)yi;
                        fr = y - yi;
                        if (i < lk.n1) {
                            i = lk.n1;
                            fr = 0.f;
                        }
                    }
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
    OPSEC_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, nsm = 0, occ = 0;
    OPSEC_CUDA(cudaGetDevice(&dev));
    OPSEC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    OPSEC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kWarps * 32, smem));
    if (occ < 1) fail(OPSEC_ERR_CUDA, "cubature kernel does not fit on an SM");
    long long want = (a.ks.nkeys + kWarps - 1) / kWarps;
    long long grid = (long long)nsm * occ;
    if (want < grid) grid = want;
    if (g_clock) g_clock->begin("cubature", s, (double)a.ks.nkeys * NP * NP * ngrp);
    k<<<(unsigned)grid, kWarps * 32, smem, s>>>(a, tab0, ngrp, lk);
    OPSEC_CUDA(cudaGetLastError());
    if (g_clock) g_clock->end(s);
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
    switch (a.ng) {
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
