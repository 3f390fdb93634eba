// cubature.cu -- cell-pair integrals Q_t(key) for every xi table at once.
//
// Q_ab = int_{[0,1]^6} xi(|x(u1..3) - y(u4..6)|) d^6u over the two cells of a
// symmetry key (sig.cpp:381-482), by the ng^3 x ng^3 Gauss-Legendre product
// rule.  Cartesian cells map affinely; spherical cells map r through r^3 so
// that the map is volume-uniform (sig.cpp:453-458).
//
// Layout and precision:
//  * one warp integrates one key; a CTA holds G xi tables in shared memory
//    (FP32) and loops its warps over keys;
//  * the 2 ng^3 Gauss points of the pair are built in FP64 from per-axis node
//    tables, shifted to the first cell (pair-relative coordinates) and stored
//    in FP32 in the warp's slice of shared memory, so FP32 differences keep
//    ~1e-7 relative accuracy at every separation;
//  * per lane: FP32 distance, log2 index into the table, linear interpolation
//    (the QSpline rule, QSpline.cpp:61-70) and FP32 sums over the ng^3 points
//    of the second cell; FP64 for the outer sum and the warp reduction.
// Periodic boxes wrap each pair difference into [-L/2, L/2) (BoxSurvey.cpp:26-30).
#include <cmath>

#include "engine.h"

namespace opsec {
namespace {


// Table index of a distance r.  Linear section: t = r n1 / r1.  Log section:
// t = n1 + (log2 r - log2 r1) (n2-1) / log2(r2/r1).  To keep the fraction of
// t at the precision of r itself, log2 r is split into its binary exponent e
// and log2 of the mantissa m in [1, 2) (the hardware log2 is accurate to
// ~2^-22 absolute there), and the offset of each exponent,
// c_e = n1 + (e - log2 r1) (n2-1)/log2(r2/r1), is precomputed in FP64 as an
// integer part plus an FP32 fraction.
constexpr int kMaxExp = 64;
struct Lookup {
    float inv_dr;   // n1 / r1: index in the linear section
    float r1;
    float inv_du;   // (n2-1) / log2(r2/r1)
    int n1;
    int imax;       // n - 2
    int e0;         // smallest exponent held in the offset table
    int ne;         // entries in the offset table
    int ci[kMaxExp];    // integer part of c_e
    float cf[kMaxExp];  // fraction of c_e
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

template <int NG>
__device__ __forceinline__ void point_xyz(const CubatureArgs& a, const int* c, int p, double* x, double* w) {
    const int i = p / (NG * NG), j = (p / NG) % NG, l = p % NG;
    *w = a.w[i] * a.w[j] * a.w[l];
    if (a.coordsys == 1) {
        x[0] = a.node1[c[0] * NG + i];
        x[1] = a.node2[c[1] * NG + j];
        x[2] = a.node3[c[2] * NG + l];
    } else {
        const double r = a.node1[c[0] * NG + i];
        const double mu = a.node2[c[1] * NG + j];
        const double s = a.snode2[c[1] * NG + j];
        const double rs = r * s;
        x[0] = rs * a.cphi[c[2] * NG + l];
        x[1] = rs * a.sphi[c[2] * NG + l];
        x[2] = r * mu;
    }
}

template <int NG, int G, int kWarps>
__global__ void __launch_bounds__(kWarps * 32, 1) cubature_kernel(CubatureArgs a, int tab0, int ngrp, Lookup lk) {
    constexpr int NP = NG * NG * NG;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nx = a.xl.n();
    float4* pts = reinterpret_cast<float4*>(smem_raw);           // [kWarps][2][NP]
    float* tab = reinterpret_cast<float*>(pts + kWarps * 2 * NP);  // [ngrp][nx]

    for (int i = threadIdx.x; i < ngrp * nx; i += blockDim.x) tab[i] = a.tab32[(size_t)tab0 * nx + i];
    __shared__ int s_ci[kMaxExp];
    __shared__ float s_cf[kMaxExp];
    for (int i = threadIdx.x; i < lk.ne; i += blockDim.x) {
        s_ci[i] = lk.ci[i];
        s_cf[i] = lk.cf[i];
    }
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* P1 = pts + warp * 2 * NP;
    float4* P2 = P1 + NP;
    const bool periodic = (a.coordsys == 1 && a.L > 0);
    const float Lf = (float)a.L, hL = (float)(0.5 * a.L);

    for (long long key = (long long)blockIdx.x * kWarps + warp; key < a.ks.nkeys;
         key += (long long)gridDim.x * kWarps) {
        int c1[3], c2[3];
        decode_key(a.ks, key, c1, c2);
        double org[3], wo;
        point_xyz<NG>(a, c1, NP / 2, org, &wo);
        for (int p = lane; p < NP; p += 32) {
            double x[3], w;
            point_xyz<NG>(a, c1, p, x, &w);
            P1[p] = make_float4((float)(x[0] - org[0]), (float)(x[1] - org[1]), (float)(x[2] - org[2]), (float)w);
            point_xyz<NG>(a, c2, p, x, &w);
            P2[p] = make_float4((float)(x[0] - org[0]), (float)(x[1] - org[1]), (float)(x[2] - org[2]), (float)w);
        }
        __syncwarp();

        double tot[G];
#pragma unroll
        for (int t = 0; t < G; t++) tot[t] = 0.0;
        for (int p = lane; p < NP; p += 32) {
            const float4 A = P1[p];
            float acc[G];
#pragma unroll
            for (int t = 0; t < G; t++) acc[t] = 0.f;
#pragma unroll 4
            for (int q = 0; q < NP; q++) {
                const float4 B = P2[q];
                float dx = B.x - A.x, dy = B.y - A.y, dz = B.z - A.z;
                if (periodic) {
                    dx += Lf * (float)((dx < -hL) - (dx >= hL));
                    dy += Lf * (float)((dy < -hL) - (dy >= hL));
                    dz += Lf * (float)((dz < -hL) - (dz >= hL));
                }
                const float r = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
                int i;
                float fr;
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
            for (int t = 0; t < G; t++) tot[t] += (double)A.w * (double)acc[t];
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

template <int NG, int G, int kWarps>
void run(const CubatureArgs& a, int tab0, int ngrp, const Lookup& lk, cudaStream_t s) {
    constexpr int NP = NG * NG * NG;
    const size_t smem = sizeof(float4) * kWarps * 2 * NP + sizeof(float) * (size_t)ngrp * a.xl.n();
    auto k = cubature_kernel<NG, G, kWarps>;
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

template <int NG, int G>
void run_w(const CubatureArgs& a, int tab0, int g, const Lookup& lk, cudaStream_t s, int warps) {
    if (warps == 16)
        run<NG, G, 16>(a, tab0, g, lk, s);
    else
        run<NG, G, 8>(a, tab0, g, lk, s);
}

template <int NG>
void run_groups(const CubatureArgs& a, const Lookup& lk, cudaStream_t s, long long* launches) {
    constexpr int NP = NG * NG * NG;
    // 16 warps per CTA (twice the latency hiding) while the point buffers leave room for tables
    const int warps = (NG <= 4) ? 16 : 8;
    const size_t budget = 224 * 1024 - sizeof(float4) * warps * 2 * NP;
    int gmax = (int)(budget / (sizeof(float) * a.xl.n()));
    if (gmax > 16) gmax = 16;
    if (gmax < 1) fail(OPSEC_ERR_CONFIG, "xi table too long for shared memory");
    const int ngroups = (a.ntab + gmax - 1) / gmax;
    const int per = (a.ntab + ngroups - 1) / ngroups;
    for (int t0 = 0; t0 < a.ntab; t0 += per) {
        const int g = (a.ntab - t0 < per) ? a.ntab - t0 : per;
        if (g <= 1)
            run_w<NG, 1>(a, t0, g, lk, s, warps);
        else if (g <= 4)
            run_w<NG, 4>(a, t0, g, lk, s, warps);
        else if (g <= 8)
            run_w<NG, 8>(a, t0, g, lk, s, warps);
        else if (g <= 12)
            run_w<NG, 12>(a, t0, g, lk, s, warps);
        else
            run_w<NG, 16>(a, t0, g, lk, s, warps);
        ++*launches;
    }
}

}  // namespace

void launch_cubature(const CubatureArgs& a, cudaStream_t s, long long* launches) {
    Lookup lk;
    const double inv_du = (a.xl.n2 - 1) / std::log2(a.xl.r2 / a.xl.r1);
    lk.inv_dr = (float)(a.xl.n1 / a.xl.r1);
    lk.r1 = (float)a.xl.r1;
    lk.inv_du = (float)inv_du;
    lk.n1 = a.xl.n1;
    lk.imax = a.xl.n() - 2;
    int e_lo = 0, e_hi = 0;
    std::frexp(a.xl.r1, &e_lo);  // r1 = f 2^e_lo, f in [0.5,1): binary exponent of r1 is e_lo - 1
    std::frexp(a.xl.r2, &e_hi);
    lk.e0 = e_lo - 1;
    lk.ne = e_hi - e_lo + 2;  // one spare exponent above r2 (clamped to the last table entry)
    if (lk.ne > kMaxExp) fail(OPSEC_ERR_CONFIG, "xi table spans too many octaves of r");
    for (int k = 0; k < lk.ne; k++) {
        const double c = a.xl.n1 + ((lk.e0 + k) - std::log2(a.xl.r1)) * inv_du;
        const double ci = std::floor(c);
        lk.ci[k] = (int)ci;
        lk.cf[k] = (float)(c - ci);
    }
    switch (a.ng) {
    case 1: run_groups<1>(a, lk, s, launches); break;
    case 2: run_groups<2>(a, lk, s, launches); break;
    case 3: run_groups<3>(a, lk, s, launches); break;
    case 4: run_groups<4>(a, lk, s, launches); break;
    case 5: run_groups<5>(a, lk, s, launches); break;
    case 6: run_groups<6>(a, lk, s, launches); break;
    default: fail(OPSEC_ERR_CONFIG, "sig.gauss must be between 1 and 6");
    }
}

}  // namespace opsec
