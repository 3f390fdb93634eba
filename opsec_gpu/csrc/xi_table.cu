// xi_table.cu -- xi(r) and band-derivative tables on the GPU, FP64.
//
// xi_l^m(r) = (1/2pi^2) int dk k^m j_l(kr) P(k) exp(-(k/kdamp)^2) by Simpson's
// rule, l = 0, m = 2 (Model.cpp:84-123):
//   table 0   GetXi       Nk = 32768 on [0, 10], P = cubic spline of the pkfile
//   table 1+p GetXiDeriv  Nk = 8192 on [k_p, k_{p+1}], P = 1 on [k_p, k_{p+1})
// (RealModel.cpp:98-127).  The spline is zero outside [x0, x_last) and the
// constant band is zero at k = k_{p+1}, so the last Simpson node of every
// band table contributes nothing, as in the reference.
#include <cmath>

#include "df64.h"
#include "engine.h"

namespace opsec {
namespace {

constexpr int kNkXi = 32768;
constexpr int kNkBand = 8192;
constexpr double kTwoPi2 = 2.0 * M_PI * M_PI;

__device__ __forceinline__ double sj0(double x) {
    double x2 = x * x;
    return (x2 < 1e-4) ? 1 - x2 * (1 / 6. + x2 * (1 / 120. - x2 * (1 / 5040.))) : sin(x) / x;
}

// second half of the scratch holds mult_j / k_j
__host__ __device__ inline size_t scratch_half(const XiTableArgs& a) {
    return (size_t)(kNkXi + 1) + (size_t)a.nbands * (kNkBand + 1);
}

struct TableSpec {
    int nk;
    double kmin, kmax;
    size_t off;  // offset of its weights in scratch
};

__device__ TableSpec table_spec(int t, int nbands, const double* lo, const double* hi) {
    TableSpec s;
    if (t == 0) {
        s.nk = kNkXi;
        s.kmin = 0.0;
        s.kmax = 10.0;
        s.off = 0;
    } else {
        s.nk = kNkBand;
        s.kmin = lo[t - 1];
        s.kmax = hi[t - 1];
        s.off = (size_t)(kNkXi + 1) + (size_t)(t - 1) * (kNkBand + 1);
    }
    return s;
}

// Simpson weights times the k-dependent factors (Model.cpp:104-112).
__global__ void simpson_weights_kernel(XiTableArgs a) {
    const int t = blockIdx.y;
    TableSpec s = table_spec(t, a.nbands, a.band_lo, a.band_hi);
    const double dk = (s.kmax - s.kmin) / s.nk;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j <= s.nk; j += gridDim.x * blockDim.x) {
        double k = s.kmin + j * dk;
        double P;
        if (t == 0)
            P = spline_eval(a.npk, a.pk_x, a.pk_y, a.pk_b, a.pk_c, a.pk_d, k);
        else
            P = (k >= s.kmin && k < s.kmax) ? 1.0 : 0.0;  // ConstantSpline(1, kmin, kmax)
        double mult = 2 + 2 * (j % 2) - (j == 0) - (j == s.nk);
        mult *= P * (k * k) * exp(-k * k / (1.0 * 1.0));
        mult *= (dk / 3) / kTwoPi2;
        a.scratch[s.off + j] = mult;
        const double mk = (k > 0.0) ? mult / k : 0.0;  // for sin(kr)/(kr) = (1/k) sin(kr) / r
        a.scratch[s.off + j + scratch_half(a)] = mk;
        reinterpret_cast<float2*>(a.scratch + 2 * scratch_half(a))[s.off + j] = df_pack(df_from(mk));
    }
}

constexpr int kRPerWarp = 4;   // r values per warp; each weight load feeds all of them
constexpr int kAnchor = 16;    // Chebyshev steps per lane between rotation anchors

// One warp per (table, 4 consecutive r): sum_j mult_j j0(k_j r), to FP64 accuracy.
//
// Terms with (k_j r)^2 < 1e-4 use the series of sj0 (Model.cpp:56-59); k_j
// grows with j, so they form a prefix j < jc of the sum, evaluated term by
// term (series, or sin(x)/x for the few prefix terms past the threshold when
// the four r values have different jc).  The rest is (1/r) sum_j (mult_j/k_j)
// sin(k_j r) with lane l taking j = jc + l + 32 m: along one lane the angle
// advances by theta = 32 dk r and sin(x + (m+1) theta) = 2 cos(theta) sin(x + m
// theta) - sin(x + (m-1) theta), two product-accumulates per term with the
// accumulation.  The recurrence restarts every kAnchor steps from anchor values
// (sin, cos) advanced by the angle-addition rotation through 32 kAnchor dk r, so
// the error stays within a few hundred ulps of the largest term (the error of
// the three-term recurrence grows at most quadratically in its length).  Six
// CTAs of 128 threads per SM (80 registers a thread): 2.75 -> 2.60 ms for the 41
// tables of the 32k-cell build against four CTAs at 128 registers.
__global__ void __launch_bounds__(128, 6) xi_sum_kernel(XiTableArgs a) {
    const int n = a.xl.n();
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int t = blockIdx.y;
    const int i0 = warp * kRPerWarp;
    if (i0 >= n) return;
    TableSpec s = table_spec(t, a.nbands, a.band_lo, a.band_hi);
    const double dk = (s.kmax - s.kmin) / s.nk;
    const double* mult = a.scratch + s.off;
    const double* minv = a.scratch + s.off + scratch_half(a);
    const float2* minv2 = reinterpret_cast<const float2*>(a.scratch + 2 * scratch_half(a)) + s.off;
    const int nk = s.nk;

    double r[kRPerWarp], acc_series[kRPerWarp], acc_sin[kRPerWarp];
    df acc_rec[kRPerWarp];
    int jc = 0;
#pragma unroll
    for (int q = 0; q < kRPerWarp; q++) {
        r[q] = a.r[min(i0 + q, n - 1)];  // past the end: a copy of the last r, not stored
        acc_series[q] = 0.0;
        acc_sin[q] = 0.0;
        acc_rec[q] = df{0.f, 0.f};
        // first j with (kmin + j dk) r >= 0.01, from below; the prefix loop tests each term exactly
        if (r[q] > 0.0) {
            const double jf = (0.01 / r[q] - s.kmin) / dk;
            jc = max(jc, jf < 0.0 ? 0 : (jf > (double)nk ? nk + 1 : (int)jf + 2));
        } else {
            // r = 0: every term is mult_j j0(0) = mult_j; sin(k_j r) = 0 below
            for (int j = lane; j <= nk; j += 32) acc_series[q] += mult[j];
        }
    }
    jc = min(jc, nk + 1);

    // prefix, term by term
    for (int j = lane; j < jc; j += 32) {
        const double k = s.kmin + j * dk;
#pragma unroll
        for (int q = 0; q < kRPerWarp; q++) {
            const double x = k * r[q];
            if (r[q] == 0.0) continue;  // summed above
            if (x * x < 1e-4)
                acc_series[q] += mult[j] * sj0(x);
            else
                acc_sin[q] += minv[j] * sin(x);
        }
    }

    // the rest, by the three-term recurrence, in double-FP32 (FP64 instructions issue at 1/64 of
    // the FP32 rate here).  The sines and cosines it starts from: one FP64 sincos per lane --
    // lane 8 q + u, for r_q, of the warp's first angle (kmin + jc dk) r_q (u = 0), of 2^(u-1)
    // dk r_q (u = 1..5), of 32 dk r_q (u = 6) and of 32 kAnchor dk r_q (u = 7) -- split into
    // (hi, lo) pairs and shared by shuffles; each lane turns the first angle into its own,
    // (kmin + (jc + lane) dk) r_q, by rotations through the powers of two in its lane number;
    // then the recurrence, its sum and the anchor rotations as (hi, lo) float pairs
    static_assert(kRPerWarp * 8 == 32, "one FP64 sincos per lane");
    if (jc <= nk) {
        df c2[kRPerWarp], cth[kRPerWarp], sth[kRPerWarp], cT[kRPerWarp], sT[kRPerWarp], sn[kRPerWarp], cs[kRPerWarp];
        df sl, cl;  // this lane's sincos
        {
            const int q = lane >> 3, u = lane & 7;
            const double rq = a.r[min(i0 + q, n - 1)];
            const double ang = u == 0   ? (s.kmin + jc * dk) * rq
                               : u <= 5 ? (double)(1 << (u - 1)) * dk * rq
                               : u == 6 ? 32.0 * dk * rq
                                        : (32.0 * kAnchor) * dk * rq;
            double sa, ca;
            sincos(ang, &sa, &ca);
            sl = df_from(sa);
            cl = df_from(ca);
        }
        auto shfl = [&](df v, int src) {
            return df{__shfl_sync(0xffffffffu, v.h, src), __shfl_sync(0xffffffffu, v.l, src)};
        };
#pragma unroll
        for (int q = 0; q < kRPerWarp; q++) {
            df sq = shfl(sl, 8 * q), cq = shfl(cl, 8 * q);
#pragma unroll
            for (int bit = 0; bit < 5; bit++) {
                const df sb = shfl(sl, 8 * q + 1 + bit), cb = shfl(cl, 8 * q + 1 + bit);
                if ((lane >> bit) & 1) {  // rotate by 2^bit dk r_q
                    const df s1 = df_fma(df_mul(sq, cb), cq, sb);
                    cq = df_fms(df_mul(cq, cb), sq, sb);
                    sq = s1;
                }
            }
            sn[q] = sq;
            cs[q] = cq;
            sth[q] = shfl(sl, 8 * q + 6);
            cth[q] = shfl(cl, 8 * q + 6);
            c2[q] = df{2.f * cth[q].h, 2.f * cth[q].l};
            sT[q] = shfl(sl, 8 * q + 7);
            cT[q] = shfl(cl, 8 * q + 7);
        }
        const df zero{0.f, 0.f};
        for (int j0 = jc + lane; j0 <= nk; j0 += 32 * kAnchor) {
            df cur[kRPerWarp], prev[kRPerWarp];
#pragma unroll
            for (int q = 0; q < kRPerWarp; q++) {
                cur[q] = sn[q];
                prev[q] = df_fms(df_fma(zero, sn[q], cth[q]), cs[q], sth[q]);  // sin(x - theta)
            }
            const int steps = min(kAnchor, (nk - j0) / 32 + 1);
            for (int m = 0; m < steps; m++) {
                const df w = df_unpack(minv2[j0 + 32 * m]);
#pragma unroll
                for (int q = 0; q < kRPerWarp; q++) {
                    acc_rec[q] = df_fma(acc_rec[q], w, cur[q]);
                    const df nxt = df_fma(df{-prev[q].h, -prev[q].l}, c2[q], cur[q]);
                    prev[q] = cur[q];
                    cur[q] = nxt;
                }
            }
#pragma unroll
            for (int q = 0; q < kRPerWarp; q++) {  // rotate the anchor by 32 kAnchor dk r
                const df sn2 = df_fma(df_fma(zero, sn[q], cT[q]), cs[q], sT[q]);
                cs[q] = df_fms(df_fma(zero, cs[q], cT[q]), sn[q], sT[q]);
                sn[q] = sn2;
            }
        }
    }

#pragma unroll
    for (int q = 0; q < kRPerWarp; q++) {
        const double sins = acc_sin[q] + df_to(acc_rec[q]);
        double acc = (r[q] > 0.0) ? acc_series[q] + sins / r[q] : acc_series[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0 && i0 + q < n) {
            a.xi64[(size_t)t * n + i0 + q] = acc;
            a.xi32[(size_t)t * n + i0 + q] = (float)acc;
        }
    }
}

}  // namespace

void launch_xi_tables(const XiTableArgs& a, cudaStream_t s, long long* launches) {
    const int ntab = 1 + a.nbands;
    simpson_weights_kernel<<<dim3(64, ntab), 256, 0, s>>>(a);
    OPSEC_CUDA(cudaGetLastError());
    const int n = a.xl.n();
    const int warps = (n + kRPerWarp - 1) / kRPerWarp;
    // 128-thread CTAs: three fit on an SM at this kernel's register count (12 warps in flight)
    xi_sum_kernel<<<dim3((warps * 32 + 127) / 128, ntab), 128, 0, s>>>(a);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 2;
}

}  // namespace opsec
