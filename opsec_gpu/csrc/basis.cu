// basis.cu -- the cell builder on the GPU (basis.cpp:89-128, 160-190): the
// expected count Nbar of every grid cell, the integral of the selection
// function over the cell, and its volume.
//
// Selections (the reference's two):
//   Cartesian  constant nbar (BoxSurvey.cpp:61-75): Nbar = nbar V, exactly.
//   spherical  radial linear spline x HEALPix completeness map
//              (SphericalSurvey.cpp:51-80): the selection is a product, so
//              Nbar = [int radial(r) r^2 dr] x [int mask dmu dphi].  The radial
//              integral is exact: per spline segment the integrand is a cubic
//              in r, integrated in closed form.  The angular integral is
//              dmu dphi without a map, else the mean of the map over an S x S
//              grid of points of the cell (uniform in mu and phi, the area
//              measure) -- the map is piecewise constant on pixels, whose edges
//              no fixed rule follows (the reference's adaptive cubature stops
//              at epsrel 1e-5 or 5e6 points there).
// The reference integrates over (r^3, mu, phi) without the Jacobian's 1/3,
// so its spherical Nbar is three times the expected count (basis.cpp:72-84,
// 103-108); `basis.quirk3 = 1` reproduces that, the default does not.
#include <cmath>

#include "engine.h"

namespace opsec {

// HEALPix pixel index (Gorski et al. 2005, ApJ 622:759): the sphere in 12
// base faces of nside^2 pixels; |z| <= 2/3 is the equatorial belt, the rest
// the polar caps.  ring: pixels numbered along iso-latitude rings from the
// north pole; nest: face-major, the pixel's (x, y) in the face bit-interleaved.
__device__ inline long long hp_ring(long long ns, double z, double tt) {
    const double za = fabs(z);
    if (za <= 2.0 / 3.0) {
        const double t1 = ns * (0.5 + tt), t2 = ns * z * 0.75;
        const long long jp = (long long)(t1 - t2), jm = (long long)(t1 + t2);  // ascending / descending edge lines
        const long long ir = ns + 1 + jp - jm;                                   // ring from z = 2/3, 1 .. 2 ns + 1
        const long long kshift = 1 - (ir & 1);
        long long ip = (jp + jm - ns + kshift + 1) / 2;                          // 0 .. 4 ns (4 ns wraps to 0)
        if (ip >= 4 * ns) ip -= 4 * ns;
        return 2 * ns * (ns - 1) + 4 * ns * (ir - 1) + ip;
    }
    const double tp = tt - floor(tt), tmp = sqrt(3.0 * (1.0 - za));
    const long long jp = (long long)(ns * tp * tmp), jm = (long long)(ns * (1.0 - tp) * tmp);
    const long long ir = jp + jm + 1;                                            // ring from the nearer pole
    long long ip = (long long)(tt * ir);
    if (ip >= 4 * ir) ip -= 4 * ir;
    return z > 0 ? 2 * ir * (ir - 1) + ip : 12 * ns * ns - 2 * ir * (ir + 1) + ip;
}

__device__ inline long long spread_bits(long long v) {  // bit k of v -> bit 2k
    long long r = 0;
    for (int k = 0; k < 31; k++) r |= ((v >> k) & 1LL) << (2 * k);
    return r;
}

__device__ inline long long hp_nest(long long ns, double z, double tt) {
    const double za = fabs(z);
    long long face, ix, iy;
    if (za <= 2.0 / 3.0) {
        const double t1 = ns * (0.5 + tt), t2 = ns * z * 0.75;
        const long long jp = (long long)(t1 - t2), jm = (long long)(t1 + t2);
        const long long fp = jp / ns, fm = jm / ns;
        face = fp == fm ? (fp | 4) : (fp < fm ? fp : fm + 8);
        ix = jm % ns;
        iy = ns - (jp % ns) - 1;
    } else {
        int nt = (int)tt;
        if (nt >= 4) nt = 3;
        const double tp = tt - nt, tmp = sqrt(3.0 * (1.0 - za));
        long long jp = (long long)(ns * tp * tmp), jm = (long long)(ns * (1.0 - tp) * tmp);
        if (jp > ns - 1) jp = ns - 1;
        if (jm > ns - 1) jm = ns - 1;
        if (z >= 0) {
            face = nt;
            ix = ns - jm - 1;
            iy = ns - jp - 1;
        } else {
            face = nt + 8;
            ix = jp;
            iy = jm;
        }
    }
    return face * ns * ns + spread_bits(ix) + 2 * spread_bits(iy);
}

// theta, phi as the reference passes them (z = cos theta, phi wrapped into [0, 2 pi))
__device__ inline long long hp_ang2pix(long long ns, int nest, double theta, double phi) {
    const double z = cos(theta);
    if (phi >= 2.0 * M_PI) phi -= 2.0 * M_PI;
    if (phi < 0.0) phi += 2.0 * M_PI;
    const double tt = phi / (0.5 * M_PI);
    return nest ? hp_nest(ns, z, tt) : hp_ring(ns, z, tt);
}

namespace {

__global__ void ang2pix_kernel(long long ns, int nest, int n, const double* theta, const double* phi, long long* pix) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        pix[i] = hp_ang2pix(ns, nest, theta[i], phi[i]);
}

// int_a^b radial(r) r^2 dr, radial linear between knots and zero outside [r_0, r_last)
__device__ double radial_integral(int nr, const double* R, const double* V, double a, double b) {
    double s = 0.0;
    for (int i = 0; i + 1 < nr; i++) {
        const double x0 = fmax(a, R[i]), x1 = fmin(b, R[i + 1]);
        if (!(x1 > x0)) continue;
        const double slope = (V[i + 1] - V[i]) / (R[i + 1] - R[i]), c0 = V[i] - slope * R[i];
        s += c0 * (x1 * x1 * x1 - x0 * x0 * x0) / 3.0 + slope * (x1 * x1 * x1 * x1 - x0 * x0 * x0 * x0) / 4.0;
    }
    return s;
}

__global__ void basis_kernel(BasisArgs b) {
    const long long ncell = (long long)b.n[0] * b.n[1] * b.n[2];
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
        const double* e = b.bounds + 6 * c;
        double V, N;
        if (b.coordsys == 1) {
            V = (e[1] - e[0]) * (e[3] - e[2]) * (e[5] - e[4]);
            N = b.nbar * V;
        } else {
            const double dmu = e[3] - e[2], dphi = e[5] - e[4];
            V = (e[1] * e[1] * e[1] - e[0] * e[0] * e[0]) / 3.0 * dmu * dphi;
            const double R = radial_integral(b.nrad, b.rad_r, b.rad_n, e[0], e[1]);
            double A = dmu * dphi;
            if (b.nside > 0 && R != 0.0) {
                double m = 0.0;
                for (int s = 0; s < b.samples; s++) {
                    const double theta = acos(e[2] + (s + 0.5) * dmu / b.samples);
                    for (int t = 0; t < b.samples; t++)
                        m += b.mask[hp_ang2pix(b.nside, b.nest, theta, e[4] + (t + 0.5) * dphi / b.samples)];
                }
                A *= m / ((double)b.samples * b.samples);
            }
            N = R * A * (b.quirk3 ? 3.0 : 1.0);
        }
        b.out[2 * c] = V;
        b.out[2 * c + 1] = N;
    }
}

unsigned grid_of(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 65536); }

}  // namespace

void launch_basis(const BasisArgs& b, cudaStream_t s, long long* launches) {
    basis_kernel<<<grid_of((long long)b.n[0] * b.n[1] * b.n[2]), 256, 0, s>>>(b);
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;
}

void launch_ang2pix(long long nside, int nest, int n, const double* theta, const double* phi, long long* pix,
                    cudaStream_t s, long long* launches) {
    ang2pix_kernel<<<grid_of(n), 256, 0, s>>>(nside, nest, n, theta, phi, pix);
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;
}

}  // namespace opsec
