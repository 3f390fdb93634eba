// mock.cu -- mock counts on the GPU: a Gaussian random field of the context's
// P(k) on a periodic mesh enclosing the survey, sampled at the cell centres,
// and Poisson counts N_a ~ Poisson(Nbar_a max(0, 1 + b delta_a)).
//
// The reference generates mocks by Poisson-sampling a Gaussian random field
// drawn in Fourier space with variance P(k) (code/opsec/utils/gmock.cpp:1-40,
// FFTW); here the field comes from white noise shaped in Fourier space, which
// has the same statistics, and counts are drawn per survey cell.
//
// Random numbers: Philox4x64-10 (Salmon, Moraes, Dror, Shaw 2011), a counter-
// based generator, so every draw is a pure function of (key, counter) and the
// order of threads does not matter:
//   white noise   key (seed, kNoiseStream), counter (i / 4, 0, 0, 0): the four
//                 64-bit outputs give two Box-Muller pairs, mesh points i..i+3
//   Poisson       key (seed, kPoissonStream), counter (a, j, 0, 0) for cell a,
//                 draw j: lambda < 10 by inversion of the CDF with one uniform
//                 (j = 0); lambda >= 10 by PTRS, the transformed rejection of
//                 Hoermann (1993), attempt j on draw j + 1
// A uniform is (x >> 11) 2^-53.  The FFTs are cuFFT D2Z / Z2D (FP64).
#include <cufft.h>

#include <cmath>
#include <string>
#include <vector>

#include "engine.h"

namespace opsec {
namespace {

__device__ __forceinline__ void philox4x64(unsigned long long c[4], unsigned long long k0, unsigned long long k1) {
    for (int r = 0; r < 10; r++) {
        if (r) {
            k0 += 0x9E3779B97F4A7C15ULL;
            k1 += 0xBB67AE8584CAA73BULL;
        }
        const unsigned long long hi0 = __umul64hi(0xD2E7470EE14C6C93ULL, c[0]), lo0 = 0xD2E7470EE14C6C93ULL * c[0];
        const unsigned long long hi1 = __umul64hi(0xCA5A826395121157ULL, c[2]), lo1 = 0xCA5A826395121157ULL * c[2];
        const unsigned long long n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
    }
}

__device__ __forceinline__ double u01(unsigned long long x) { return (double)(x >> 11) * 0x1.0p-53; }

// white noise: mesh points 4t .. 4t+3 from counter t
__global__ void mock_noise_kernel(long long npts, unsigned long long seed, double* g) {
    const long long nblk = (npts + 3) / 4;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nblk; t += (long long)gridDim.x * blockDim.x) {
        unsigned long long c[4] = {(unsigned long long)t, 0ULL, 0ULL, 0ULL};
        philox4x64(c, seed, kMockNoiseStream);
        const double ra = sqrt(-2.0 * log(1.0 - u01(c[0]))), pa = 2.0 * M_PI * u01(c[1]);
        const double rb = sqrt(-2.0 * log(1.0 - u01(c[2]))), pb = 2.0 * M_PI * u01(c[3]);
        const double v[4] = {ra * cos(pa), ra * sin(pa), rb * cos(pb), rb * sin(pb)};
        for (int j = 0; j < 4; j++)
            if (4 * t + j < npts) g[4 * t + j] = v[j];
    }
}

// F(k) *= sqrt(P(|k|) / V) n^1.5 / n^3 (the last factor normalises the unnormalised inverse):
// unit white noise has |F|^2 = n^3 per mode, so the field's variance is sum_k P(k) / V
__global__ void mock_spectrum_kernel(int n, double box, int npk, const double* pk, double2* F) {
    const int nz = n / 2 + 1;
    const long long total = (long long)n * n * nz;
    const double kf = 2.0 * M_PI / box;
    const double scale = 1.0 / pow((double)n, 1.5);
    const double* X = pk;
    const double* Y = pk + npk;
    const double* B = pk + 2 * npk;
    const double* C = pk + 3 * npk;
    const double* D = pk + 4 * npk;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const int l = (int)(e % nz);
        const long long t = e / nz;
        const int j = (int)(t % n), i = (int)(t / n);
        // numpy fftfreq order: 0 .. (n-1)/2, then -(n/2) .. -1
        const int fx = i < (n - 1) / 2 + 1 ? i : i - n, fy = j < (n - 1) / 2 + 1 ? j : j - n;
        const double kk = kf * sqrt((double)fx * fx + (double)fy * fy + (double)l * l);
        double amp = 0.0;
        if (e != 0) amp = sqrt(spline_eval(npk, X, Y, B, C, D, kk) / (box * box * box)) * scale;
        F[e].x *= amp;
        F[e].y *= amp;
    }
}

__device__ int poisson_draw(double lam, unsigned long long cell, unsigned long long seed) {
    if (!(lam > 0.0)) return 0;
    if (lam < 10.0) {
        unsigned long long c[4] = {cell, 0ULL, 0ULL, 0ULL};
        philox4x64(c, seed, kMockPoissonStream);
        const double u = u01(c[0]);
        int k = 0;
        double p = exp(-lam), F = p;
        while (u > F && k < 1000) {
            ++k;
            p *= lam / k;
            F += p;
        }
        return k;
    }
    const double slam = sqrt(lam), loglam = log(lam);
    const double b = 0.931 + 2.53 * slam, a = -0.059 + 0.02483 * b;
    const double invalpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2.0);
    for (int j = 0; j < kMockMaxAttempts; j++) {
        unsigned long long c[4] = {cell, (unsigned long long)(j + 1), 0ULL, 0ULL};
        philox4x64(c, seed, kMockPoissonStream);
        const double U = u01(c[0]) - 0.5, V = u01(c[1]);
        const double us = 0.5 - fabs(U);
        const double k = floor((2.0 * a / us + b) * U + lam + 0.43);
        if (us >= 0.07 && V <= vr) return (int)k;
        if (k < 0.0 || (us < 0.013 && V > us)) continue;
        if (log(V) + log(invalpha) - log(a / (us * us) + b) <= -lam + k * loglam - lgamma(k + 1.0)) return (int)k;
    }
    return (int)floor(lam);  // kMockMaxAttempts rejections in a row: probability below 1e-60
}

__global__ void mock_counts_kernel(int ncells, const long long* idx, const double* nbar, const double* field,
                                   double bias, unsigned long long seed, double* counts, double* delta) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < ncells; a += gridDim.x * blockDim.x) {
        const double d = field[idx[a]];
        const double lam = fmax(nbar[a] * (1.0 + bias * d), 0.0);
        counts[a] = (double)poisson_draw(lam, (unsigned long long)a, seed);
        delta[a] = d;
    }
}

unsigned blocks_for(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 65536); }

void cufft_check(cufftResult r, const char* what) {
    if (r != CUFFT_SUCCESS) fail(OPSEC_ERR_CUDA, std::string(what) + ": cuFFT error " + std::to_string((int)r));
}

}  // namespace

void launch_mock_counts(const MockArgs& m, MockPlans& plans, cudaStream_t s, long long* launches) {
    const int n = m.ngrid;
    const long long npts = (long long)n * n * n;
    if (plans.n != n) {
        if (plans.fwd) cufftDestroy(plans.fwd);
        if (plans.inv) cufftDestroy(plans.inv);
        plans.fwd = plans.inv = 0;
        plans.n = 0;
        cufftHandle f = 0, i = 0;
        cufft_check(cufftPlan3d(&f, n, n, n, CUFFT_D2Z), "cufftPlan3d(D2Z)");
        if (cufftPlan3d(&i, n, n, n, CUFFT_Z2D) != CUFFT_SUCCESS) {
            cufftDestroy(f);
            fail(OPSEC_ERR_CUDA, "cufftPlan3d(Z2D) failed");
        }
        plans.fwd = f;
        plans.inv = i;
        plans.n = n;
    }
    cufft_check(cufftSetStream(plans.fwd, s), "cufftSetStream");
    cufft_check(cufftSetStream(plans.inv, s), "cufftSetStream");
    mock_noise_kernel<<<blocks_for((npts + 3) / 4), 256, 0, s>>>(npts, m.seed, m.grid);
    OPSEC_CUDA(cudaGetLastError());
    cufft_check(cufftExecD2Z(plans.fwd, m.grid, reinterpret_cast<cufftDoubleComplex*>(m.spec)), "cufftExecD2Z");
    mock_spectrum_kernel<<<blocks_for((long long)n * n * (n / 2 + 1)), 256, 0, s>>>(n, m.box, m.npk, m.pk, m.spec);
    OPSEC_CUDA(cudaGetLastError());
    cufft_check(cufftExecZ2D(plans.inv, reinterpret_cast<cufftDoubleComplex*>(m.spec), m.grid), "cufftExecZ2D");
    mock_counts_kernel<<<blocks_for(m.ncells), 256, 0, s>>>(m.ncells, m.idx, m.nbar, m.grid, m.bias, m.seed, m.counts,
                                                            m.delta);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 3;
}

void destroy_mock_plans(MockPlans& plans) {
    if (plans.fwd) cufftDestroy(plans.fwd);
    if (plans.inv) cufftDestroy(plans.inv);
    plans.fwd = plans.inv = 0;
    plans.n = 0;
}

}  // namespace opsec
