// project_simt.cu -- CUDA-core form of the fused projection C_p = B'^T Q_p B'.
//
// Per band (comma-scalapack.cpp:228-265, with S_p = D Q_p D and B' = D B):
//   step 1  T[j][a] = sum_b Q_p(a,b) B'[j][b]   -- Q_p tiles gathered from the
//           key table straight into shared memory; S_p is never stored
//   step 2  C[i][j] = sum_a B'[i][a] T[j][a]    -- upper-triangle tiles only,
//           written packed (k = j(j+1)/2 + i)
// FP32 products with FP32 sums over 256-long K chunks and FP64 across
// chunks.  This is the portable form; the tensor-core kernel in
// project_tc.cu is the fast path and this one checks it.
#include <cmath>

#include "engine.h"

namespace opsec {
namespace {

constexpr int BM = 64, BN = 64, BK = 32, KFLUSH = 256;

struct QGather {
    KeySpace ks;
    const int* h;  // spherical arc / Cartesian dx
    const int* f;  // spherical phi / Cartesian dy
    const int* g;  // Cartesian dz
    const float* Q;
    int n;
    __device__ __forceinline__ float operator()(int a, int b) const {
        if (a >= n || b >= n) return 0.f;
        long long key;
        if (ks.coordsys == 1) {
            int kx = abs(h[a] - h[b]), ky = abs(f[a] - f[b]), kz = abs(g[a] - g[b]);
            key = ((long long)kx * ks.N2 + ky) * ks.N3 + kz;
        } else {
            int df = abs(f[a] - f[b]);
            if (ks.fold && df > ks.N3 - df) df = ks.N3 - df;
            key = ((long long)h[a] * ks.H + h[b]) * ks.nf + df;
        }
        return Q[key];
    }
};

struct RowF64 {  // element (row, k) of a row-major [rows][ld] FP64 matrix
    const double* p;
    int rows, ld;
    __device__ __forceinline__ float operator()(int r, int k) const {
        return (r < rows && k < ld) ? (float)p[(size_t)r * ld + k] : 0.f;
    }
};

struct RowF32 {
    const float* p;
    int rows, ld;
    __device__ __forceinline__ float operator()(int r, int k) const {
        return (r < rows && k < ld) ? p[(size_t)r * ld + k] : 0.f;
    }
};

// acc[4][4] (FP64) += sum over K of A(m,k) B(n,k) for this thread's 4x4 outputs
template <class LA, class LB>
__device__ void tile_mma(const LA& A, const LB& B, int m0, int n0, int K, double (&acc)[4][4]) {
    __shared__ float As[BK][BM + 4];
    __shared__ float Bs[BK][BN + 4];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    float part[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) part[i][j] = 0.f;
    for (int k0 = 0; k0 < K; k0 += BK) {
        for (int e = threadIdx.x; e < BM * BK; e += blockDim.x) {
            int mm = e / BK, kk = e % BK;
            As[kk][mm] = A(m0 + mm, k0 + kk);
            Bs[kk][mm] = B(n0 + mm, k0 + kk);
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < BK; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) part[i][j] = fmaf(a[i], b[j], part[i][j]);
        }
        __syncthreads();
        if (((k0 + BK) % KFLUSH) == 0 || k0 + BK >= K) {
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    acc[i][j] += (double)part[i][j];
                    part[i][j] = 0.f;
                }
        }
    }
}

// step 1: T[j][a] for a-tile (x) and mode tile (y)
__global__ void __launch_bounds__(256) step1_kernel(QGather Qg, RowF64 Bp, float* T, int N, int M) {
    const int a0 = blockIdx.x * BM, j0 = blockIdx.y * BN;
    double acc[4][4] = {};
    tile_mma(Qg, Bp, a0, j0, N, acc);
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int a = a0 + ty * 4 + i, jj = j0 + tx * 4 + j;
            if (a < N && jj < M) T[(size_t)jj * N + a] = (float)acc[i][j];
        }
}

// step 2: packed upper tiles of C = B'^T T
__global__ void __launch_bounds__(256) step2_kernel(RowF64 Bp, RowF32 Tt, float* Dp, int N, int M, int nt) {
    // blockIdx.x -> (ti <= tj)
    int t = blockIdx.x, tj = 0;
    while (t > tj) {
        t -= tj + 1;
        ++tj;
    }
    const int ti = t;
    const int i0 = ti * BM, j0 = tj * BN;
    double acc[4][4] = {};
    tile_mma(Bp, Tt, i0, j0, N, acc);
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            int ii = i0 + ty * 4 + i, jj = j0 + tx * 4 + j;
            if (ii < M && jj < M && ii <= jj) Dp[(size_t)jj * (jj + 1) / 2 + ii] = (float)acc[i][j];
        }
}

}  // namespace

void launch_project_simt(const ProjectArgs& a, cudaStream_t s, long long* launches) {
    const int N = a.ncells, M = a.nmodes;
    float* T = static_cast<float*>(a.work);
    const size_t K = (size_t)M * (M + 1) / 2;
    const int nt = (M + BN - 1) / BN;
    for (int p = 0; p < a.nbands; p++) {
        QGather Qg{a.ks, a.cell_h, a.cell_f, a.cell_g, a.Qsq + (size_t)(1 + p) * a.ks.nsquare, N};
        RowF64 Bp{a.Bs, M, N};
        step1_kernel<<<dim3((N + BM - 1) / BM, (M + BN - 1) / BN), 256, 0, s>>>(Qg, Bp, T, N, M);
        OPSEC_CUDA(cudaGetLastError());
        RowF32 Tt{T, M, N};
        step2_kernel<<<nt * (nt + 1) / 2, 256, 0, s>>>(Bp, Tt, a.Dp + (size_t)p * K, N, M, nt);
        OPSEC_CUDA(cudaGetLastError());
        *launches += 2;
    }
}

}  // namespace opsec
