// gemm_df.cu -- FP64-accurate products C = A^T B or A B in double-FP32 arithmetic on the FP32 pipes,
// for the iterative eigensolver's refinement (chfsi.cu), whose Rayleigh-Ritz step needs S Q to
// about 1e-11 of |S| |Q| (residuals of 1e-6 theta for eigenvalues down to 1e-4 of the largest).
//
// On this part FP64 instructions issue at 1/64 of the FP32 rate (cuBLAS DGEMM: ~1.0 TF/s).  Here
// every FP64 operand is held as the unevaluated sum hi + lo of two floats (~48 bits; df_split
// converts once, so the products' inner loops run no FP64 instruction) and each
// product-accumulate is error-free up to the accumulator's own rounding:
//   p = ah bh (rounded), e = ah bh - p (one FMA, exact) + ah bl + al bh (two FMAs),
//   (sh, sl) += p by Knuth's two-sum, sl += e
// -- twelve FP32 instructions per FP64 multiply-add, kept in order by the _rn intrinsics (no
// contraction into FMAs that would change the error terms).  The lo part of the accumulator is
// renormalised once, at the end.  Relative accuracy: ~2^-46 of sum_k |A_ki B_kj| per element.
//
// Tiles: 128 (rows of C) x 64 (columns) per CTA of 256 threads, K in slices of 16 staged through
// shared memory as (hi, lo) pairs, column index XOR k within each group of 16 (so that the
// stores of one column's 16 values spread over the banks); each thread accumulates 8 x 4 outputs
// (rows tx + 16 r, columns ty + 16 c), so its operand reads are conflict-free (A) or broadcasts
// (B) and its stores of C are coalesced along the rows.  The next slice's global loads are in
// flight during the current slice's arithmetic.  One CTA per SM (up to 255 registers a thread):
// 32 independent accumulator pairs per thread keep the FP32 pipes fed from eight warps.  Products
// with few output tiles and a long K (Q^T Z: (M+8)^2 outputs over N) split K over the grid's z
// extent into FP64 partial sums that a second kernel adds, so that the launch fills the SMs.
#include <algorithm>

#include "engine.h"
#include "gemm_df.h"

namespace opsec {
namespace {

constexpr int DM = 128, DN = 64, DK = 16, DT = 256;

__global__ void df_split_kernel(size_t n, const double* x, float2* out) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const float h = __double2float_rn(x[e]);
        out[e] = make_float2(h, __double2float_rn(x[e] - (double)h));
    }
}

// C[i + j ldc] = sum_z P[z][j][i] (the split-K partials, M x N each)
__global__ void df_reduce_kernel(int M, int N, int nz, const double* P, double* C, long long ldc) {
    const size_t total = (size_t)M * N;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        double v = 0.0;
        for (int z = 0; z < nz; z++) v += P[(size_t)z * total + e];
        C[(e / M) * ldc + e % M] = v;
    }
}

// (sh, sl) += a b, a = (ah, al), b = (bh, bl)
__device__ __forceinline__ void df_acc(float& sh, float& sl, float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    const float s = __fadd_rn(sh, p);
    const float v = __fsub_rn(s, sh);
    const float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, v)), __fsub_rn(p, v));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(t, e));
}

// AK: A stored K-major (element (k, i) at A[k + i lda], C = A^T B), else rows-major along i
// (element (i, k) at A[i + k lda], C = A B).  B is always K-major: element (k, j) at B[k + j ldb].
template <bool AK>
__global__ void __launch_bounds__(DT, 1)
    df_gemm_kernel(int M, int N, int K, int kchunk, const float2* __restrict__ A, long long lda,
                   const float2* __restrict__ B, long long ldb, double* __restrict__ C, long long ldc) {
    __shared__ float2 As[2][DK][DM];
    __shared__ float2 Bs[2][DK][DN];
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const int i0 = blockIdx.x * DM, j0 = blockIdx.y * DN;
    // this CTA's range of K: [kb, ke); its partial sums go to slice z of C (ldc = M)
    const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    if (gridDim.z > 1) C += (size_t)blockIdx.z * M * N;

    // staging: element e = t + 256 q of the slice; K-major operands: column e / 16 of the tile,
    // k = e % 16 (each column's 16 values are one 128-byte segment); A along i: i = e % 128,
    // k = e / 128 (a warp reads 32 consecutive rows)
    float2 ra[DM * DK / DT], rb[DN * DK / DT];
    auto a_ik = [&](int e, int& i, int& k) {
        if (AK) {
            i = e / DK;
            k = e % DK;
        } else {
            i = e % DM;
            k = e / DM;
        }
    };
    auto fetch = [&](int k0) {
#pragma unroll
        for (int q = 0; q < DM * DK / DT; q++) {
            int i, k;
            a_ik(t + DT * q, i, k);
            i += i0;
            k += k0;
            ra[q] = (i < M && k < ke) ? (AK ? A[(size_t)i * lda + k] : A[(size_t)k * lda + i]) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int q = 0; q < DN * DK / DT; q++) {
            const int e = t + DT * q, j = j0 + e / DK, k = k0 + e % DK;
            rb[q] = (j < N && k < ke) ? B[(size_t)j * ldb + k] : make_float2(0.f, 0.f);
        }
    };
    auto stash = [&](int buf) {
#pragma unroll
        for (int q = 0; q < DM * DK / DT; q++) {
            int i, k;
            a_ik(t + DT * q, i, k);
            As[buf][k][i ^ k] = ra[q];
        }
#pragma unroll
        for (int q = 0; q < DN * DK / DT; q++) {
            const int e = t + DT * q, k = e % DK;
            Bs[buf][k][(e / DK) ^ k] = rb[q];
        }
    };

    float sh[8][4], sl[8][4];
#pragma unroll
    for (int r = 0; r < 8; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) sh[r][c] = sl[r][c] = 0.f;

    const int nk = (ke - kb + DK - 1) / DK;
    fetch(kb);
    stash(0);
    __syncthreads();
    for (int kt = 0; kt < nk; kt++) {
        const int buf = kt & 1;
        if (kt + 1 < nk) fetch(kb + (kt + 1) * DK);
#pragma unroll 4
        for (int k = 0; k < DK; k++) {
            float2 a[8], b[4];
#pragma unroll
            for (int r = 0; r < 8; r++) a[r] = As[buf][k][(tx + 16 * r) ^ k];
#pragma unroll
            for (int c = 0; c < 4; c++) b[c] = Bs[buf][k][(ty + 16 * c) ^ k];
#pragma unroll
            for (int r = 0; r < 8; r++)
#pragma unroll
                for (int c = 0; c < 4; c++) df_acc(sh[r][c], sl[r][c], a[r], b[c]);
        }
        if (kt + 1 < nk) stash(buf ^ 1);
        __syncthreads();
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int j = j0 + ty + 16 * c;
        if (j >= N) continue;
#pragma unroll
        for (int r = 0; r < 8; r++) {
            const int i = i0 + tx + 16 * r;
            if (i < M) C[(size_t)j * ldc + i] = (double)sh[r][c] + (double)sl[r][c];
        }
    }
}

}  // namespace

void df_split(size_t n, const double* x, float* out, cudaStream_t s, long long* launches) {
    if (n == 0) return;
    df_split_kernel<<<(unsigned)std::min<size_t>((n + 255) / 256, 8192), 256, 0, s>>>(n, x,
                                                                                     reinterpret_cast<float2*>(out));
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;
}

void df_gemm(bool a_kmajor, int M, int N, int K, const float* A, long long lda, const float* B, long long ldb,
             double* C, long long ldc, DevBuf<double>& work, cudaStream_t s, long long* launches) {
    if (M < 1 || N < 1) return;
    int dev = 0, nsm = 0;
    OPSEC_CUDA(cudaGetDevice(&dev));
    OPSEC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const long long tiles = (long long)((M + DM - 1) / DM) * ((N + DN - 1) / DN);
    // split K when the tiles fill less than two waves, keeping at least 256 of K per split
    int nz = 1;
    if (tiles < 2LL * nsm) nz = (int)std::max(1LL, std::min<long long>((2LL * nsm + tiles - 1) / tiles, K / 256));
    const int kchunk = ((K + nz - 1) / nz + DK - 1) / DK * DK;
    nz = std::max(1, (K + kchunk - 1) / kchunk);
    double* out = C;
    long long ldo = ldc;
    if (nz > 1) {
        work.alloc((size_t)nz * M * N);
        out = work.p;
        ldo = M;
    }
    const dim3 grid((unsigned)((M + DM - 1) / DM), (unsigned)((N + DN - 1) / DN), (unsigned)nz);
    const float2* a = reinterpret_cast<const float2*>(A);
    const float2* b = reinterpret_cast<const float2*>(B);
    if (a_kmajor)
        df_gemm_kernel<true><<<grid, DT, 0, s>>>(M, N, K, kchunk, a, lda, b, ldb, out, ldo);
    else
        df_gemm_kernel<false><<<grid, DT, 0, s>>>(M, N, K, kchunk, a, lda, b, ldb, out, ldo);
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;
    if (nz > 1) {
        df_reduce_kernel<<<(unsigned)std::min<long long>(((long long)M * N + 255) / 256, 4096), 256, 0, s>>>(
            M, N, nz, work.p, C, ldc);
        OPSEC_CUDA(cudaGetLastError());
        ++*launches;
    }
}

}  // namespace opsec
