// chfsi.cu -- the top M eigenpairs of the dense signal matrix S by Chebyshev-filtered
// subspace iteration, for grids whose dense FP64 eigensolve is too slow.
//
// The reference finds them with implicitly restarted Lanczos (ARPACK, "LA", tol 1e-5,
// ncv = 2 Nmodes; ParpackSolver.cpp:111-123, called from klt.cpp:173-248): one
// matrix-vector product at a time.  With S resident in HBM the work here is GEMMs of S
// with a block of B = M + g vectors:
//   bounds      k Lanczos steps on S (FP64 matrix-vector products): the extreme Ritz
//               values theta_min, theta_max of the tridiagonal T_k, hi = theta_max +
//               |beta_k| above the spectrum (Zhou & Li, Linear Algebra Appl. 435 (2011)
//               480-493) and lo = theta_min - 2 % of the spread below it
//   filter      Y = p_d(S) X with p_d the degree-d Chebyshev polynomial of [lo, cut],
//               scaled to 1 at hi, by the scaled three-term recurrence (Zhou, Saad,
//               Tiago, Chelikowsky, J. Comput. Phys. 219 (2006) 172-184): d GEMMs
//               N x N x B on the tensor cores, by the engine's tcgen05 kernel (gemm_tc.cu:
//               S split once into FP16 hi + lo, the block at every step, three FP16
//               products, the recurrence's axpy fused into the epilogue; `klt.gemm = tc`)
//               or cuBLAS (BF16x9: each FP32 operand as three BF16 terms; or FP32 SIMT).
//               Every product with S (filter, Rayleigh-Ritz, correction solve) takes
//               the same route.  d is the largest degree
//               (up to klt.degree) whose gain p(hi) / p(theta_M) stays below 1e4, so
//               that the wanted columns keep FP32 precision beside the top ones
//   basis       Householder QR of Y (FP32)
//   Rayleigh-   H = Y^T S Y, its eigenpairs in FP64, X = Y V, residuals |S x - theta x|;
//   Ritz        cut = the smallest Ritz value; stop when the top M residuals are below
//               tol theta_i or the FP32 floor, or stop improving
//   refinement  on the top Mr = M + 8 vectors, up to klt.refine rounds of: Rayleigh-Ritz
//               in FP64 (products with the FP64 S in double-FP32 on the FP32 pipes,
//               gemm_df.cu, or cuBLAS DGEMM: `klt.fp64`), the FP64 residuals r_j = S u_j -
//               theta_j u_j, and the correction equation of Jacobi-Davidson,
//               (I - U U^T)(theta_j - S)(I - U U^T) d_j = r_j, positive definite on the
//               complement of U, solved by CG with FP32 GEMMs (klt.cg steps), x_j = u_j +
//               d_j.  The FP32 filter leaves the vectors eigenvectors of S rounded to
//               FP32 (relative residual ~1e-7 lambda_max / lambda); each round gains
//               the CG's reduction on it, the last Rayleigh-Ritz fixes the eigenvalues
// Eigenvectors come out mode-major (M x N) with the eigenvalues descending, the sign of
// each mode fixed so that its entry of largest magnitude is positive.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "chfsi_host.h"
#include "engine.h"
#include "gemm_df.h"
#include "gemm_tc.h"

namespace opsec {
namespace {

constexpr int kLanczos = 32;  // Lanczos steps for the spectrum bounds

void blas_ok(cublasStatus_t st, const char* what) {
    if (st != CUBLAS_STATUS_SUCCESS) fail(OPSEC_ERR_CUDA, std::string(what) + ": cuBLAS status " + std::to_string((int)st));
}
void solver_ok(cusolverStatus_t st, const char* what) {
    if (st != CUSOLVER_STATUS_SUCCESS)
        fail(OPSEC_ERR_CUDA, std::string(what) + ": cuSOLVER status " + std::to_string((int)st));
}

unsigned blocks(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16); }

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {  // splitmix64 finaliser
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

template <typename T>
__global__ void random_kernel(size_t n, unsigned long long seed, T* x) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        x[e] = (T)((double)(mix64(seed * 0x9E3779B97F4A7C15ULL + e) >> 11) * 0x1.0p-52 - 1.0);  // uniform [-1, 1)
}

__global__ void narrow_kernel(size_t n, const double* in, float* out) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        out[e] = (float)in[e];
}

// A = I (n x n)
__global__ void identity_kernel(int n, double* A) {
    const size_t total = (size_t)n * n;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        A[e] = (e % n == e / n) ? 1.0 : 0.0;
}

__global__ void widen_kernel(size_t n, const float* in, double* out) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        out[e] = (double)in[e];
}

// x += a y over n entries
__global__ void axpy_kernel(size_t n, float a, const float* y, float* x) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        x[e] = fmaf(a, y[e], x[e]);
}

// out = (H + H^T) / 2 in FP64, H b x b column-major
template <typename T>
__global__ void symmetrize_kernel(int b, const T* H, double* out) {
    const size_t n = (size_t)b * b;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % b), j = (int)(e / b);
        out[e] = 0.5 * ((double)H[(size_t)i + (size_t)j * b] + (double)H[(size_t)j + (size_t)i * b]);
    }
}

__device__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    if (w == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;  // valid in thread 0
}

// r[j] = |AX_j - theta_j X_j| for the b columns (n rows, column-major); one block per column
template <typename T>
__global__ void residual_kernel(int n, const T* AX, const T* X, const double* theta, double* r) {
    __shared__ double sh[32];
    const int j = blockIdx.x;
    const T* a = AX + (size_t)j * n;
    const T* x = X + (size_t)j * n;
    const double th = theta[j];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double d = (double)a[i] - th * (double)x[i];
        s += d * d;
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) r[j] = sqrt(s);
}

// modes[i] (n entries each) times -1 where its entry of largest magnitude (first on ties) is negative
__global__ void fix_signs_kernel(int n, double* modes) {
    __shared__ double sv[32];
    __shared__ int si[32];
    double* v = modes + (size_t)blockIdx.x * n;
    double best = -1.0, val = 0.0;
    int idx = n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double a = fabs(v[i]);
        if (a > best) best = a, val = v[i], idx = i;  // i ascends per thread: first on ties
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o), ov = __shfl_xor_sync(0xffffffffu, val, o);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
        if (ob > best || (ob == best && oi < idx)) best = ob, val = ov, idx = oi;
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sv[w] = val, si[w] = idx;
    __shared__ double sb[32];
    if (l == 0) sb[w] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); k++)
            if (sb[k] > sb[0] || (sb[k] == sb[0] && si[k] < si[0])) sb[0] = sb[k], sv[0] = sv[k], si[0] = si[k];
    }
    __syncthreads();
    if (sv[0] < 0.0)
        for (int i = threadIdx.x; i < n; i += blockDim.x) v[i] = -v[i];
}

// modes[i][a] = U[(m - 1 - i) n + a], evals[i] = w[m - 1 - i]: the last m columns, descending
__global__ void reverse_kernel(int n, int m, const double* U, const double* w, double* modes, double* evals) {
    const size_t total = (size_t)n * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e / n), a = (int)(e % n);
        modes[e] = U[(size_t)(m - 1 - i) * n + a];
        if (a == 0) evals[i] = w[m - 1 - i];
    }
}

// R_j = AX_j - theta_j X_j, norms[j] = |R_j|; one block per column (FP64)
__global__ void residual_vectors_kernel(int n, const double* AX, const double* X, const double* theta, double* R,
                                        double* norms) {
    __shared__ double sh[32];
    const int j = blockIdx.x;
    const double* a = AX + (size_t)j * n;
    const double* x = X + (size_t)j * n;
    double* r = R + (size_t)j * n;
    const double th = theta[j];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double d = a[i] - th * x[i];
        r[i] = d;
        s += d * d;
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) norms[j] = sqrt(s);
}

// out[j][i] = (float)(in[j][i] / scale[j]) over n x m column-major
__global__ void scaled_narrow_kernel(int n, int m, const double* in, const double* scale, float* out) {
    const size_t total = (size_t)n * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        out[e] = (float)(in[e] / scale[e / n]);
}

// out[j] = A_j . B_j in FP64 (FP32 columns); one block per column
__global__ void col_dot_kernel(int n, const float* A, const float* B, double* out) {
    __shared__ double sh[32];
    const int j = blockIdx.x;
    const float* a = A + (size_t)j * n;
    const float* b = B + (size_t)j * n;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += (double)a[i] * (double)b[i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[j] = s;
}

// Q_j <- theta_j P_j - Q_j   (Q holds S P on entry)
__global__ void shift_sub_kernel(int n, int m, const double* theta, const float* P, float* Q) {
    const size_t total = (size_t)n * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        Q[e] = (float)theta[e / n] * P[e] - Q[e];
}

// D_j += alpha_j P_j, R_j -= alpha_j Q_j
__global__ void cg_step_kernel(int n, int m, const double* alpha, const float* P, const float* Q, float* D, float* R) {
    const size_t total = (size_t)n * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const float a = (float)alpha[e / n];
        D[e] = fmaf(a, P[e], D[e]);
        R[e] = fmaf(-a, Q[e], R[e]);
    }
}

// P_j <- R_j + beta_j P_j
__global__ void cg_direction_kernel(int n, int m, const double* beta, const float* R, float* P) {
    const size_t total = (size_t)n * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        P[e] = fmaf((float)beta[e / n], P[e], R[e]);
}

// X_j = U_j + scale_j D_j (FP64)
__global__ void correct_kernel(int n, int m, const double* U, const double* scale, const float* D, double* X) {
    const size_t total = (size_t)n * m;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        X[e] = U[e] + scale[e / n] * (double)D[e];
}

struct Gemm32 {
    cublasHandle_t h;
    bool emulate;
    // C = alpha op(A) op(B) + beta C, FP32 storage
    void operator()(cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k, float alpha, const float* A,
                    int lda, const float* B, int ldb, float beta, float* C, int ldc) const {
        blas_ok(cublasGemmEx(h, ta, tb, m, n, k, &alpha, A, CUDA_R_32F, lda, B, CUDA_R_32F, ldb, &beta, C, CUDA_R_32F,
                             ldc, emulate ? CUBLAS_COMPUTE_32F_EMULATED_16BFX9 : CUBLAS_COMPUTE_32F,
                             CUBLAS_GEMM_DEFAULT),
                "chfsi GEMM");
    }
};

}  // namespace

void chfsi_eigensolve(const ChfsiArgs& g, cublasHandle_t blas, cusolverDnHandle_t solver, cudaStream_t st,
                      long long* launches, ChfsiStats* stats) {
    const int N = g.N, M = g.M;
    const int B = chfsi::block_size(N, M, g.guard);
    const int Mr = std::min(B, M + 8);  // columns of the FP64 refinement
    if (M < 1 || M > N) fail(OPSEC_ERR_ARG, "iterative eigensolver: Nmodes must be in [1, Ncells]");
    const size_t NN = (size_t)N * N, NB = (size_t)N * B;
    blas_ok(cublasSetStream(blas, st), "cublasSetStream");
    solver_ok(cusolverDnSetStream(solver, st), "cusolverDnSetStream");
    blas_ok(cublasSetPointerMode(blas, CUBLAS_POINTER_MODE_HOST), "cublasSetPointerMode");
    const Gemm32 gemm{blas, g.emulate != 0};
    ChfsiStats s{};

    // ---- spectrum bounds: Lanczos on the FP64 S
    DevBuf<double> lz;
    lz.alloc((size_t)3 * N);
    double *v0 = lz.p, *v1 = lz.p + N, *w = lz.p + 2 * N;
    random_kernel<double><<<blocks(N), 256, 0, st>>>((size_t)N, g.seed ^ 0x4C414E43ULL, v1);
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;
    OPSEC_CUDA(cudaMemsetAsync(v0, 0, sizeof(double) * N, st));
    double nrm = 0.0;
    blas_ok(cublasDnrm2(blas, N, v1, 1, &nrm), "Dnrm2");
    double inv = 1.0 / nrm;
    blas_ok(cublasDscal(blas, N, &inv, v1, 1), "Dscal");
    std::vector<double> al, be;
    double beta = 0.0;
    const int steps = std::min(kLanczos, N);
    if (g_clock) g_clock->begin("chfsi_bounds", st, 2.0 * NN * steps);
    for (int j = 0; j < steps; j++) {
        const double one = 1.0, zero = 0.0;
        blas_ok(cublasDgemv(blas, CUBLAS_OP_N, N, N, &one, g.S, N, v1, 1, &zero, w, 1), "Dgemv");
        double a = 0.0;
        blas_ok(cublasDdot(blas, N, w, 1, v1, 1, &a), "Ddot");
        const double ma = -a, mb = -beta;
        blas_ok(cublasDaxpy(blas, N, &ma, v1, 1, w, 1), "Daxpy");
        blas_ok(cublasDaxpy(blas, N, &mb, v0, 1, w, 1), "Daxpy");
        al.push_back(a);
        blas_ok(cublasDnrm2(blas, N, w, 1, &beta), "Dnrm2");
        if (!(beta > 1e-300) || j + 1 == steps) break;
        be.push_back(beta);
        inv = 1.0 / beta;
        std::swap(v0, v1);
        OPSEC_CUDA(cudaMemcpyAsync(v1, w, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        blas_ok(cublasDscal(blas, N, &inv, v1, 1), "Dscal");
    }
    if (g_clock) g_clock->end(st);
    const double tmin = chfsi::tridiag_eig(al, be, 0), tmax = chfsi::tridiag_eig(al, be, (int)al.size() - 1);
    double hi = tmax + std::fabs(beta);
    const double lo = tmin - 0.02 * (hi - tmin);
    if (!(hi > lo) || !std::isfinite(hi) || !std::isfinite(lo))
        fail(OPSEC_ERR_NUMERIC, "iterative eigensolver: the signal matrix has no spread of eigenvalues (zero or not finite)");
    lz.release();

    // ---- S for the block products (an FP32 copy for cuBLAS, or the FP16 hi/lo split of the
    // FP64 S for the tensor-core kernel) and the block buffers
    DevBuf<float> S32, Xb, Yb, Zb, Hb, Vf;
    TcOperand Stc, Btc;
    DevBuf<int> tc_err;
    if (g.tc) {
        Stc.shape(N, N);
        tc_split(g.S, N, Stc, st, launches);
        tc_err.alloc(1);
        OPSEC_CUDA(cudaMemsetAsync(tc_err.p, 0, sizeof(int), st));
    } else {
        S32.alloc(NN);
        narrow_kernel<<<blocks(NN), 256, 0, st>>>(NN, g.S, S32.p);
        OPSEC_CUDA(cudaGetLastError());
    }
    // C = alpha S X + beta C + gamma D for an N x ncols block X (C, D: N x ncols, leading dimension N)
    auto sprod = [&](int ncols, float alpha, const float* X, float beta, float* C, float gamma, const float* D) {
        if (g.tc) {
            Btc.shape(ncols, N);
            tc_split(X, N, Btc, st, launches);
            tc_gemm(Stc, Btc, alpha, beta, C, N, gamma, D, N, 1, g.tile, tc_err.p, g.wait_cycles, st, launches);
        } else {
            gemm(CUBLAS_OP_N, CUBLAS_OP_N, N, ncols, N, alpha, S32.p, N, X, N, beta, C, N);
            if (gamma != 0.f) {
                axpy_kernel<<<blocks((size_t)N * ncols), 256, 0, st>>>((size_t)N * ncols, gamma, D, C);
                OPSEC_CUDA(cudaGetLastError());
                ++*launches;
            }
        }
    };
    Xb.alloc(NB);
    Yb.alloc(NB);
    Zb.alloc(NB);
    Hb.alloc((size_t)B * B);
    Vf.alloc((size_t)B * B);
    DevBuf<double> Hd, Wd, rd, tau64;
    Hd.alloc((size_t)B * B);
    Wd.alloc(B);
    rd.alloc(B);
    DevBuf<int> info;
    info.alloc(1);
    DevBuf<float> tau;
    tau.alloc(B);
    int lw_qr = 0, lw_og = 0, lw_ev = 0;
    solver_ok(cusolverDnSgeqrf_bufferSize(solver, N, B, Yb.p, N, &lw_qr), "Sgeqrf_bufferSize");
    solver_ok(cusolverDnSorgqr_bufferSize(solver, N, B, B, Yb.p, N, tau.p, &lw_og), "Sorgqr_bufferSize");
    solver_ok(cusolverDnDsyevd_bufferSize(solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, B, Hd.p, B, Wd.p,
                                          &lw_ev),
              "Dsyevd_bufferSize");
    DevBuf<float> wsf;
    wsf.alloc((size_t)std::max(std::max(lw_qr, lw_og), 1));
    DevBuf<double> wsd;
    wsd.alloc((size_t)std::max(lw_ev, 1));
    auto check_info = [&](const char* what) {
        int h = 0, te = 0;
        OPSEC_CUDA(cudaMemcpyAsync(&h, info.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        if (g.tc) OPSEC_CUDA(cudaMemcpyAsync(&te, tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        OPSEC_CUDA(cudaStreamSynchronize(st));
        if (te != 0) fail(OPSEC_ERR_CUDA, "iterative eigensolver: tensor-core GEMM timed out waiting on a pipeline barrier");
        if (h != 0) fail(OPSEC_ERR_NUMERIC, std::string("iterative eigensolver: ") + what + " failed (info " + std::to_string(h) + ")");
    };
    auto orthonormalize = [&](float* Y) {
        solver_ok(cusolverDnSgeqrf(solver, N, B, Y, N, tau.p, wsf.p, lw_qr, info.p), "Sgeqrf");
        solver_ok(cusolverDnSorgqr(solver, N, B, B, Y, N, tau.p, wsf.p, lw_og, info.p), "Sorgqr");
    };
    std::vector<double> theta(B), res(B);
    // Rayleigh-Ritz on the orthonormal Y: X = Y V, Y <- S X, theta and residuals on the host
    auto rayleigh_ritz = [&]() {
        if (g_clock) g_clock->begin("chfsi_rayleigh_ritz", st, 2.0 * NN * B + 2.0 * NB * B * 3);
        sprod(B, 1.f, Yb.p, 0.f, Zb.p, 0.f, nullptr);                                           // Z = S Y
        gemm(CUBLAS_OP_T, CUBLAS_OP_N, B, B, N, 1.f, Yb.p, N, Zb.p, N, 0.f, Hb.p, B);              // H = Y^T Z
        symmetrize_kernel<float><<<blocks((size_t)B * B), 256, 0, st>>>(B, Hb.p, Hd.p);
        OPSEC_CUDA(cudaGetLastError());
        solver_ok(cusolverDnDsyevd(solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, B, Hd.p, B, Wd.p, wsd.p,
                                   lw_ev, info.p),
                  "Dsyevd");
        narrow_kernel<<<blocks((size_t)B * B), 256, 0, st>>>((size_t)B * B, Hd.p, Vf.p);
        OPSEC_CUDA(cudaGetLastError());
        gemm(CUBLAS_OP_N, CUBLAS_OP_N, N, B, B, 1.f, Yb.p, N, Vf.p, B, 0.f, Xb.p, N);              // X = Y V
        gemm(CUBLAS_OP_N, CUBLAS_OP_N, N, B, B, 1.f, Zb.p, N, Vf.p, B, 0.f, Yb.p, N);              // S X = Z V
        residual_kernel<float><<<B, 256, 0, st>>>(N, Yb.p, Xb.p, Wd.p, rd.p);
        OPSEC_CUDA(cudaGetLastError());
        if (g_clock) g_clock->end(st);
        *launches += 4;
        OPSEC_CUDA(cudaMemcpyAsync(theta.data(), Wd.p, sizeof(double) * B, cudaMemcpyDeviceToHost, st));
        OPSEC_CUDA(cudaMemcpyAsync(res.data(), rd.p, sizeof(double) * B, cudaMemcpyDeviceToHost, st));
        check_info("Dsyevd");
        s.gemms += 1;
    };

    // ---- start: a random block, orthonormalised, and its Ritz values
    random_kernel<float><<<blocks(NB), 256, 0, st>>>(NB, g.seed, Yb.p);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 2;
    orthonormalize(Yb.p);
    check_info("Sgeqrf/Sorgqr");
    rayleigh_ritz();

    const double eps32 = 5.96e-8;
    double best = 1e300;
    int stall = 0, it = 0, degree = 1;
    for (; it < g.maxit; it++) {
        hi = std::max(hi, theta[B - 1] * (1.0 + 1e-9));
        const double cut = std::max(theta[0], lo + 1e-3 * (hi - lo));
        const double e = 0.5 * (cut - lo), c0 = 0.5 * (cut + lo);
        degree = chfsi::filter_degree(lo, cut, hi, theta[B - M], g.degree, chfsi::kMaxGain);
        if (g_clock) g_clock->begin("chfsi_filter", st, 2.0 * NN * B * degree);
        // X holds the Ritz vectors.  Y = (S X - c0 X) sigma1 / e
        const double sigma1 = e / (hi - c0);
        double sigma = sigma1;
        sprod(B, (float)(sigma1 / e), Xb.p, 0.f, Yb.p, (float)(-c0 * sigma1 / e), Xb.p);
        float* Xp = Xb.p;
        float* Yp = Yb.p;
        for (int k = 2; k <= degree; k++) {
            const double sn = 1.0 / (2.0 / sigma1 - sigma);
            // X <- (2 sn / e)(S Y - c0 Y) - sigma sn X, then swap so that Y is the newest
            sprod(B, (float)(2.0 * sn / e), Yp, (float)(-sigma * sn), Xp, (float)(-2.0 * sn * c0 / e), Yp);
            std::swap(Xp, Yp);
            sigma = sn;
        }
        if (g_clock) g_clock->end(st);
        s.gemms += degree;
        if (Yp != Yb.p) OPSEC_CUDA(cudaMemcpyAsync(Yb.p, Yp, sizeof(float) * NB, cudaMemcpyDeviceToDevice, st));
        if (g_clock) g_clock->begin("chfsi_qr32", st, 4.0 * NB * B);
        orthonormalize(Yb.p);
        if (g_clock) g_clock->end(st);
        rayleigh_ritz();
        // convergence of the top M: residual below tol theta_i or the FP32 floor
        double worst = 0.0;
        bool done = true;
        const double floor32 = 64.0 * eps32 * hi;
        for (int i = B - M; i < B; i++) {
            const double r = res[i], scale = std::max(std::fabs(theta[i]), 1e-300);
            worst = std::max(worst, r / scale);
            if (r > std::max(g.tol * scale, floor32)) done = false;
        }
        if (done) {
            it++;
            break;
        }
        if (worst < 0.9 * best) {
            best = worst;
            stall = 0;
        } else if (++stall >= 3) {
            it++;
            break;
        }
    }
    s.iterations = it;
    s.degree = degree;
    s.lo = lo;
    s.hi = hi;
    Zb.release();
    Hb.release();
    Vf.release();

    // ---- FP64 refinement of the top Mr Ritz vectors
    const size_t NR = (size_t)N * Mr;
    DevBuf<double> X64, Z64, U64, Hs;
    X64.alloc(NR);
    Z64.alloc(NR);
    U64.alloc(NR);
    Hs.alloc((size_t)Mr * Mr);
    widen_kernel<<<blocks(NR), 256, 0, st>>>(NR, Xb.p + (size_t)(B - Mr) * N, X64.p);
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;
    Xb.release();
    Yb.release();
    // FP32 buffers of the correction solve
    DevBuf<float> U32, R32, P32, Q32, D32, G32;
    U32.alloc(NR);
    R32.alloc(NR);
    P32.alloc(NR);
    Q32.alloc(NR);
    D32.alloc(NR);
    G32.alloc((size_t)Mr * Mr);
    DevBuf<double> colv;  // per-column scalars: theta, scale, alpha, beta
    colv.alloc((size_t)4 * Mr);
    tau64.alloc(Mr);
    int lq = 0, lo2 = 0, le = 0, lc = 0;
    DevBuf<double> G64, Ri64;  // CholeskyQR: the Gram matrix / its Cholesky factor, the factor's inverse
    G64.alloc((size_t)Mr * Mr);
    Ri64.alloc((size_t)Mr * Mr);
    solver_ok(cusolverDnDpotrf_bufferSize(solver, CUBLAS_FILL_MODE_UPPER, Mr, G64.p, Mr, &lc), "Dpotrf_bufferSize");
    solver_ok(cusolverDnDgeqrf_bufferSize(solver, N, Mr, X64.p, N, &lq), "Dgeqrf_bufferSize");
    solver_ok(cusolverDnDorgqr_bufferSize(solver, N, Mr, Mr, X64.p, N, tau64.p, &lo2), "Dorgqr_bufferSize");
    solver_ok(cusolverDnDsyevd_bufferSize(solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, Mr, Hs.p, Mr,
                                          Wd.p, &le),
              "Dsyevd_bufferSize");
    wsd.release();
    wsd.alloc((size_t)std::max(std::max(std::max(lq, lo2), std::max(le, 1)), lc));
    const int lmax = (int)wsd.n;
    std::vector<double> w64(Mr), r64(Mr), hv(4 * (size_t)Mr), pq(Mr), rho(Mr), rho0(Mr);
    const double one = 1.0, zero = 0.0;
    // The FP64-accurate products: double-FP32 on the FP32 pipes (gemm_df.cu; operands split into
    // float pairs first, S once per solve), or cuBLAS DGEMM.  A is K-major (C = A^T B) when at.
    DevBuf<float> dfS, dfA, dfB;
    DevBuf<double> dwork;
    if (g.df64) {
        dfS.alloc(2 * NN);
        df_split(NN, g.S, dfS.p, st, launches);
    }
    auto dprod = [&](bool at, int m, int n, int k, const double* A, int lda, const double* Bm, int ldb, double* Cm,
                     int ldc) {
        if (!g.df64) {
            blas_ok(cublasDgemm(blas, at ? CUBLAS_OP_T : CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &one, A, lda, Bm, ldb, &zero,
                                Cm, ldc),
                    "Dgemm");
            return;
        }
        const float* a = dfS.p;
        if (A != g.S) {
            const size_t na = (size_t)lda * (at ? m : k);
            dfA.alloc(2 * na);
            df_split(na, A, dfA.p, st, launches);
            a = dfA.p;
        }
        const size_t nb = (size_t)ldb * n;
        dfB.alloc(2 * nb);
        df_split(nb, Bm, dfB.p, st, launches);
        df_gemm(at, m, n, k, a, lda, dfB.p, ldb, Cm, ldc, dwork, st, launches);
    };
    const double target = 0.1 * g.tol;  // refine until the residuals are a tenth of the tolerance
    for (int round = 0;; round++) {
        // orthonormal basis Q of the current vectors and Z = S Q.  First pass: Z by a DGEMM with
        // the FP64 S.  Later passes: X = U + D and Z = S U + S D are carried in (S U from the last
        // pass in FP64, S D by an FP32 GEMM: D is small, so FP32 costs it nothing), and X = Q R
        // turns Z into Z R^-1 = S Q by a triangular solve before R is overwritten
        if (g_clock) g_clock->begin("chfsi_qr64", st, 4.0 * NR * Mr);
        bool qr_done = false;
        if (g.cholqr && g.df64) {
            // CholeskyQR2 (Fukaya, Nakatsukasa, Yanagisawa, Yamamoto 2014): twice G = X^T X,
            // G = R^T R (Cholesky), X <- X R^-1 (and Z <- Z R^-1); the products in double-FP32,
            // R^-1 from a triangular solve on the identity.  The refinement's X has nearly
            // orthonormal columns, so the first pass already leaves X orthonormal to ~eps64 cond^2
            // and the second to ~eps64.  A failed factorisation falls back to Householder QR.
            qr_done = true;
            for (int pass = 0; pass < 2 && qr_done; pass++) {
                dprod(true, Mr, Mr, N, X64.p, N, X64.p, N, G64.p, Mr);
                solver_ok(cusolverDnDpotrf(solver, CUBLAS_FILL_MODE_UPPER, Mr, G64.p, Mr, wsd.p, lmax, info.p),
                          "Dpotrf");
                int h = 0;
                OPSEC_CUDA(cudaMemcpyAsync(&h, info.p, sizeof(int), cudaMemcpyDeviceToHost, st));
                OPSEC_CUDA(cudaStreamSynchronize(st));
                if (h != 0) {
                    qr_done = false;
                    break;
                }
                identity_kernel<<<blocks((size_t)Mr * Mr), 256, 0, st>>>(Mr, Ri64.p);
                OPSEC_CUDA(cudaGetLastError());
                ++*launches;
                blas_ok(cublasDtrsm(blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT,
                                    Mr, Mr, &one, G64.p, Mr, Ri64.p, Mr),
                        "Dtrsm");
                dprod(false, N, Mr, Mr, X64.p, N, Ri64.p, Mr, U64.p, N);
                OPSEC_CUDA(cudaMemcpyAsync(X64.p, U64.p, sizeof(double) * NR, cudaMemcpyDeviceToDevice, st));
                if (round > 0) {
                    dprod(false, N, Mr, Mr, Z64.p, N, Ri64.p, Mr, U64.p, N);
                    OPSEC_CUDA(cudaMemcpyAsync(Z64.p, U64.p, sizeof(double) * NR, cudaMemcpyDeviceToDevice, st));
                }
            }
            // a failure in the second pass leaves X and Z transformed consistently by the first:
            // Householder below starts from there
        }
        if (!qr_done) {
            solver_ok(cusolverDnDgeqrf(solver, N, Mr, X64.p, N, tau64.p, wsd.p, lmax, info.p), "Dgeqrf");
            if (round > 0)
                blas_ok(cublasDtrsm(blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, N,
                                    Mr, &one, X64.p, N, Z64.p, N),
                        "Dtrsm");
            solver_ok(cusolverDnDorgqr(solver, N, Mr, Mr, X64.p, N, tau64.p, wsd.p, lmax, info.p), "Dorgqr");
        }
        if (g_clock) g_clock->end(st);
        check_info("Dgeqrf/Dorgqr");
        if (g_clock)
            g_clock->begin("chfsi_refine", st, (round == 0 ? 2.0 * NN * Mr : 2.0 * NR * Mr) + 6.0 * NR * Mr);
        if (round == 0) dprod(true, N, Mr, N, g.S, N, X64.p, N, Z64.p, N);  // Z = S X (S symmetric)
        dprod(true, Mr, Mr, N, X64.p, N, Z64.p, N, U64.p, Mr);              // X^T Z
        symmetrize_kernel<double><<<blocks((size_t)Mr * Mr), 256, 0, st>>>(Mr, U64.p, Hs.p);
        OPSEC_CUDA(cudaGetLastError());
        solver_ok(cusolverDnDsyevd(solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, Mr, Hs.p, Mr, Wd.p, wsd.p,
                                   lmax, info.p),
                  "Dsyevd");
        dprod(false, N, Mr, Mr, X64.p, N, Hs.p, Mr, U64.p, N);  // U = X V
        dprod(false, N, Mr, Mr, Z64.p, N, Hs.p, Mr, X64.p, N);  // S U = Z V
        // X64 = S U kept; Z64 <- S u - theta u (the residual vectors), rd <- their norms
        residual_vectors_kernel<<<Mr, 256, 0, st>>>(N, X64.p, U64.p, Wd.p, Z64.p, rd.p);
        OPSEC_CUDA(cudaGetLastError());
        if (g_clock) g_clock->end(st);
        *launches += 2;
        s.rounds += 1;
        OPSEC_CUDA(cudaMemcpyAsync(w64.data(), Wd.p, sizeof(double) * Mr, cudaMemcpyDeviceToHost, st));
        OPSEC_CUDA(cudaMemcpyAsync(r64.data(), rd.p, sizeof(double) * Mr, cudaMemcpyDeviceToHost, st));
        check_info("Dsyevd");
        s.resid = 0.0;
        for (int i = Mr - M; i < Mr; i++) s.resid = std::max(s.resid, r64[i] / std::max(std::fabs(w64[i]), 1e-300));
        if (s.resid <= target || round >= g.refine) break;

        // correction: for every column j solve (I - P)(theta_j - S)(I - P) d_j = r_j (P = U U^T), which is
        // positive definite on the complement of U, by CG with FP32 GEMMs; then x_j = u_j + d_j
        if (g_clock) g_clock->begin("chfsi_correct", st, 2.0 * NN * Mr * g.cg_steps);
        for (int i = 0; i < Mr; i++) {
            hv[i] = w64[i];
            hv[Mr + i] = r64[i] > 0 ? r64[i] : 1.0;
        }
        OPSEC_CUDA(cudaMemcpyAsync(colv.p, hv.data(), sizeof(double) * 2 * Mr, cudaMemcpyHostToDevice, st));
        narrow_kernel<<<blocks(NR), 256, 0, st>>>(NR, U64.p, U32.p);
        scaled_narrow_kernel<<<blocks(NR), 256, 0, st>>>(N, Mr, Z64.p, colv.p + Mr, R32.p);  // b_j = r_j / |r_j|
        OPSEC_CUDA(cudaGetLastError());
        *launches += 2;
        auto project = [&](float* V) {  // V <- V - U (U^T V)
            gemm(CUBLAS_OP_T, CUBLAS_OP_N, Mr, Mr, N, 1.f, U32.p, N, V, N, 0.f, G32.p, Mr);
            gemm(CUBLAS_OP_N, CUBLAS_OP_N, N, Mr, Mr, -1.f, U32.p, N, G32.p, Mr, 1.f, V, N);
        };
        project(R32.p);
        OPSEC_CUDA(cudaMemsetAsync(D32.p, 0, sizeof(float) * NR, st));
        OPSEC_CUDA(cudaMemcpyAsync(P32.p, R32.p, sizeof(float) * NR, cudaMemcpyDeviceToDevice, st));
        col_dot_kernel<<<Mr, 256, 0, st>>>(N, R32.p, R32.p, rd.p);
        OPSEC_CUDA(cudaGetLastError());
        ++*launches;
        OPSEC_CUDA(cudaMemcpyAsync(rho.data(), rd.p, sizeof(double) * Mr, cudaMemcpyDeviceToHost, st));
        OPSEC_CUDA(cudaStreamSynchronize(st));
        rho0 = rho;
        for (int k = 0; k < g.cg_steps; k++) {
            // Q = (I - P)(theta P - S P)
            sprod(Mr, 1.f, P32.p, 0.f, Q32.p, 0.f, nullptr);
            shift_sub_kernel<<<blocks(NR), 256, 0, st>>>(N, Mr, colv.p, P32.p, Q32.p);
            OPSEC_CUDA(cudaGetLastError());
            project(Q32.p);
            col_dot_kernel<<<Mr, 256, 0, st>>>(N, P32.p, Q32.p, rd.p);
            OPSEC_CUDA(cudaGetLastError());
            OPSEC_CUDA(cudaMemcpyAsync(pq.data(), rd.p, sizeof(double) * Mr, cudaMemcpyDeviceToHost, st));
            OPSEC_CUDA(cudaStreamSynchronize(st));
            for (int i = 0; i < Mr; i++) hv[2 * Mr + i] = pq[i] > 1e-30 * rho0[i] ? rho[i] / pq[i] : 0.0;
            OPSEC_CUDA(cudaMemcpyAsync(colv.p + 2 * Mr, hv.data() + 2 * Mr, sizeof(double) * Mr, cudaMemcpyHostToDevice,
                                       st));
            cg_step_kernel<<<blocks(NR), 256, 0, st>>>(N, Mr, colv.p + 2 * Mr, P32.p, Q32.p, D32.p, R32.p);
            OPSEC_CUDA(cudaGetLastError());
            col_dot_kernel<<<Mr, 256, 0, st>>>(N, R32.p, R32.p, rd.p);
            OPSEC_CUDA(cudaGetLastError());
            std::vector<double> rn(Mr);
            OPSEC_CUDA(cudaMemcpyAsync(rn.data(), rd.p, sizeof(double) * Mr, cudaMemcpyDeviceToHost, st));
            OPSEC_CUDA(cudaStreamSynchronize(st));
            bool all = true;
            for (int i = 0; i < Mr; i++) {
                hv[3 * Mr + i] = rho[i] > 0 ? rn[i] / rho[i] : 0.0;
                if (rn[i] > 1e-8 * rho0[i]) all = false;
                rho[i] = rn[i];
            }
            *launches += 4;
            s.cg_steps += 1;
            if (all) break;
            OPSEC_CUDA(cudaMemcpyAsync(colv.p + 3 * Mr, hv.data() + 3 * Mr, sizeof(double) * Mr, cudaMemcpyHostToDevice,
                                       st));
            cg_direction_kernel<<<blocks(NR), 256, 0, st>>>(N, Mr, colv.p + 3 * Mr, R32.p, P32.p);  // P = R + beta P
            OPSEC_CUDA(cudaGetLastError());
            ++*launches;
        }
        // Z = S U + |r| S d (S d by an FP32 GEMM), then X = U + |r| d
        sprod(Mr, 1.f, D32.p, 0.f, Q32.p, 0.f, nullptr);
        correct_kernel<<<blocks(NR), 256, 0, st>>>(N, Mr, X64.p, colv.p + Mr, Q32.p, Z64.p);
        correct_kernel<<<blocks(NR), 256, 0, st>>>(N, Mr, U64.p, colv.p + Mr, D32.p, X64.p);
        OPSEC_CUDA(cudaGetLastError());
        *launches += 2;
        if (g_clock) g_clock->end(st);
    }
    reverse_kernel<<<blocks((size_t)N * M), 256, 0, st>>>(N, M, U64.p + (size_t)(Mr - M) * N, Wd.p + (Mr - M), g.modes,
                                                          g.evals);
    OPSEC_CUDA(cudaGetLastError());
    fix_signs_kernel<<<M, 256, 0, st>>>(N, g.modes);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 2;
    OPSEC_CUDA(cudaStreamSynchronize(st));
    s.block = B;
    if (stats) *stats = s;
}

}  // namespace opsec
