// fisher.cu -- Fisher matrix, bias and quadratic estimates over the packed
// derivative matrices, then the Nb x Nb estimate epilogue, both on the GPU.
//
// With w_i = 1/(1+lambda_i) and m_ij = 1/2 on the diagonal, 1 off it
// (estimate-mpi.cpp:480-546, one rank):
//   F_pq = sum_k m w_i w_j D_p[k] D_q[k]
//   f_p  = sum_k m w_i w_j D_p[k] R[k],  R[k] = delta_ij (1+lambda_i) - sum_n p_n D_n[k]
//   q_p  = sum_k m w_i w_j D_p[k] y_i y_j
// One pass over the packed triangle reads every D_p[k] once: a CTA stages a
// chunk of k for all bands in shared memory as h_p[k] = sqrt(m w_i w_j) D_p[k]
// (plus the rows R and y_i y_j), each thread owns a few (p,q) outputs, FP32
// products summed over the chunk and FP64 across chunks.  Per-CTA partials
// are reduced in a fixed order, so reruns are bit-identical.
#include <cmath>

#include "engine.h"

namespace opsec {
namespace {

constexpr int kThreads = 512;
constexpr int kChunk = 128;
constexpr int kMaxOut = 8;  // outputs per thread: nb(nb+1)/2 + 2nb <= 4096

__device__ __forceinline__ void unpack(long long k, int* i, int* j) {
    long long jj = (long long)((sqrt(8.0 * (double)k + 1.0) - 1.0) * 0.5);
    while (jj * (jj + 1) / 2 > k) --jj;
    while ((jj + 1) * (jj + 2) / 2 <= k) ++jj;
    *j = (int)jj;
    *i = (int)(k - jj * (jj + 1) / 2);
}

// output o -> (p, q): q in [p, nb) for F, q = nb for f (row R), q = nb+1 for q (row yy)
__device__ __forceinline__ void out_pair(int o, int nb, int* p, int* q) {
    const int nF = nb * (nb + 1) / 2;
    if (o < nF) {
        int pp = 0, rem = o;
        while (rem >= nb - pp) {
            rem -= nb - pp;
            ++pp;
        }
        *p = pp;
        *q = pp + rem;
    } else if (o < nF + nb) {
        *p = o - nF;
        *q = nb;
    } else {
        *p = o - nF - nb;
        *q = nb + 1;
    }
}

template <class T>
__global__ void __launch_bounds__(kThreads) fisher_kernel(int M, int nb, const T* Dp, const double* evals,
                                                          const double* y, const double* prior, double* partial) {
    extern __shared__ float hs[];  // [nb+2][kChunk]
    const long long K = (long long)M * (M + 1) / 2;
    const int nout = nb * (nb + 1) / 2 + 2 * nb;
    int op[kMaxOut], oq[kMaxOut];
    double acc[kMaxOut];
#pragma unroll
    for (int s = 0; s < kMaxOut; s++) {
        int o = threadIdx.x + s * kThreads;
        op[s] = oq[s] = -1;
        acc[s] = 0.0;
        if (o < nout) out_pair(o, nb, &op[s], &oq[s]);
    }
    for (long long k0 = (long long)blockIdx.x * kChunk; k0 < K; k0 += (long long)gridDim.x * kChunk) {
        // stage raw D_p[k]
        for (int e = threadIdx.x; e < nb * kChunk; e += kThreads) {
            int p = e / kChunk, kk = e % kChunk;
            long long k = k0 + kk;
            hs[p * kChunk + kk] = (k < K) ? (float)Dp[(size_t)p * K + k] : 0.f;
        }
        __syncthreads();
        // per-k weights, residual row, data row
        for (int kk = threadIdx.x; kk < kChunk; kk += kThreads) {
            long long k = k0 + kk;
            float sc = 0.f, R = 0.f, yy = 0.f;
            if (k < K) {
                int i, j;
                unpack(k, &i, &j);
                double wi = 1.0 / (1.0 + evals[i]), wj = 1.0 / (1.0 + evals[j]);
                double c = (i == j ? 0.5 : 1.0) * wi * wj;
                sc = (float)sqrt(c);
                double r = (i == j) ? 1.0 + evals[i] : 0.0;
                for (int n = 0; n < nb; n++) r -= prior[n] * (double)hs[n * kChunk + kk];
                R = (float)r;
                yy = (float)(y[i] * y[j]);
            }
            for (int p = 0; p < nb; p++) hs[p * kChunk + kk] *= sc;
            hs[nb * kChunk + kk] = R * sc;
            hs[(nb + 1) * kChunk + kk] = yy * sc;
        }
        __syncthreads();
#pragma unroll
        for (int s = 0; s < kMaxOut; s++) {
            if (op[s] < 0) continue;
            const float* a = hs + op[s] * kChunk;
            const float* b = hs + oq[s] * kChunk;
            float part = 0.f;
#pragma unroll 8
            for (int kk = 0; kk < kChunk; kk++) part = fmaf(a[kk], b[kk], part);
            acc[s] += (double)part;
        }
        __syncthreads();
    }
#pragma unroll
    for (int s = 0; s < kMaxOut; s++) {
        int o = threadIdx.x + s * kThreads;
        if (o < nout) partial[(size_t)blockIdx.x * nout + o] = acc[s];
    }
}

// fixed-order reduction of the per-CTA partials into F (full), f, q
__global__ void fisher_reduce_kernel(int nb, int nblocks, const double* partial, double* out) {
    const int nout = nb * (nb + 1) / 2 + 2 * nb;
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < nout; o += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nblocks; b++) s += partial[(size_t)b * nout + o];
        int p, q;
        out_pair(o, nb, &p, &q);
        if (q < nb) {
            out[p * nb + q] = s;
            out[q * nb + p] = s;
        } else if (q == nb) {
            out[nb * nb + p] = s;       // f
        } else {
            out[nb * nb + nb + p] = s;  // q
        }
    }
}

// ---------------------------------------------------------------- epilogue
// Gauss-Jordan inverse with partial pivoting of an n x n row-major matrix in
// shared memory (A destroyed, X = A^-1).  Returns false if a pivot vanishes.
__device__ bool gj_inverse(int n, double* A, double* X, int* piv_row) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) X[e] = (e / n == e % n) ? 1.0 : 0.0;
    __syncthreads();
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int c = 0; c < n; c++) {
        if (threadIdx.x == 0) {
            int best = c;
            double bv = fabs(A[c * n + c]);
            for (int r = c + 1; r < n; r++)
                if (fabs(A[r * n + c]) > bv) {
                    bv = fabs(A[r * n + c]);
                    best = r;
                }
            *piv_row = best;
            if (!(bv > 0.0) || !isfinite(bv)) bad = 1;
        }
        __syncthreads();
        if (bad) return false;
        const int pr = *piv_row;
        if (pr != c)
            for (int e = threadIdx.x; e < n; e += blockDim.x) {
                double t = A[c * n + e];
                A[c * n + e] = A[pr * n + e];
                A[pr * n + e] = t;
                t = X[c * n + e];
                X[c * n + e] = X[pr * n + e];
                X[pr * n + e] = t;
            }
        __syncthreads();
        const double inv = 1.0 / A[c * n + c];
        __syncthreads();
        for (int e = threadIdx.x; e < n; e += blockDim.x) {
            A[c * n + e] *= inv;
            X[c * n + e] *= inv;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
            int r = e / n, col = e % n;
            if (r == c) continue;
            double f = A[r * n + c];
            if (col != c) A[r * n + col] -= f * A[c * n + col];
            X[r * n + col] -= f * X[c * n + col];
        }
        __syncthreads();
        for (int r = threadIdx.x; r < n; r += blockDim.x)
            if (r != c) A[r * n + c] = 0.0;
        __syncthreads();
    }
    return true;
}

// cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (thread 0);
// A -> diagonal of eigenvalues, V -> eigenvectors as columns
__device__ void jacobi_eig(int n, double* A, double* V) {
    if (threadIdx.x != 0) return;
    for (int e = 0; e < n * n; e++) V[e] = (e / n == e % n) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, diag = 0.0;
        for (int r = 0; r < n; r++)
            for (int c = 0; c < n; c++) {
                if (r != c) off += A[r * n + c] * A[r * n + c];
                else diag += A[r * n + c] * A[r * n + c];
            }
        if (off <= 1e-30 * diag) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                double apq = A[p * n + q];
                if (apq == 0.0) continue;
                double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
}

// C = A B (n x n, row-major) by the block
__device__ void matmul(int n, const double* A, const double* B, double* Cm) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        int r = e / n, c = e % n;
        double s = 0.0;
        for (int k = 0; k < n; k++) s += A[r * n + k] * B[k * n + c];
        Cm[e] = s;
    }
    __syncthreads();
}

// estimate-mpi.cpp:565-611 including MyMatrix multiply()'s storage-order
// behaviour (MyMatrix.hpp:447-456): stored W = (M F)^T, stored Cov = M^T M F,
// stored q record = q - f.
__global__ void epilogue_kernel(int nb, int mixing, const double* Fqf, double* out, int* status) {
    extern __shared__ double sm[];
    double* F = sm;
    double* A = F + nb * nb;
    double* Mx = A + nb * nb;
    double* T = Mx + nb * nb;
    double* V = T + nb * nb;
    double* rs = V + nb * nb;
    __shared__ int piv;
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) F[e] = Fqf[e];
    __syncthreads();
    if (threadIdx.x == 0) *status = 0;
    if (mixing == OPSEC_MIXING_IDENTITY) {
        for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) Mx[e] = (e / nb == e % nb) ? 1.0 : 0.0;
        __syncthreads();
    } else {
        for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) A[e] = F[e];
        __syncthreads();
        if (!gj_inverse(nb, A, Mx, &piv)) {
            if (threadIdx.x == 0) *status = OPSEC_ERR_NUMERIC;
            return;
        }
        if (mixing == OPSEC_MIXING_INVERSE_SQRT) {
            // M = F^{-1/2} = V diag(sqrt w) V^T of F^{-1} (MyMatrix.hpp:479-524)
            for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) A[e] = Mx[e];
            __syncthreads();
            jacobi_eig(nb, A, V);
            __syncthreads();
            for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
                int r = e / nb, c = e % nb;
                double s = 0.0;
                for (int k = 0; k < nb; k++) s += V[r * nb + k] * sqrt(A[k * nb + k]) * V[c * nb + k];
                T[e] = s;
            }
            __syncthreads();
            for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) Mx[e] = T[e];
            __syncthreads();
        }
    }
    // W^T = M F; the stored W is its transpose; normalise rows of the stored W
    matmul(nb, Mx, F, T);
    for (int m = threadIdx.x; m < nb; m += blockDim.x) {
        double s = 0.0;
        for (int n = 0; n < nb; n++) s += T[n * nb + m];  // row m of (M F)^T
        rs[m] = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) Mx[e] /= rs[e / nb];
    __syncthreads();
    matmul(nb, Mx, F, T);  // T = M F
    const double* q = Fqf + nb * nb + nb;
    const double* f = Fqf + nb * nb;
    double* o_phat = out;
    double* o_pcov = o_phat + nb;
    double* o_F = o_pcov + nb * nb;
    double* o_W = o_F + nb * nb;
    double* o_M = o_W + nb * nb;
    double* o_q = o_M + nb * nb;
    double* o_f = o_q + nb;
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
        int r = e / nb, c = e % nb;
        o_W[e] = T[c * nb + r];
        o_F[e] = F[e];
        o_M[e] = Mx[e];
        // Cov = M^T (M F)
        double s = 0.0;
        for (int k = 0; k < nb; k++) s += Mx[k * nb + r] * T[k * nb + c];
        o_pcov[e] = s;
    }
    for (int m = threadIdx.x; m < nb; m += blockDim.x) {
        double s = 0.0;
        for (int n = 0; n < nb; n++) s += Mx[m * nb + n] * (q[n] - f[n]);
        o_phat[m] = s;
        o_q[m] = q[m] - f[m];
        o_f[m] = f[m];
    }
}

}  // namespace

int fisher_blocks(int nmodes) {
    const long long K = (long long)nmodes * (nmodes + 1) / 2;
    long long chunks = (K + kChunk - 1) / kChunk;
    long long b = 152LL * 2;
    if (chunks < b) b = chunks;
    return (int)(b < 1 ? 1 : b);
}

template <class T>
static void run_fisher(const FisherArgs& a, const T* Dp, cudaStream_t s, long long* launches) {
    const int nb = a.nbands;
    const int nout = nb * (nb + 1) / 2 + 2 * nb;
    if (nout > kThreads * kMaxOut) fail(OPSEC_ERR_ARG, "too many bands for the Fisher kernel (max 88)");
    const size_t smem = sizeof(float) * (size_t)(nb + 2) * kChunk;
    auto k = fisher_kernel<T>;
    OPSEC_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem((const void*)k)));
    const double K = (double)a.nmodes * (a.nmodes + 1) / 2;
    if (g_clock) g_clock->begin("fisher", s, 2.0 * K * nout, K * nb * sizeof(T));
    k<<<a.nblocks, kThreads, smem, s>>>(a.nmodes, nb, Dp, a.evals, a.y, a.prior, a.partial);
    OPSEC_CUDA(cudaGetLastError());
    if (g_clock) g_clock->end(s);
    fisher_reduce_kernel<<<(nout + 255) / 256, 256, 0, s>>>(nb, a.nblocks, a.partial, a.out);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 2;
}

void launch_fisher(const FisherArgs& a, cudaStream_t s, long long* launches) { run_fisher(a, a.Dp, s, launches); }

void launch_fisher64(const FisherArgs& a, const double* Dp64, cudaStream_t s, long long* launches) {
    run_fisher(a, Dp64, s, launches);
}

void launch_epilogue(int nb, int mixing, const double* Fqf, double* out, int* status, cudaStream_t s,
                     long long* launches) {
    const size_t smem = sizeof(double) * (5 * (size_t)nb * nb + nb);
    OPSEC_CUDA(cudaFuncSetAttribute(epilogue_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem((const void*)epilogue_kernel)));
    epilogue_kernel<<<1, 256, smem, s>>>(nb, mixing, Fqf, out, status);
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;
}

}  // namespace opsec

// ---------------------------------------------------------------- no-allocation entry point
// Some callers cannot call cudaMalloc: applications whose device memory is all
// owned by their own pool allocator (a pipeline framework that hands out
// buffers and forbids raw allocations), and latency-critical loops where an
// allocation or free could synchronize the device between kernels on the
// caller's stream.  For them the Fisher reduction below allocates nothing:
// inputs and outputs are caller-owned device buffers, and the only scratch --
// the per-CTA partial sums -- lives in one file-scope device array that every
// GPU loading this library keeps until the process exits.
namespace opsec {
namespace {

constexpr int kNoallocBlocks = 152;
constexpr int kNoallocMaxBands = OPSEC_NOALLOC_MAX_BANDS;
constexpr int kNoallocMaxOut = kNoallocMaxBands * (kNoallocMaxBands + 1) / 2 + 2 * kNoallocMaxBands;

// 152 x 2208 doubles = 2.7 MB
static __device__ __align__(256) double g_noalloc_partial[kNoallocBlocks * kNoallocMaxOut];

constexpr int kMaxDevices = 64;
double* g_partial_addr[kMaxDevices] = {nullptr};
bool g_attr_done[kMaxDevices] = {false};

}  // namespace

}  // namespace opsec

extern "C" int opsec_gpu_fisher_noalloc(int nmodes, int nbands, const float* cov_packed, const double* evals,
                                        const double* y, const double* prior, double* out, void* stream) {
    using namespace opsec;
    if (nmodes <= 0 || nbands <= 0 || !cov_packed || !evals || !y || !prior || !out) return OPSEC_ERR_ARG;
    if (nbands > kNoallocMaxBands) return OPSEC_ERR_ARG;  // scratch holds at most 64 bands
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return OPSEC_ERR_CUDA;
    // once per device, with that device current: the device address of the scratch array
    if (!g_partial_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_partial) != cudaSuccess || !p) return OPSEC_ERR_CUDA;
        g_partial_addr[dev] = static_cast<double*>(p);
    }
    const int nb = nbands;
    const int nout = nb * (nb + 1) / 2 + 2 * nb;
    const size_t smem = sizeof(float) * (size_t)(nb + 2) * kChunk;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!g_attr_done[dev]) {
        if (cudaFuncSetAttribute(fisher_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(float) * (size_t)(kNoallocMaxBands + 2) * kChunk)) != cudaSuccess)
            return OPSEC_ERR_CUDA;
        g_attr_done[dev] = true;
    }
    // every CTA writes all nout partials of its slot, so nothing needs clearing
    fisher_kernel<float><<<kNoallocBlocks, kThreads, smem, s>>>(nmodes, nb, cov_packed, evals, y, prior,
                                                                g_partial_addr[dev]);
    fisher_reduce_kernel<<<(nout + 255) / 256, 256, 0, s>>>(nb, kNoallocBlocks, g_partial_addr[dev], out);
    return cudaGetLastError() == cudaSuccess ? OPSEC_OK : OPSEC_ERR_CUDA;
}
