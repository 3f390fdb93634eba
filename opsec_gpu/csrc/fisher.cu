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
// (plus the rows R and y_i y_j); the outputs are the upper triangle of the
// Gram matrix of those rows, and each thread owns a 4 x 4 tile of it over a
// slice of the chunk (8 shared loads per 16 FMAs, rows padded to 129 floats so
// that the rows read by one warp sit in different banks).  FP32 products are
// summed over the slice and FP64 across chunks; slices and per-CTA partials
// are reduced in a fixed order, so reruns are bit-identical.
#include <cmath>
#include <mutex>

#include "engine.h"

namespace opsec {
namespace {

constexpr int kChunk = 128;
constexpr int kStride = kChunk + 1;  // padded row: rows a multiple of 32 floats apart fall in different banks
constexpr int kTile = 4;             // each thread owns a 4 x 4 tile of the Gram matrix of the staged rows
constexpr int kMaxThreads = 512;
constexpr int kMaxBands = 88;
constexpr int kFlush = 4;  // chunks summed in FP32 per FP64 update (128 products per slice of 32)

// Staged rows: h_0..h_{nb-1}, then R sc and y_i y_j sc, zero rows up to a
// multiple of 4.  Tiles (I <= J) of 4 rows x 4 rows; the chunk's k range is cut
// into `slices` parts so that ntiles x slices threads share the work.
struct FisherTiling {
    int rows, nt, ntiles, slices, threads;
    size_t smem;
};

__host__ __device__ inline FisherTiling fisher_tiling(int nb) {
    FisherTiling t;
    t.nt = (nb + 2 + kTile - 1) / kTile;
    t.rows = t.nt * kTile;
    t.ntiles = t.nt * (t.nt + 1) / 2;
    t.slices = 1;
    while (t.slices < 32 && t.ntiles * t.slices * 2 <= kMaxThreads) t.slices *= 2;
    t.threads = (t.ntiles * t.slices + 31) / 32 * 32;
    if (t.threads < kChunk) t.threads = kChunk;
    const size_t stage = 2 * sizeof(float) * (size_t)t.rows * kStride;  // two chunk buffers
    const size_t red = sizeof(double) * (size_t)t.ntiles * t.slices * kTile * kTile;
    t.smem = stage > red ? stage : red;
    return t;
}

__device__ __forceinline__ void unpack(long long k, int* i, int* j) {
    long long jj = (long long)((sqrtf((float)(8 * k + 1)) - 1.0f) * 0.5f);
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

// (row, col) of the staged Gram matrix -> output index, or -1
__device__ __forceinline__ int out_index(int row, int col, int nb) {
    if (row > col || row >= nb) return -1;
    const int nF = nb * (nb + 1) / 2;
    if (col < nb) return row * nb - row * (row - 1) / 2 + (col - row);
    if (col == nb) return nF + row;
    if (col == nb + 1) return nF + nb + row;
    return -1;
}

// Where the entries come from.  An entry is one (i <= j) mode pair: its
// indices and the position of its value in each band's array.
//
// Packed: every pair of the packed upper triangle, D_p at p K + k.
template <class T>
struct PackedSource {
    const T* Dp;
    long long K;
    __device__ long long count() const { return K; }
    __device__ void entry(long long k, int* i, int* j, long long* off) const {
        unpack(k, i, j);
        *off = k;
    }
    __device__ float value(int p, long long off) const { return (float)Dp[(size_t)p * K + off]; }
    __device__ const T* addr(int p, long long off) const { return Dp + (size_t)p * K + off; }
};

// Block: only the pairs whose packed value can be nonzero on the azimuthal
// path -- both modes in the same (block, trig class) group -- with the value
// read from the group block's K x K matrix C_b of band p (column j, row i, as
// the scatter into the packed triangle reads it).
struct BlockSource {
    BlockFisherArgs b;
    __device__ long long count() const { return b.g_entry[b.ngroups]; }
    __device__ void entry(long long k, int* i, int* j, long long* off) const {
        int lo = 0, hi = b.ngroups - 1;  // the group holding entry k
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (b.g_entry[mid] <= k) lo = mid;
            else hi = mid - 1;
        }
        int u, v;
        unpack(k - b.g_entry[lo], &u, &v);
        const int* md = b.modes + b.g_mode[lo];
        *i = md[u];
        *j = md[v];
        const int blk = b.g_blk[lo];
        *off = b.off[blk] + (long long)b.mode_col[*j] * b.Km[blk] + b.mode_col[*i];
    }
    __device__ const float* addr(int p, long long off) const { return b.C + (size_t)p * b.csize + off; }
};

// 4-byte asynchronous copy global -> shared (zero-filled when !valid; src must still be a
// valid address then)
__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(valid ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Stage the raw D_p of one chunk: asynchronously for FP32 sources, by plain loads for FP64.
template <class Src>
__device__ __forceinline__ void stage_chunk(const Src& src, int nb, long long k0, long long K, const long long* offs,
                                            float* h) {
    for (int e = threadIdx.x; e < nb * kChunk; e += blockDim.x) {
        const int p = e / kChunk, kk = e % kChunk;
        const bool ok = k0 + kk < K;
        if constexpr (sizeof(*src.addr(0, 0)) == sizeof(float))
            cp_async4(h + p * kStride + kk, ok ? src.addr(p, offs[kk]) : src.addr(0, 0), ok);
        else
            h[p * kStride + kk] = ok ? src.value(p, offs[kk]) : 0.f;
    }
}

template <class Src>
__global__ void __launch_bounds__(kMaxThreads) fisher_kernel(Src src, int nb, const double* evals, const double* y,
                                                             const double* prior, double* partial) {
    extern __shared__ __align__(16) unsigned char fisher_smem[];
    float* hs = reinterpret_cast<float*>(fisher_smem);  // [rows][kStride]
    __shared__ float p_hi[kMaxBands], p_lo[kMaxBands];   // prior p_n = p_hi + p_lo
    __shared__ int s_i[2 * kChunk], s_j[2 * kChunk];    // the entries of the two staged chunks
    __shared__ long long s_off[2 * kChunk];
    const FisherTiling tl = fisher_tiling(nb);
    for (int n = threadIdx.x; n < nb; n += blockDim.x) {
        p_hi[n] = (float)prior[n];
        p_lo[n] = (float)(prior[n] - (double)p_hi[n]);
    }
    const long long K = src.count();
    const int nout = nb * (nb + 1) / 2 + 2 * nb;

    // this thread's tile (I <= J) and k slice
    const int me = threadIdx.x;
    const bool worker = me < tl.ntiles * tl.slices;
    const int tile = worker ? me % tl.ntiles : 0;
    const int slice = worker ? me / tl.ntiles : 0;
    int I = 0, rem = tile;
    while (rem >= tl.nt - I) {
        rem -= tl.nt - I;
        ++I;
    }
    const int J = I + rem;
    const int per = kChunk / tl.slices;
    const float* ra = hs + (size_t)(I * kTile) * kStride + slice * per;
    const float* rb = hs + (size_t)(J * kTile) * kStride + slice * per;
    double acc[kTile][kTile];
    float part[kTile][kTile];  // FP32 over kFlush chunks of this thread's slice, then into acc
    int nsum = 0;
#pragma unroll
    for (int a = 0; a < kTile; a++)
#pragma unroll
        for (int b = 0; b < kTile; b++) {
            acc[a][b] = 0.0;
            part[a][b] = 0.f;
        }

    const size_t buf_floats = (size_t)tl.rows * kStride;
    for (int b = 0; b < 2; b++)
        for (int e = me; e < (tl.rows - nb - 2) * kStride; e += blockDim.x)
            hs[b * buf_floats + (size_t)(nb + 2) * kStride + e] = 0.f;
    auto entries = [&](long long k0, int b) {
        for (int kk = me; kk < kChunk; kk += blockDim.x) {
            const long long k = k0 + kk;
            int i = 0, j = 0;
            long long off = 0;
            if (k < K) src.entry(k, &i, &j, &off);
            s_i[b * kChunk + kk] = i;
            s_j[b * kChunk + kk] = j;
            s_off[b * kChunk + kk] = off;
        }
    };
    // two chunk buffers: the copies of chunk c+1 are in flight while chunk c is weighted and summed
    const long long step = (long long)gridDim.x * kChunk;
    long long k0 = (long long)blockIdx.x * kChunk;
    if (k0 < K) {
        entries(k0, 0);
        __syncthreads();
        stage_chunk(src, nb, k0, K, s_off, hs);
        cp_async_commit();
    }
    for (int it = 0; k0 < K; k0 += step, it++) {
        const int bs = it & 1;  // this chunk's buffer
        const long long k1 = k0 + step;
        if (k1 < K) entries(k1, bs ^ 1);
        __syncthreads();  // entries of chunk k1 visible; chunk it-1 no longer read from buffer b^1
        if (k1 < K) {
            stage_chunk(src, nb, k1, K, s_off + (bs ^ 1) * kChunk, hs + (bs ^ 1) * buf_floats);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();  // chunk k0's copies visible to every thread
        float* const hb = hs + bs * buf_floats;
        const int* const si = s_i + bs * kChunk;
        const int* const sj = s_j + bs * kChunk;
        // per-k weights sqrt(m w_i w_j), residual row R, data row y_i y_j.  R's
        // diagonal is 1 + lambda_i less a sum close to lambda_i, so the sum runs
        // in compensated FP32 (a two-sum per term plus the exact rounding error
        // of each product, about FP64 accuracy) instead of on the FP64 pipe.
        for (int kk = me; kk < kChunk; kk += blockDim.x) {
            const long long k = k0 + kk;
            float sc = 0.f, R = 0.f, yy = 0.f;
            if (k < K) {
                const int i = si[kk], j = sj[kk];
                const float wi = 1.0f / (1.0f + (float)evals[i]), wj = 1.0f / (1.0f + (float)evals[j]);
                sc = sqrtf((i == j ? 0.5f : 1.0f) * wi * wj);
                float rs = 0.f, rc = 0.f;
                if (i == j) {
                    const double d = 1.0 + evals[i];
                    rs = (float)d;
                    rc = (float)(d - (double)rs);
                }
                for (int n = 0; n < nb; n++) {
                    const float dn = hb[n * kStride + kk];
                    const float t = -p_hi[n] * dn;
                    const float te = fmaf(-p_hi[n], dn, -t);  // exact: -p_hi dn = t + te
                    const float u = rs + t;                    // two-sum: rs + t = u + ue
                    const float bb = u - rs;
                    const float ue = (rs - (u - bb)) + (t - bb);
                    rs = u;
                    rc += ue + te - p_lo[n] * dn;
                }
                R = rs + rc;
                yy = (float)(y[i] * y[j]);
            }
            for (int p = 0; p < nb; p++) hb[p * kStride + kk] *= sc;
            hb[nb * kStride + kk] = R * sc;
            hb[(nb + 1) * kStride + kk] = yy * sc;
        }
        __syncthreads();
        if (worker) {
#pragma unroll 4
            for (int kk = 0; kk < per; kk++) {
                float va[kTile], vb[kTile];
#pragma unroll
                for (int a = 0; a < kTile; a++) {
                    va[a] = ra[bs * buf_floats + a * kStride + kk];
                    vb[a] = rb[bs * buf_floats + a * kStride + kk];
                }
#pragma unroll
                for (int a = 0; a < kTile; a++)
#pragma unroll
                    for (int b = 0; b < kTile; b++) part[a][b] = fmaf(va[a], vb[b], part[a][b]);
            }
            if (++nsum == kFlush) {
#pragma unroll
                for (int a = 0; a < kTile; a++)
#pragma unroll
                    for (int b = 0; b < kTile; b++) {
                        acc[a][b] += (double)part[a][b];
                        part[a][b] = 0.f;
                    }
                nsum = 0;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < kTile; a++)
#pragma unroll
        for (int b = 0; b < kTile; b++) acc[a][b] += (double)part[a][b];

    // slices of one tile summed in a fixed order, then one write per output
    double* red = reinterpret_cast<double*>(fisher_smem);  // [ntiles * slices][16]
    if (worker)
#pragma unroll
        for (int a = 0; a < kTile; a++)
#pragma unroll
            for (int b = 0; b < kTile; b++) red[(size_t)me * kTile * kTile + a * kTile + b] = acc[a][b];
    __syncthreads();
    // Every CTA writes all nout outputs of its slot, zeros included when it had no chunk: the
    // no-allocation entry point keeps its partials in a shared array that it never clears.
    if (me < tl.ntiles) {
        for (int e = 0; e < kTile * kTile; e++) {
            const int o = out_index(I * kTile + e / kTile, J * kTile + e % kTile, nb);
            if (o < 0) continue;
            double sum = 0.0;
            for (int sl = 0; sl < tl.slices; sl++) sum += red[(size_t)(sl * tl.ntiles + me) * kTile * kTile + e];
            partial[(size_t)blockIdx.x * nout + o] = sum;
        }
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

int fisher_blocks(int nmodes) { return fisher_blocks_for((long long)nmodes * (nmodes + 1) / 2); }

int fisher_blocks_for(long long K) {
    long long chunks = (K + kChunk - 1) / kChunk;
    long long b = 152LL * 2;
    if (chunks < b) b = chunks;
    return (int)(b < 1 ? 1 : b);
}

template <class Src>
static void run_fisher(const FisherArgs& a, const Src& src, double K, double elem_bytes, cudaStream_t s,
                       long long* launches) {
    const int nb = a.nbands;
    const int nout = nb * (nb + 1) / 2 + 2 * nb;
    if (nb > kMaxBands) fail(OPSEC_ERR_ARG, "too many bands for the Fisher kernel (max 88)");
    const FisherTiling tl = fisher_tiling(nb);
    auto k = fisher_kernel<Src>;
    OPSEC_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic_smem((const void*)k)));
    if (g_clock) g_clock->begin("fisher", s, 2.0 * K * nout, K * nb * elem_bytes);
    k<<<a.nblocks, tl.threads, tl.smem, s>>>(src, nb, a.evals, a.y, a.prior, a.partial);
    OPSEC_CUDA(cudaGetLastError());
    if (g_clock) g_clock->end(s);
    fisher_reduce_kernel<<<(nout + 255) / 256, 256, 0, s>>>(nb, a.nblocks, a.partial, a.out);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 2;
}

void launch_fisher(const FisherArgs& a, cudaStream_t s, long long* launches) {
    const long long K = (long long)a.nmodes * (a.nmodes + 1) / 2;
    run_fisher(a, PackedSource<float>{a.Dp, K}, (double)K, sizeof(float), s, launches);
}

void launch_fisher64(const FisherArgs& a, const double* Dp64, cudaStream_t s, long long* launches) {
    const long long K = (long long)a.nmodes * (a.nmodes + 1) / 2;
    run_fisher(a, PackedSource<double>{Dp64, K}, (double)K, sizeof(double), s, launches);
}

void launch_fisher_blocks(const FisherArgs& a, const BlockFisherArgs& b, long long entries, cudaStream_t s,
                          long long* launches) {
    run_fisher(a, BlockSource{b}, (double)entries, sizeof(float), s, launches);
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
int g_setup_rc[kMaxDevices] = {0};
std::once_flag g_setup_once[kMaxDevices];

// Once per device, with that device current: the device address of the scratch array and the
// kernel's shared-memory limit.  std::call_once makes concurrent first calls from several host
// threads safe; a failed set-up is not retried.
int noalloc_setup(int dev) {
    std::call_once(g_setup_once[dev], [dev] {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_partial) != cudaSuccess || !p) {
            g_setup_rc[dev] = OPSEC_ERR_CUDA;
            return;
        }
        size_t most = 0;  // the largest request of any band count this entry point accepts
        for (int n = 1; n <= kNoallocMaxBands; n++) most = fisher_tiling(n).smem > most ? fisher_tiling(n).smem : most;
        if (cudaFuncSetAttribute(fisher_kernel<PackedSource<float>>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)most) != cudaSuccess) {
            g_setup_rc[dev] = OPSEC_ERR_CUDA;
            return;
        }
        g_partial_addr[dev] = static_cast<double*>(p);
        g_setup_rc[dev] = OPSEC_OK;
    });
    return g_setup_rc[dev];
}

}  // namespace

}  // namespace opsec

extern "C" int opsec_gpu_fisher_noalloc(int nmodes, int nbands, const float* cov_packed, const double* evals,
                                        const double* y, const double* prior, double* out, void* stream) {
    using namespace opsec;
    if (nmodes <= 0 || nbands <= 0 || !cov_packed || !evals || !y || !prior || !out) return OPSEC_ERR_ARG;
    if (nbands > kNoallocMaxBands) return OPSEC_ERR_ARG;  // scratch holds at most 64 bands
    // an error left pending by the caller's own launches is not taken for this call's
    if (cudaPeekAtLastError() != cudaSuccess) return OPSEC_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return OPSEC_ERR_CUDA;
    const int rc = noalloc_setup(dev);
    if (rc != OPSEC_OK) return rc;
    const int nb = nbands;
    const int nout = nb * (nb + 1) / 2 + 2 * nb;
    const FisherTiling tl = fisher_tiling(nb);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long K = (long long)nmodes * (nmodes + 1) / 2;
    const int nblocks = fisher_blocks_for(K) < kNoallocBlocks ? fisher_blocks_for(K) : kNoallocBlocks;
    const PackedSource<float> src{cov_packed, K};
    fisher_kernel<PackedSource<float>><<<nblocks, tl.threads, tl.smem, s>>>(src, nb, evals, y, prior,
                                                                            g_partial_addr[dev]);
    if (cudaGetLastError() != cudaSuccess) return OPSEC_ERR_CUDA;  // the reduction would read stale partials
    fisher_reduce_kernel<<<(nout + 255) / 256, 256, 0, s>>>(nb, nblocks, g_partial_addr[dev], out);
    return cudaGetLastError() == cudaSuccess ? OPSEC_OK : OPSEC_ERR_CUDA;
}
