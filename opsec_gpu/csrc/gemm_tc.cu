// gemm_tc.cu -- products of the dense signal matrix with blocks of vectors on the 5th-generation
// tensor cores (tcgen05 + TMEM + TMA), sm_103a: the Chebyshev filter, Rayleigh-Ritz and
// correction-solve GEMMs of the iterative eigensolver (chfsi.cu).
//
// The reference multiplies S by one vector at a time inside ARPACK's Lanczos iteration
// (ParpackSolver.cpp:111-123, the matrix-vector product of klt.cpp:173-248).  Here
//   C[i + j ldc] = alpha sum_k A[i][k] B[j][k] + beta C[i + j ldc] + gamma D[i + j ldd]
// with A = S (symmetric: row i is column i, contiguous along k) and B the block's columns, both
// "K-major".  Each operand is split once into FP16 hi + lo after an exact power-of-two scaling
// that puts its largest magnitude in [2^13, 2^14) (tc_split); hi + lo carry ~22 significant
// bits and the tensor core forms Ah Bh + Ah Bl + Al Bh (the dropped Al Bl is ~2^-22 of each
// product).  One CTA per 128 x 256 output tile:
//   - warp 0 loads A (128 rows) and B (256 rows) hi/lo slices of 64 along K by TMA (128-byte
//     swizzle), two stages (three for 128-column tiles);
//   - warp 1 (one lane) issues tcgen05.mma kind::f16 M = 128, N = 128, K = 16 for the two
//     halves of the 256 columns into two TMEM accumulators, the cross terms of a slice first
//     (while the accumulator is small);
//   (tiles of 128 columns, one half, when they fill the SMs' waves better: a 640-column block
//   of a 13,824-row S makes 324 tiles of 256 columns, 2.1 waves of 152, or 540 of 128, 3.6);
//   - warps 4-11 add each half's accumulator into its FP32 running sum in TMEM (round to
//     nearest) after every `chunk` slices while the tensor core works on the other half, and
//     write the tile from the running sums at the end, with the scale, alpha, beta and gamma.
// The tensor core truncates its FP32 accumulation toward zero; restarting the accumulator per
// chunk keeps that bias at the scale of one slice's partial sum.  Every mbarrier wait is
// bounded: on timeout the kernel raises an error word (read by the caller), frees its TMEM and
// returns.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "engine.h"
#include "gemm_tc.h"
#include "tcgen05.h"

namespace opsec {
namespace {
using namespace tc;

constexpr int GM = 128, GN = 256, GK = 64;  // output tile (GN: the widest), K slice (64 FP16 = one 128-byte row)
constexpr uint32_t GA_BYTES = GM * GK * 2;  // 16 KB
// NH halves of 128 columns per tile: B tiles of 128 NH rows; as many stages as fit in shared
// memory (three of 64 KB for 128-column tiles, two of 96 KB for 256-column ones)
template <int NH>
struct TileShape {
    static constexpr int N = 128 * NH;
    static constexpr uint32_t B_BYTES = N * GK * 2;
    static constexpr uint32_t STAGE_BYTES = 2 * GA_BYTES + 2 * B_BYTES;
    static constexpr int STAGES = NH == 1 ? 3 : 2;
    static constexpr size_t SMEM = (size_t)STAGES * STAGE_BYTES + 1024;
};
constexpr int kMaxStages = 3;
constexpr uint32_t G_TMEM_COLS = 512;  // D0, D1 (128 each), R0, R1
constexpr int kDrain = 8;              // warps 4-11: TMEM lane quarter x column half of a half
constexpr int kGThreads = 32 * (4 + kDrain);
// instruction descriptor: D = F32, A = B = F16, both K-major, M = 128, N = 128
constexpr uint32_t kIdescH =
    (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(128 >> 3) << 17) | ((uint32_t)(GM >> 4) << 24);

// 2^s with m 2^s in [2^13, 2^14)
__host__ __device__ __forceinline__ float scale_of(float m) {
    if (!(m > 0.f) || !(m < 3.0e38f)) return 1.f;
    int e;
    (void)frexpf(m, &e);
    return ldexpf(1.f, 14 - e);
}

struct GemmParams {
    int ntj;                 // column tiles
    int nk;                  // K slices
    int nrows, ncols;        // output extent
    int chunk;               // K slices per accumulator restart
    float alpha, beta, gamma;
    const unsigned* maxA;    // scales of the operands (float bits of their max |x|)
    const unsigned* maxB;
    float* C;
    long long ldc;
    const float* D;
    long long ldd;
    int* err;
    long long wait_cycles;
};

// one K-slice of one 128-column half: cross terms first, then the main term
__device__ __forceinline__ void issue_half(uint32_t d, uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl,
                                           bool restart) {
#pragma unroll
    for (int kk = 0; kk < GK / 16; kk++) {
        const uint64_t adv = (uint64_t)(kk * 32) >> 4;
        umma_f16(d, ah + adv, bl + adv, kIdescH, (!restart || kk > 0) ? 1u : 0u);
        umma_f16(d, al + adv, bh + adv, kIdescH, 1u);
    }
#pragma unroll
    for (int kk = 0; kk < GK / 16; kk++) {
        const uint64_t adv = (uint64_t)(kk * 32) >> 4;
        umma_f16(d, ah + adv, bh + adv, kIdescH, 1u);
    }
}

template <int NH>
__global__ void __launch_bounds__(kGThreads, 1)
    tn_gemm_kernel(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
                   const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl, GemmParams p) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    constexpr int GSTAGES = TileShape<NH>::STAGES;
    __shared__ __align__(8) unsigned long long bar_full[kMaxStages], bar_empty[kMaxStages], bar_chunk[2], bar_drained[2];
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr uint32_t GB_BYTES = TileShape<NH>::B_BYTES, GSTAGE_BYTES = TileShape<NH>::STAGE_BYTES;
    const int i0 = (blockIdx.x / p.ntj) * GM, j0 = (blockIdx.x % p.ntj) * TileShape<NH>::N;
    const int nk = p.nk;
    const int chunk = p.chunk > 0 ? p.chunk : 1;
    const int nchunks = (nk + chunk - 1) / chunk;

    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int s = 0; s < GSTAGES; s++) {
            mbar_init(smem_u32(&bar_full[s]), 1);
            mbar_init(smem_u32(&bar_empty[s]), 1);
        }
        for (int h = 0; h < 2; h++) {
            mbar_init(smem_u32(&bar_chunk[h]), 1);
            mbar_init(smem_u32(&bar_drained[h]), kDrain);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), G_TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    auto A_hi = [&](int s) { return smem + s * GSTAGE_BYTES; };
    auto A_lo = [&](int s) { return smem + s * GSTAGE_BYTES + GA_BYTES; };
    auto B_hi = [&](int s) { return smem + s * GSTAGE_BYTES + 2 * GA_BYTES; };
    auto B_lo = [&](int s) { return smem + s * GSTAGE_BYTES + 2 * GA_BYTES + GB_BYTES; };

    if (warp == 0) {
        if (lane == 0) {
            for (int k = 0; k < nk; k++) {
                const int s = k % GSTAGES, n = k / GSTAGES;
                if (n > 0 && !mbar_wait(smem_u32(&bar_empty[s]), (n - 1) & 1, &abort_flag, p.err, p.wait_cycles)) break;
                const uint32_t fb = smem_u32(&bar_full[s]);
                mbar_arrive_tx(fb, GSTAGE_BYTES);
                tma_load_2d(smem_u32(A_hi(s)), &mAh, fb, k * GK, i0);
                tma_load_2d(smem_u32(A_lo(s)), &mAl, fb, k * GK, i0);
                tma_load_2d(smem_u32(B_hi(s)), &mBh, fb, k * GK, j0);
                tma_load_2d(smem_u32(B_lo(s)), &mBl, fb, k * GK, j0);
            }
        }
    } else if (warp == 1) {
        bool ok = true;
        for (int k = 0; k < nk && ok; k++) {
            const int s = k % GSTAGES, n = k / GSTAGES;
            const bool first = (k % chunk) == 0, last = (k % chunk) == chunk - 1 || k == nk - 1;
            if (!mbar_wait(smem_u32(&bar_full[s]), n & 1, &abort_flag, p.err, p.wait_cycles)) break;
            for (int h = 0; h < NH; h++) {
                // this half's previous chunk must be drained before its accumulator restarts
                if (first && k > 0 &&
                    !mbar_wait(smem_u32(&bar_drained[h]), ((k / chunk) - 1) & 1, &abort_flag, p.err, p.wait_cycles)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                if (lane == 0) {
                    const uint32_t boff = (uint32_t)h * (128 * 128);  // B rows 128 h: 16 atoms of 8 rows x 128 B
                    issue_half(tmem + (uint32_t)(128 * h), sdesc(smem_u32(A_hi(s))), sdesc(smem_u32(A_lo(s))),
                               sdesc(smem_u32(B_hi(s)) + boff), sdesc(smem_u32(B_lo(s)) + boff), first);
                    if (h == NH - 1) umma_commit(smem_u32(&bar_empty[s]));
                    if (last) umma_commit(smem_u32(&bar_chunk[h]));
                }
                __syncwarp();
            }
        }
    } else if (warp >= 4) {
        // TMEM lane quarter q holds output rows i0 + 32 q + lane; this warp takes columns
        // [64 part, 64 part + 64) of each half
        const int q = warp & 3, part = (warp - 4) >> 2;
        const int i = i0 + 32 * q + lane;
        const uint32_t lane_base = (uint32_t)(32 * q) << 16;
        const float sc = p.alpha / (scale_of(__uint_as_float(*p.maxA)) * scale_of(__uint_as_float(*p.maxB)));
        bool ok = true;
        for (int c = 0; c < nchunks && ok; c++) {
            const bool last = (c == nchunks - 1);
            for (int h = 0; h < NH; h++) {
                if (!mbar_wait(smem_u32(&bar_chunk[h]), c & 1, &abort_flag, p.err, p.wait_cycles)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t col = (uint32_t)(128 * h + 64 * part);
                for (int cc = 0; cc < 2; cc++) {
                    float v[32];
                    tmem_ld32(tmem + lane_base + col + (uint32_t)(32 * cc), v);
                    if (c > 0) {
                        float r[32];
                        tmem_ld32(tmem + lane_base + 256u + col + (uint32_t)(32 * cc), r);
#pragma unroll
                        for (int t = 0; t < 32; t++) v[t] += r[t];
                    }
                    if (!last) {
                        tmem_st32(tmem + lane_base + 256u + col + (uint32_t)(32 * cc), v);
                    } else if (i < p.nrows) {
                        const int jb = j0 + (int)col + 32 * cc;
#pragma unroll
                        for (int t = 0; t < 32; t++) {
                            const int j = jb + t;
                            if (j < p.ncols) {
                                float o = v[t] * sc;
                                if (p.beta != 0.f) o = fmaf(p.beta, p.C[(size_t)j * p.ldc + i], o);
                                if (p.gamma != 0.f) o = fmaf(p.gamma, p.D[(size_t)j * p.ldd + i], o);
                                p.C[(size_t)j * p.ldc + i] = o;
                            }
                        }
                    }
                }
                if (!last) tmem_wait_st();
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&bar_drained[h]));
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, G_TMEM_COLS);
    }
}

__device__ __forceinline__ void split_h(float x, __half& h, __half& l) {
    h = __float2half_rn(x);
    l = __float2half_rn(x - __half2float(h));
}

__global__ void absmax_f64_rows_kernel(int rows, int k, long long ld, const double* x, unsigned* out) {
    float m = 0.f;
    const size_t total = (size_t)rows * k;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        m = fmaxf(m, (float)fabs(x[(e / k) * ld + e % k]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

__global__ void absmax_f32_rows_kernel(int rows, int k, long long ld, const float* x, unsigned* out) {
    float m = 0.f;
    const size_t total = (size_t)rows * k;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[(e / k) * ld + e % k]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// row r < rows_pad, k < kpad of the operand: x[r ld + k] scaled, zero outside rows x k; the split
// of an FP64 value takes lo from the FP64 remainder
template <class T>
__global__ void split_rows_kernel(int rows, int k, long long ld, int rows_pad, int kpad, const T* x,
                                  const unsigned* maxbits, __half* hi, __half* lo) {
    const float sc = scale_of(__uint_as_float(*maxbits));
    const size_t total = (size_t)rows_pad * kpad;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e / kpad), c = (int)(e % kpad);
        __half h = __float2half_rn(0.f), l = h;
        if (r < rows && c < k) {
            const T v = x[(size_t)r * ld + c];
            if (sizeof(T) == 8) {
                const double xs = (double)v * (double)sc;
                h = __float2half_rn((float)xs);
                l = __float2half_rn((float)(xs - (double)__half2float(h)));
            } else {
                split_h((float)v * sc, h, l);
            }
        }
        hi[e] = h;
        lo[e] = l;
    }
}

// 2-D FP16 tensor [rows][kpad], box 64 x box_rows, 128-byte swizzle; rows beyond the tensor read as 0
CUtensorMap make_map(const __half* base, int rows, int kpad, int box_rows) {
    CUtensorMap m;
    std::memset(&m, 0, sizeof m);
    cuuint64_t dims[2] = {(cuuint64_t)kpad, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)kpad * sizeof(__half)};
    cuuint32_t box[2] = {(cuuint32_t)GK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<__half*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(OPSEC_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

int grid_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 4096); }

}  // namespace

void TcOperand::shape(int rows_, int k_) {
    rows = rows_;
    k = k_;
    rows_pad = (rows_ + GN - 1) / GN * GN;  // whole 256-row boxes: no TMA box crosses the end
    kpad = (k_ + GK - 1) / GK * GK;
    store.alloc(4 * elems() + 256);
}

template <class T>
static void split_any(const T* x, long long ld, TcOperand& op, cudaStream_t s, long long* launches) {
    if (op.rows < 1 || op.k < 1) return;
    __half* hi = static_cast<__half*>(op.hi());
    __half* lo = static_cast<__half*>(op.lo());
    OPSEC_CUDA(cudaMemsetAsync(op.maxbits(), 0, sizeof(unsigned), s));
    const size_t n = (size_t)op.rows * op.k;
    if (sizeof(T) == 8)
        absmax_f64_rows_kernel<<<grid_for(n), 256, 0, s>>>(op.rows, op.k, ld, reinterpret_cast<const double*>(x),
                                                           op.maxbits());
    else
        absmax_f32_rows_kernel<<<grid_for(n), 256, 0, s>>>(op.rows, op.k, ld, reinterpret_cast<const float*>(x),
                                                           op.maxbits());
    split_rows_kernel<T><<<grid_for((size_t)op.rows_pad * op.kpad), 256, 0, s>>>(
        op.rows, op.k, ld, op.rows_pad, op.kpad, x, op.maxbits(), hi, lo);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 2;
}

void tc_split(const double* x, long long ld, TcOperand& op, cudaStream_t s, long long* launches) {
    split_any<double>(x, ld, op, s, launches);
}
void tc_split(const float* x, long long ld, TcOperand& op, cudaStream_t s, long long* launches) {
    split_any<float>(x, ld, op, s, launches);
}

void tc_gemm(const TcOperand& A, const TcOperand& B, float alpha, float beta, float* C, long long ldc, float gamma,
             const float* D, long long ldd, int chunk, int tile_cols, int* err, long long wait_cycles, cudaStream_t s,
             long long* launches) {
    if (A.kpad != B.kpad || A.k != B.k) fail(OPSEC_ERR_ARG, "tensor-core GEMM: operands differ in K");
    if (A.rows < 1 || B.rows < 1) return;
    // tile width: 256 columns (two halves) unless 128-column tiles fill the SMs' waves better
    // (cost ~ waves x (column halves + a half for the A slices every tile loads)); tile_cols
    // 128 or 256 fixes it
    int dev = 0, nsm = 0;
    OPSEC_CUDA(cudaGetDevice(&dev));
    OPSEC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const long long nti = (A.rows + GM - 1) / GM;
    auto cost = [&](int nh) {
        const long long tiles = nti * ((B.rows + 128 * nh - 1) / (128 * nh));
        return (double)((tiles + nsm - 1) / nsm) * (nh + 0.5);
    };
    const int NH = tile_cols == 128 ? 1 : tile_cols == 256 ? 2 : cost(1) < cost(2) ? 1 : 2;
    auto h = [](void* p) { return static_cast<const __half*>(p); };
    const CUtensorMap mAh = make_map(h(A.hi()), A.rows_pad, A.kpad, GM), mAl = make_map(h(A.lo()), A.rows_pad, A.kpad, GM);
    const CUtensorMap mBh = make_map(h(B.hi()), B.rows_pad, B.kpad, 128 * NH);
    const CUtensorMap mBl = make_map(h(B.lo()), B.rows_pad, B.kpad, 128 * NH);
    const size_t smem = NH == 1 ? TileShape<1>::SMEM : TileShape<2>::SMEM;
    GemmParams p;
    p.ntj = (B.rows + 128 * NH - 1) / (128 * NH);
    p.nk = A.kpad / GK;
    p.nrows = A.rows;
    p.ncols = B.rows;
    p.chunk = chunk;
    p.alpha = alpha;
    p.beta = beta;
    p.gamma = gamma;
    p.maxA = A.maxbits();
    p.maxB = B.maxbits();
    p.C = C;
    p.ldc = ldc;
    p.D = D;
    p.ldd = ldd;
    p.err = err;
    p.wait_cycles = wait_cycles;
    const unsigned grid = (unsigned)(nti * p.ntj);
    if (NH == 1) {
        OPSEC_CUDA(cudaFuncSetAttribute(tn_gemm_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        tn_gemm_kernel<1><<<grid, kGThreads, smem, s>>>(mAh, mAl, mBh, mBl, p);
    } else {
        OPSEC_CUDA(cudaFuncSetAttribute(tn_gemm_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        tn_gemm_kernel<2><<<grid, kGThreads, smem, s>>>(mAh, mAl, mBh, mBl, p);
    }
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;
}

}  // namespace opsec
