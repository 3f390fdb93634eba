// az_tc.cu -- the block projection of the azimuthal path on the 5th-generation tensor cores
// (tcgen05 + TMEM + TMA), sm_103a.
//
// On a full-sky grid C_p = B^T S_p B (comma-scalapack.cpp:243-252) is block diagonal: per band p
// and azimuthal block m, T = S_p(m) U_m (H x H times H x K_m) and C_m = U_m^T T (K_m x K_m), U_m
// the block eigenvectors the modes use.  Both products are "TN" (each operand row contiguous
// along K = H): S_p(m) is symmetric, U_m and T are stored column by column.  One persistent
// kernel runs the tiles of every (band, block) problem of one product:
//   - warp 0 loads the FP32 A and B tiles (128 rows x 32 K) by TMA (128-byte swizzle);
//   - warps 2-3 split each loaded tile in place into TF32 hi = round(x) and lo = round(x - hi)
//     (the same swizzled layout: the split is elementwise), fence, and release the stage;
//   - warp 1 (one lane) issues tcgen05.mma kind::tf32 (M = 128, N = 128, K = 8): per K-slice
//     the cross terms hi*lo + lo*hi of all four 8-wide steps and the first main term hi*hi into
//     one TMEM accumulator, then each further main term into a fresh one (four accumulators in
//     rotation);
//   - warps 4-11 add every accumulator into running sums in their registers (round to nearest)
//     and store them at the end of the tile.
// The tensor core truncates its FP32 accumulation toward zero, a bias of about half an ulp of
// |D| per MMA that does not average out over a sum; with one main-term MMA per accumulator the
// bias is half an ulp of an 8-term partial, not of the growing tile sum (measured: Fisher matrix
// at 32k cells 4.5e-7 with four main terms per accumulator).  hi + lo carry 22 significant bits
// of each FP32 operand; the dropped lo*lo term is below 2^-22 of each product.
// Every mbarrier wait is bounded: on timeout the kernel raises an error flag that the host turns
// into OPSEC_ERR_CUDA, frees its TMEM and returns.
#include <cuda.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"
#include "tcgen05.h"

namespace opsec {
namespace {
using namespace tc;

constexpr int AM = 128, AN = 128, AK = 32;          // output tile, K slice (32 FP32 = one 128-byte row)
constexpr int ASTAGES = 3;
constexpr uint32_t TILE_BYTES = AM * AK * 4;         // 16 KB: A and B tiles have the same size
constexpr uint32_t ASTAGE_BYTES = 4 * TILE_BYTES;    // A hi, A lo, B hi, B lo
constexpr uint32_t AZ_TMEM_COLS = 512;               // four accumulators of 128 columns
constexpr int kAcc = 4;
constexpr int kSplitThreads = 64;                    // warps 2-3
constexpr int kDrainWarps = 8;                       // warps 4-11: lane quarter x column half
constexpr int kAzThreads = 32 * (4 + kDrainWarps);
// instruction descriptor: D = F32, A = B = TF32 (format 2), both K-major, M = 128, N = 128
constexpr uint32_t kIdescTf32 =
    (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(AN >> 3) << 17) | ((uint32_t)(AM >> 4) << 24);

struct AzTile {
    int z;      // problem: band (within the batch) * nblk + block
    int i0, j0; // first output row and column
    int pad;
};

struct AzGemmParams {
    int mode;               // 0: T = S U (A: block rows, B: U columns); 1: C = U^T T (A: U columns, B: T columns)
    int H;                  // block order: the K extent
    int nblk;
    int ncol;               // columns of U over all blocks
    int ntiles;
    const AzTile* tiles;
    const int* Km;          // [nblk] columns of block m
    const int* base;        // [nblk] first column of block m in U (and in each band's T)
    const long long* off;   // [nblk] offset of C_m within a band's block outputs
    long long csize;        // floats of all blocks' C_m of one band
    float* out;             // mode 0: T [band][ncol][H]; mode 1: C [band][csize], C_m column-major
    int* err;
    long long wait_cycles;  // bound of every mbarrier wait
};

// x rounded to the 10 explicit mantissa bits TF32 keeps (ties away from zero): a value the
// tensor core reads exactly
__device__ __forceinline__ float round_tf32(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}
// TF32 split of one FP32 value: hi = round(x), lo = round(x - hi) (x - hi is exact in FP32)
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
    hi = round_tf32(x);
    lo = round_tf32(x - hi);
}

// Step kk (8 of K, 32 bytes along the swizzled rows) of a K-slice into accumulator d: at kk = 0
// the cross terms of all four steps, then the main term; otherwise the main term alone, into a
// fresh accumulator
__device__ __forceinline__ void issue_step_tf32(uint32_t d, int kk, uint64_t ah, uint64_t al, uint64_t bh,
                                                uint64_t bl) {
    if (kk == 0) {
#pragma unroll
        for (int k2 = 0; k2 < AK / 8; k2++) {
            const uint64_t adv = (uint64_t)(k2 * 32) >> 4;
            umma_tf32(d, ah + adv, bl + adv, kIdescTf32, k2 > 0 ? 1u : 0u);
            umma_tf32(d, al + adv, bh + adv, kIdescTf32, 1u);
        }
        umma_tf32(d, ah, bh, kIdescTf32, 1u);
    } else {
        const uint64_t adv = (uint64_t)(kk * 32) >> 4;
        umma_tf32(d, ah + adv, bh + adv, kIdescTf32, 0u);
    }
}

__global__ void __launch_bounds__(kAzThreads, 1)
    azgemm_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB, AzGemmParams p) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) unsigned long long bar_full[ASTAGES], bar_split[ASTAGES], bar_empty[ASTAGES];
    __shared__ __align__(8) unsigned long long bar_chunk[kAcc], bar_drained[kAcc];  // per accumulator
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nk = (p.H + AK - 1) / AK;

    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int s = 0; s < ASTAGES; s++) {
            mbar_init(smem_u32(&bar_full[s]), 1);
            mbar_init(smem_u32(&bar_split[s]), kSplitThreads);
            mbar_init(smem_u32(&bar_empty[s]), 1);
        }
        for (int b = 0; b < kAcc; b++) {
            mbar_init(smem_u32(&bar_chunk[b]), 1);
            mbar_init(smem_u32(&bar_drained[b]), kDrainWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), AZ_TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    auto A_hi = [&](int s) { return smem + s * ASTAGE_BYTES; };
    auto A_lo = [&](int s) { return smem + s * ASTAGE_BYTES + TILE_BYTES; };
    auto B_hi = [&](int s) { return smem + s * ASTAGE_BYTES + 2 * TILE_BYTES; };
    auto B_lo = [&](int s) { return smem + s * ASTAGE_BYTES + 3 * TILE_BYTES; };

    if (warp == 0) {
        // TMA producer: the raw FP32 tiles into the hi buffers
        if (lane == 0) {
            long long g = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x) {
                const AzTile tl = p.tiles[t];
                const int band = tl.z / p.nblk, m = tl.z % p.nblk, bm = p.base[m];
                for (int k = 0; k < nk; k++, g++) {
                    const int s = (int)(g % ASTAGES);
                    const long long n = g / ASTAGES;
                    if (n > 0 && !mbar_wait(smem_u32(&bar_empty[s]), (uint32_t)((n - 1) & 1), &abort_flag, p.err,
                                            p.wait_cycles)) {
                        ok = false;
                        break;
                    }
                    const uint32_t fb = smem_u32(&bar_full[s]);
                    mbar_arrive_tx(fb, 2 * TILE_BYTES);
                    if (p.mode == 0) {
                        tma_load_3d(smem_u32(A_hi(s)), &mA, fb, k * AK, tl.i0, tl.z);
                        tma_load_3d(smem_u32(B_hi(s)), &mB, fb, k * AK, bm + tl.j0, 0);
                    } else {
                        tma_load_3d(smem_u32(A_hi(s)), &mA, fb, k * AK, bm + tl.i0, 0);
                        tma_load_3d(smem_u32(B_hi(s)), &mB, fb, k * AK, bm + tl.j0, band);
                    }
                }
            }
        }
    } else if (warp == 1) {
        // MMA issue: four accumulators per K-slice, in rotation over the whole sequence
        long long g = 0, cg = 0;  // K slices and accumulators used so far
        bool ok = true;
        for (int t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x) {
            for (int k = 0; k < nk && ok; k++, g++) {
                const int s = (int)(g % ASTAGES);
                const long long n = g / ASTAGES;
                if (!mbar_wait(smem_u32(&bar_split[s]), (uint32_t)(n & 1), &abort_flag, p.err, p.wait_cycles)) {
                    ok = false;
                    break;
                }
                for (int kk = 0; kk < AK / 8; kk++, cg++) {
                    const int b = (int)(cg % kAcc);
                    // the accumulator's previous use (cg - kAcc) must be drained first
                    if (cg >= kAcc && !mbar_wait(smem_u32(&bar_drained[b]), (uint32_t)(((cg / kAcc) - 1) & 1),
                                                 &abort_flag, p.err, p.wait_cycles)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    if (lane == 0) {
                        issue_step_tf32(tmem + (uint32_t)(b * AN), kk, sdesc(smem_u32(A_hi(s))),
                                        sdesc(smem_u32(A_lo(s))), sdesc(smem_u32(B_hi(s))), sdesc(smem_u32(B_lo(s))));
                        if (kk == AK / 8 - 1) umma_commit(smem_u32(&bar_empty[s]));
                        umma_commit(smem_u32(&bar_chunk[b]));
                    }
                    __syncwarp();
                }
            }
        }
    } else if (warp == 2 || warp == 3) {
        // TF32 split of each landed stage, in place
        const int st = threadIdx.x - 64;
        long long g = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x) {
            for (int k = 0; k < nk; k++, g++) {
                const int s = (int)(g % ASTAGES);
                const long long n = g / ASTAGES;
                if (!mbar_wait(smem_u32(&bar_full[s]), (uint32_t)(n & 1), &abort_flag, p.err, p.wait_cycles)) {
                    ok = false;
                    break;
                }
                float4* ah = reinterpret_cast<float4*>(A_hi(s));
                float4* al = reinterpret_cast<float4*>(A_lo(s));
                float4* bh = reinterpret_cast<float4*>(B_hi(s));
                float4* bl = reinterpret_cast<float4*>(B_lo(s));
                for (int i = st; i < (int)(TILE_BYTES / 16); i += kSplitThreads) {
                    float4 x = ah[i], h, l;
                    split_tf32(x.x, h.x, l.x);
                    split_tf32(x.y, h.y, l.y);
                    split_tf32(x.z, h.z, l.z);
                    split_tf32(x.w, h.w, l.w);
                    ah[i] = h;
                    al[i] = l;
                    x = bh[i];
                    split_tf32(x.x, h.x, l.x);
                    split_tf32(x.y, h.y, l.y);
                    split_tf32(x.z, h.z, l.z);
                    split_tf32(x.w, h.w, l.w);
                    bh[i] = h;
                    bl[i] = l;
                }
                // the generic-proxy writes become visible to the tensor core's async proxy
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(smem_u32(&bar_split[s]));
            }
        }
    } else if (warp >= 4) {
        // accumulator drain: TMEM lane quarter q holds output rows i0 + 32 q + lane; this warp
        // sums columns [64 hh, 64 hh + 64) of every accumulator into R and stores them per tile
        const int q = warp & 3, hh = (warp - 4) >> 2;
        const uint32_t lane_base = ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * hh);
        long long cg = 0;
        bool ok = true;
        for (int t = blockIdx.x; t < p.ntiles && ok; t += gridDim.x) {
            const AzTile tl = p.tiles[t];
            const int band = tl.z / p.nblk, m = tl.z % p.nblk;
            const int K = p.Km[m], bm = p.base[m];
            const int i = tl.i0 + 32 * q + lane;
            float R[64];
#pragma unroll
            for (int u = 0; u < 64; u++) R[u] = 0.f;
            for (int c = 0; c < nk * (AK / 8); c++, cg++) {
                const int b = (int)(cg % kAcc);
                if (!mbar_wait(smem_u32(&bar_chunk[b]), (uint32_t)((cg / kAcc) & 1), &abort_flag, p.err,
                               p.wait_cycles)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                {
                    float v[64];
                    tmem_ld64(tmem + lane_base + (uint32_t)(b * AN), v);
#pragma unroll
                    for (int u = 0; u < 64; u++) R[u] += v[u];
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&bar_drained[b]));  // the accumulator may be reused
            }
            if (!ok) break;
            const int j0 = tl.j0 + 64 * hh;
            if (p.mode == 0) {
                // T column j of block m, band `band`: [band][bm + j][i], rows i < H
                if (i < p.H) {
                    float* o = p.out + ((size_t)band * p.ncol + bm) * p.H + i;
#pragma unroll
                    for (int u = 0; u < 64; u++)
                        if (j0 + u < K) o[(size_t)(j0 + u) * p.H] = R[u];
                }
            } else if (i < K) {
                float* o = p.out + (size_t)band * p.csize + p.off[m] + i;
#pragma unroll
                for (int u = 0; u < 64; u++)
                    if (j0 + u < K) o[(size_t)(j0 + u) * K] = R[u];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, AZ_TMEM_COLS);
    }
}

// 3-D FP32 tensor [d2][d1][d0] (d0 contiguous, row stride d0, slice stride d0 d1), box 32 x 128 x 1,
// 128-byte swizzle
CUtensorMap make_map3(const float* base, int d0, int d1, int d2) {
    CUtensorMap m;
    std::memset(&m, 0, sizeof m);
    cuuint64_t dims[3] = {(cuuint64_t)d0, (cuuint64_t)d1, (cuuint64_t)d2};
    cuuint64_t strides[2] = {(cuuint64_t)d0 * sizeof(float), (cuuint64_t)d0 * d1 * sizeof(float)};
    cuuint32_t box[3] = {(cuuint32_t)AK, (cuuint32_t)AM, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(OPSEC_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

}  // namespace

bool az_tc_supported(int H) { return H >= AK && H % 4 == 0; }

size_t az_tc_smem() { return (size_t)ASTAGES * ASTAGE_BYTES + 1024; }

// The two products of the block projection for `np` bands: S [np][nblk][H][H], U [ncol][H] (block
// m's columns from base[m]), T scratch [np][ncol][H], C out [np][csize].  Tiles, block tables and
// the error word live in `work` (az_tc_work_bytes); Km, base, off are device copies of the host
// tables kmh, baseh.
size_t az_tc_work_bytes(int nblk, int np, const std::vector<int>& kmh, int H) {
    size_t n0 = 0, n1 = 0;
    for (int m = 0; m < nblk; m++) {
        const size_t kt = (size_t)(kmh[m] + AN - 1) / AN;
        n0 += kt * (size_t)((H + AM - 1) / AM);
        n1 += kt * kt;
    }
    return sizeof(AzTile) * (n0 + n1) * (size_t)np + 256;
}

void launch_az_tc(int H, int nblk, int ncol, int np, const float* S, const float* U, float* T, float* C,
                  long long csize, const int* Km, const int* base, const long long* off, const std::vector<int>& kmh,
                  void* work, size_t work_bytes, int* err, long long wait_cycles, cudaStream_t s,
                  long long* launches) {
    if (!az_tc_supported(H)) fail(OPSEC_ERR_ARG, "tensor-core block projection: block order must be a multiple of 4");
    std::vector<AzTile> t0, t1;
    for (int b = 0; b < np; b++)
        for (int m = 0; m < nblk; m++) {
            const int K = kmh[m];
            if (K == 0) continue;
            const int z = b * nblk + m;
            for (int i0 = 0; i0 < H; i0 += AM)
                for (int j0 = 0; j0 < K; j0 += AN) t0.push_back(AzTile{z, i0, j0, 0});
            for (int i0 = 0; i0 < K; i0 += AM)
                for (int j0 = 0; j0 < K; j0 += AN) t1.push_back(AzTile{z, i0, j0, 0});
        }
    if (t0.empty()) return;
    if (sizeof(AzTile) * (t0.size() + t1.size()) > work_bytes) fail(OPSEC_ERR_ARG, "tensor-core block projection: scratch");
    AzTile* d0 = static_cast<AzTile*>(work);
    AzTile* d1 = d0 + t0.size();
    OPSEC_CUDA(cudaMemcpyAsync(d0, t0.data(), sizeof(AzTile) * t0.size(), cudaMemcpyHostToDevice, s));
    OPSEC_CUDA(cudaMemcpyAsync(d1, t1.data(), sizeof(AzTile) * t1.size(), cudaMemcpyHostToDevice, s));
    const CUtensorMap mS = make_map3(S, H, H, np * nblk);
    const CUtensorMap mU = make_map3(U, H, ncol, 1);
    const CUtensorMap mT = make_map3(T, H, ncol, np);
    const size_t smem = az_tc_smem();
    OPSEC_CUDA(cudaFuncSetAttribute(azgemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, nsm = 0;
    OPSEC_CUDA(cudaGetDevice(&dev));
    OPSEC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    AzGemmParams p{};
    p.H = H;
    p.nblk = nblk;
    p.ncol = ncol;
    p.Km = Km;
    p.base = base;
    p.off = off;
    p.csize = csize;
    p.err = err;
    p.wait_cycles = wait_cycles;
    // T = S U
    p.mode = 0;
    p.ntiles = (int)t0.size();
    p.tiles = d0;
    p.out = T;
    azgemm_kernel<<<(unsigned)std::min<size_t>(t0.size(), (size_t)nsm), kAzThreads, smem, s>>>(mS, mU, p);
    OPSEC_CUDA(cudaGetLastError());
    // C = U^T T
    p.mode = 1;
    p.ntiles = (int)t1.size();
    p.tiles = d1;
    p.out = C;
    azgemm_kernel<<<(unsigned)std::min<size_t>(t1.size(), (size_t)nsm), kAzThreads, smem, s>>>(mU, mT, p);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 2;
}

}  // namespace opsec
