// project_tc.cu -- fused projection C_p = B'^T Q_p B' on the 5th-generation
// tensor cores (tcgen05 + TMEM + TMA), sm_103a.
//
// Per band (comma-scalapack.cpp:228-265; S_p = D Q_p D, B' = D B, D = diag sqrt Nbar):
//
//  step 1  T = Q_p B'  (N x N times N x M).  128x256 output tile per CTA,
//          K = cells in blocks of 64.  The A operand (Q_p tile) is gathered
//          from the symmetry-key table by eight producer warps straight into
//          shared memory in the 128B-swizzled K-major layout, split into FP16
//          hi + lo; S_p is never written to memory.  The B operand (B' hi/lo,
//          mode-major) arrives by TMA.  One thread issues
//          tcgen05.mma kind::f16 (M=128, N=256, K=16) three times per K-slice:
//          Ah*Bh + Ah*Bl + Al*Bh accumulate into one FP32 accumulator in TMEM.
//          The epilogue reads TMEM (tcgen05.ld) and writes T^T split into FP16
//          hi/lo.
//  step 2  C_p = B'^T T, both operands by TMA, only tiles touching the upper
//          triangle; the epilogue writes the packed triangle (k = j(j+1)/2+i).
//
// FP16 operands are scaled by powers of two (exact) so that their largest
// magnitude sits near 2^14; hi + lo then carry ~22 significant bits.
// Every mbarrier wait is bounded: on timeout the kernel raises an error flag
// that the host turns into OPSEC_ERR_CUDA, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"
#include "tcgen05.h"

namespace opsec {
namespace {

constexpr int BM = 128, BN = 256, BK = 64;
constexpr int STAGES = 2;
constexpr uint32_t A_BYTES = BM * BK * 2;  // one FP16 operand tile, 16 KB
constexpr uint32_t B_BYTES = BN * BK * 2;  // 32 KB
constexpr uint32_t STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
constexpr int TMEM_COLS = 512;  // [0,256) accumulator D, [256,512) running sum R

// instruction descriptor: D=F32, A=B=F16, both K-major, M=128, N=256
constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

using namespace tc;

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
    umma_f16(tmem_d, a, b, kIdesc, accumulate);
}
__device__ __forceinline__ void tmem_alloc(uint32_t slot) { tc::tmem_alloc(slot, TMEM_COLS); }
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr) { tc::tmem_dealloc(taddr, TMEM_COLS); }

// The tensor core accumulates FP32 with truncation, so a long K loop biases
// every sum toward zero by ~1 ulp per MMA.  The K loop is therefore cut into
// chunks of `chunk` K-slices: the MMA restarts the accumulator D at each
// chunk, and four drain warps (one per TMEM lane quarter) add D into an FP32
// running sum R (round to nearest) in the other half of TMEM while the MMA
// waits.  The last drain hands the final sums to `store(col_block, v[32])`.
struct ChunkBars {
    uint32_t chunk_done;  // MMA -> drain warps (tcgen05.commit)
    uint32_t drained;     // drain warps -> MMA (4 arrivals)
    long long wait_cycles;
};

template <class Store>
__device__ __forceinline__ void drain_loop(uint32_t tmem, int q, int lane, int nchunks, ChunkBars b,
                                           volatile int* abort_flag, int* err, Store store) {
    const uint32_t lane_base = (uint32_t)(32 * q) << 16;
    for (int c = 0; c < nchunks; c++) {
        if (!mbar_wait(b.chunk_done, c & 1, abort_flag, err, b.wait_cycles)) return;
        tc_fence_after();
        const bool last = (c == nchunks - 1);
        for (int cc = 0; cc < 8; cc++) {
            float v[32];
            tmem_ld32(tmem + lane_base + (uint32_t)(32 * cc), v);
            if (c > 0) {
                float r[32];
                tmem_ld32(tmem + lane_base + 256u + (uint32_t)(32 * cc), r);
#pragma unroll
                for (int t = 0; t < 32; t++) v[t] += r[t];
            }
            if (last)
                store(cc, v);
            else
                tmem_st32(tmem + lane_base + 256u + (uint32_t)(32 * cc), v);
        }
        if (!last) {
            tmem_wait_st();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(b.drained);
        }
    }
}

// MMA issue for one K-slice of 64 (3-term split), restarting D at chunk starts.
// The tensor core rounds each accumulation toward zero, a bias of about half
// an FP32 ulp of |D| per MMA.  The two cross terms (2^-11 of the main term)
// are issued first, while D is small, so only the four main-term MMAs of a
// slice add bias at the scale of the result.
__device__ __forceinline__ void issue_slice(uint32_t tmem, uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl,
                                            bool first_in_chunk) {
#pragma unroll
    for (int kk = 0; kk < BK / 16; kk++) {
        const uint64_t adv = (uint64_t)(kk * 32) >> 4;
        umma(tmem, ah + adv, bl + adv, (!first_in_chunk || kk > 0) ? 1u : 0u);
        umma(tmem, al + adv, bh + adv, 1u);
    }
#pragma unroll
    for (int kk = 0; kk < BK / 16; kk++) {
        const uint64_t adv = (uint64_t)(kk * 32) >> 4;
        umma(tmem, ah + adv, bh + adv, 1u);
    }
}

// Step 1 issues each K-slice as two N = 128 halves into two accumulators, so that one half's
// drain (into its running sum) overlaps the tensor core's work on the other half.
constexpr uint32_t kIdesc128 =
    (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(128 >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void issue_slice_n128(uint32_t tmem, uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl,
                                                 bool first_in_chunk) {
#pragma unroll
    for (int kk = 0; kk < BK / 16; kk++) {
        const uint64_t adv = (uint64_t)(kk * 32) >> 4;
        umma_f16(tmem, ah + adv, bl + adv, kIdesc128, (!first_in_chunk || kk > 0) ? 1u : 0u);
        umma_f16(tmem, al + adv, bh + adv, kIdesc128, 1u);
    }
#pragma unroll
    for (int kk = 0; kk < BK / 16; kk++) {
        const uint64_t adv = (uint64_t)(kk * 32) >> 4;
        umma_f16(tmem, ah + adv, bh + adv, kIdesc128, 1u);
    }
}

__device__ __forceinline__ void split_half(float x, __half& h, __half& l) {
    h = __float2half_rn(x);
    l = __float2half_rn(x - __half2float(h));
}

// 2^s with m * 2^s in [2^13, 2^14): exact power-of-two scaling into the FP16 range
__host__ __device__ __forceinline__ float pow2_scale(float m) {
    if (!(m > 0.f) || !(m < 3.0e38f)) return 1.f;
    int e;
    (void)frexpf(m, &e);  // m = f 2^e, f in [0.5, 1)
    return ldexpf(1.f, 14 - e);
}

// ---------------------------------------------------------------- step 1
struct Step1Params {
    KeySpace ks;
    int N, Npad, Mpad;
    int n_at;                 // a-tiles (Npad / BM)
    const int4* ckey;         // per padded cell: key pieces; .w = 0 for padding
    const uint32_t* Qhl;      // square key table of this band, scaled by 2^sQ, FP16 hi | lo << 16
    float out_scale;          // 2^-(sQ + sB): T in its natural units
    float* Tf;                // [Mpad][Npad] T^T, FP32
    int chunk;                // K-slices per accumulator chunk
    int* err;
    long long wait_cycles;  // bound of every mbarrier wait
    int arcs;                 // > 0: cells in arc order with this many phi cells per arc (a divisor of BK)
};

// Arc-run tables of the spherical gather: when the cells are in arc order (cell = h N3 + f) and
// N3 divides BK (and so BM), the 128 x 64 A tile of a K-slice spans BM/N3 row arcs and BK/N3
// column arcs, and every element is Q(h_a, h_b, |f_a - f_b|): one run of nf consecutive words
// of the square table per arc pair.  Each producer warp loads those runs (at most kArcTab words,
// N3 >= 16) once per slice into its own buffer and expands its rows of the tile from there.
// Entry e = ((ra (BK/N3) + ca) nf + df) of slice k's table is the word of row arc a0/N3 + ra,
// column arc k BK/N3 + ca and offset df (zero past the last arc: padding rows and columns).
constexpr int kArcTab = 288;  // (BM/16) (BK/16) 9 words at N3 = 16, the smallest arc run allowed

__device__ __forceinline__ int arc_table_size(const KeySpace& ks, int n3) { return (BM / n3) * (BK / n3) * ks.nf; }

__device__ __forceinline__ int pair_key(const KeySpace& ks, int4 a, int4 b) {
    if (ks.coordsys == 1) {
        int kx = abs(a.x - b.x), ky = abs(a.y - b.y), kz = abs(a.z - b.z);
        return (kx * ks.N2 + ky) * ks.N3 + kz;
    }
    int df = abs(a.y - b.y);
    if (ks.fold) df = min(df, ks.N3 - df);
    return a.x * ks.H + b.x + df;  // a.x = h_a nf, b.x = h_b nf
}

// warps: 0 TMA, 1 MMA, 2-9 gather producers, 10-11 idle, 12-15 drain + epilogue (lane quarters 0-3)
// N3A: 0 for the key gather, else the phi cells per arc of the arc-run tables (p.arcs), a
// compile-time constant so that the producers' row and column splits are shifts
template <int N3A>
__global__ void __launch_bounds__(512, 1)
    step1_kernel(const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl, Step1Params p) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) unsigned long long bar_full[STAGES], bar_empty[STAGES], bar_chunk[2], bar_drained[2];
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;
    __shared__ int4 rowkey[BM];

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int jt = blockIdx.x / p.n_at, at = blockIdx.x % p.n_at;
    const int a0 = at * BM, j0 = jt * BN;
    const int nk = p.Npad / BK;
    const int chunk = p.chunk > 0 ? p.chunk : 1;
    const int nchunks = (nk + chunk - 1) / chunk;

    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int s = 0; s < STAGES; s++) {
            mbar_init(smem_u32(&bar_full[s]), 1 + 8);
            mbar_init(smem_u32(&bar_empty[s]), 1);
        }
        for (int h = 0; h < 2; h++) {
            mbar_init(smem_u32(&bar_chunk[h]), 1);
            mbar_init(smem_u32(&bar_drained[h]), 4);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < BM) rowkey[threadIdx.x] = p.ckey[a0 + threadIdx.x];
    if (warp == 0) tmem_alloc(smem_u32(&tmem_slot));
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    auto A_hi = [&](int s) { return smem + s * STAGE_BYTES; };
    auto A_lo = [&](int s) { return smem + s * STAGE_BYTES + A_BYTES; };
    auto B_hi = [&](int s) { return smem + s * STAGE_BYTES + 2 * A_BYTES; };
    auto B_lo = [&](int s) { return smem + s * STAGE_BYTES + 2 * A_BYTES + B_BYTES; };

    if (warp == 0) {
        // TMA producer for B' hi/lo
        if (lane == 0) {
            for (int k = 0; k < nk; k++) {
                const int s = k % STAGES, n = k / STAGES;
                if (n > 0 && !mbar_wait(smem_u32(&bar_empty[s]), (n - 1) & 1, &abort_flag, p.err, p.wait_cycles)) break;
                const uint32_t fb = smem_u32(&bar_full[s]);
                mbar_arrive_tx(fb, 2 * B_BYTES);
                tma_load_2d(smem_u32(B_hi(s)), &mBh, fb, k * BK, j0);
                tma_load_2d(smem_u32(B_lo(s)), &mBl, fb, k * BK, j0);
            }
        }
    } else if (warp == 1) {
        // MMA issuer: accumulator halves D0 = columns [0, 128) of TMEM for output columns
        // j0 .. j0 + 127, D1 = [128, 256) for j0 + 128 ..; running sums R0, R1 at [256, 512)
        bool ok = true;
        for (int k = 0; k < nk && ok; k++) {
            const int s = k % STAGES, n = k / STAGES;
            const bool first = (k % chunk) == 0, last = (k % chunk) == chunk - 1 || k == nk - 1;
            if (!mbar_wait(smem_u32(&bar_full[s]), n & 1, &abort_flag, p.err, p.wait_cycles)) break;
            for (int h = 0; h < 2; h++) {
                // this half's previous chunk must be drained before it restarts
                if (first && k > 0 &&
                    !mbar_wait(smem_u32(&bar_drained[h]), ((k / chunk) - 1) & 1, &abort_flag, p.err, p.wait_cycles)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                if (lane == 0) {
                    const uint32_t boff = (uint32_t)h * (128 * 128);  // rows 128 h of the B tiles (8-row atoms of 1 KB)
                    issue_slice_n128(tmem + (uint32_t)(128 * h), sdesc(smem_u32(A_hi(s))), sdesc(smem_u32(A_lo(s))),
                                     sdesc(smem_u32(B_hi(s)) + boff), sdesc(smem_u32(B_lo(s)) + boff), first);
                    if (h == 1) umma_commit(smem_u32(&bar_empty[s]));
                    if (last) umma_commit(smem_u32(&bar_chunk[h]));
                }
                __syncwarp();
            }
        }
    } else if (warp >= 12) {
        // drain warps + epilogue: T^T[j][a] in natural units; per chunk, half 0 then half 1,
        // each drained while the tensor core works on the other
        const int q = warp & 3;
        const int a = a0 + 32 * q + lane;
        const uint32_t lane_base = (uint32_t)(32 * q) << 16;
        bool ok = true;
        for (int c = 0; c < nchunks && ok; c++) {
            const bool last = (c == nchunks - 1);
            for (int h = 0; h < 2; h++) {
                if (!mbar_wait(smem_u32(&bar_chunk[h]), c & 1, &abort_flag, p.err, p.wait_cycles)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t dcol = lane_base + (uint32_t)(128 * h), rcol = lane_base + 256u + (uint32_t)(128 * h);
                for (int cc = 0; cc < 4; cc++) {
                    float v[32];
                    tmem_ld32(tmem + dcol + (uint32_t)(32 * cc), v);
                    if (c > 0) {
                        float r[32];
                        tmem_ld32(tmem + rcol + (uint32_t)(32 * cc), r);
#pragma unroll
                        for (int t = 0; t < 32; t++) v[t] += r[t];
                    }
                    if (last) {
#pragma unroll
                        for (int t = 0; t < 32; t++)
                            p.Tf[(size_t)(j0 + 128 * h + 32 * cc + t) * p.Npad + a] = v[t] * p.out_scale;
                    } else {
                        tmem_st32(tmem + rcol + (uint32_t)(32 * cc), v);
                    }
                }
                if (!last) tmem_wait_st();
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&bar_drained[h]));
            }
        }
    } else if (N3A > 0 && warp < 10) {
        // eight producers expanding arc-run tables: each warp loads slice k+1's table into
        // registers while it expands slice k from its own shared buffer.
        constexpr int n3 = N3A > 0 ? N3A : 1;
        const int pw = warp - 2;
        uint32_t* tab = reinterpret_cast<uint32_t*>(smem + STAGES * STAGE_BYTES) + pw * 2 * kArcTab;  // [2][kArcTab]
        const int T = arc_table_size(p.ks, n3);
        constexpr int kPer = kArcTab / 32;
        constexpr int nca = BK / n3;
        // the table entries' index split, once per lane: entry e of every slice's table is word
        // (ha0 + ra) H nf + (kb + ca) nf + df of the key table, kb = k BK / n3; packed as
        // rel = (ra H + ca) nf + df, ca and whether row arc ha0 + ra exists (the host keeps
        // (BM / n3) H nf below 2^23)
        const int H = p.ks.H, nf = p.ks.nf, ha0 = a0 / n3;
        int packed[kPer];
#pragma unroll
        for (int q = 0; q < kPer; q++) {
            const int e = lane + 32 * q;
            const int df = e % nf, pr = e / nf, ca = pr % nca, ra = pr / nca;
            const int rel = (ra * H + ca) * nf + df;
            packed[q] = e < T && ha0 + ra < H ? (rel << 8) | (ca << 1) | 1 : 0;
        }
        uint32_t nxt[kPer];
        auto load = [&](int k) {
            const int kb = (k * BK) / n3;
            const uint32_t* base = p.Qhl + ((size_t)ha0 * H + kb) * nf;
#pragma unroll
            for (int q = 0; q < kPer; q++) {
                const int pk = packed[q];
                nxt[q] = (pk & 1) && kb + ((pk >> 1) & 127) < H ? __ldg(base + (pk >> 8)) : 0u;
            }
        };
        auto store = [&](int buf) {
#pragma unroll
            for (int q = 0; q < kPer; q++) tab[buf * kArcTab + lane + 32 * q] = nxt[q];
        };
        if (nk > 0) {
            load(0);
            store(0);
        }
        const int c0 = 2 * lane, c1 = c0 + 1;
        const int ca0 = c0 / n3, fb0 = c0 % n3, ca1 = c1 / n3, fb1 = c1 % n3;
        for (int k = 0; k < nk; k++) {
            __syncwarp();  // table k complete in this warp's buffer
            if (k + 1 < nk) load(k + 1);
            const int s = k % STAGES, n = k / STAGES;
            if (n > 0 && !mbar_wait(smem_u32(&bar_empty[s]), (n - 1) & 1, &abort_flag, p.err, p.wait_cycles)) break;
            const uint32_t* tb = tab + (k & 1) * kArcTab;
            unsigned char* ahi = A_hi(s);
            unsigned char* alo = A_lo(s);
#pragma unroll
            for (int i = 0; i < BM / 8; i++) {
                const int r = pw + 8 * i;
                const int ra = r / n3, fa = r % n3;
                int d0 = abs(fa - fb0), d1 = abs(fa - fb1);
                if (p.ks.fold) {
                    d0 = min(d0, n3 - d0);
                    d1 = min(d1, n3 - d1);
                }
                const uint32_t x0 = tb[(ra * nca + ca0) * p.ks.nf + d0];
                const uint32_t x1 = tb[(ra * nca + ca1) * p.ks.nf + d1];
                const uint32_t off = (r >> 3) * 1024 + (r & 7) * 128 + ((((uint32_t)lane >> 2) ^ (r & 7)) << 4) + (lane & 3) * 4;
                *reinterpret_cast<uint32_t*>(ahi + off) = __byte_perm(x0, x1, 0x5410);  // (hi0, hi1)
                *reinterpret_cast<uint32_t*>(alo + off) = __byte_perm(x0, x1, 0x7632);  // (lo0, lo1)
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();  // also: every lane is done reading buffer k & 1 before it is refilled
            if (lane == 0) mbar_arrive(smem_u32(&bar_full[s]));
            if (k + 1 < nk) store((k + 1) & 1);
        }
    } else if (N3A == 0 && warp < 10) {
        // eight gather producers: warp pw fills rows pw, pw+8, ...; lane covers columns 2 lane, 2 lane + 1.
        // Software-pipelined: the 32 gathers of K-slice k+1 are in flight while the warp waits for
        // its stage to drain and while the tensor core works on slice k.
        const int pw = warp - 2;
        uint32_t x0[BM / 8], x1[BM / 8];
        auto gather = [&](int k) {
            const int b = k * BK + 2 * lane;
            const int4 kb0 = p.ckey[b], kb1 = p.ckey[b + 1];
#pragma unroll
            for (int i = 0; i < BM / 8; i++) {
                const int4 ka = rowkey[pw + 8 * i];
                x0[i] = (ka.w && kb0.w) ? __ldg(p.Qhl + pair_key(p.ks, ka, kb0)) : 0u;
                x1[i] = (ka.w && kb1.w) ? __ldg(p.Qhl + pair_key(p.ks, ka, kb1)) : 0u;
            }
        };
        if (nk > 0) gather(0);
        for (int k = 0; k < nk; k++) {
            const int s = k % STAGES, n = k / STAGES;
            if (n > 0 && !mbar_wait(smem_u32(&bar_empty[s]), (n - 1) & 1, &abort_flag, p.err, p.wait_cycles)) break;
            unsigned char* ahi = A_hi(s);
            unsigned char* alo = A_lo(s);
#pragma unroll
            for (int i = 0; i < BM / 8; i++) {
                const int r = pw + 8 * i;
                const uint32_t off = (r >> 3) * 1024 + (r & 7) * 128 + ((((uint32_t)lane >> 2) ^ (r & 7)) << 4) + (lane & 3) * 4;
                *reinterpret_cast<uint32_t*>(ahi + off) = __byte_perm(x0[i], x1[i], 0x5410);  // (hi0, hi1)
                *reinterpret_cast<uint32_t*>(alo + off) = __byte_perm(x0[i], x1[i], 0x7632);  // (lo0, lo1)
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&bar_full[s]));
            if (k + 1 < nk) gather(k + 1);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem);
    }
}

// ---------------------------------------------------------------- step 2
struct Step2Params {
    int M, Npad;
    const int2* tiles;  // (i-tile, j-tile) pairs touching the upper triangle
    float sB;           // scale of B'
    const unsigned* maxT;  // max |T| of this band (float bits); T was scaled by pow2_scale(maxT)
    float* Dp;          // packed output of this band
    int chunk;          // K-slices per accumulator chunk
    int* err;
    long long wait_cycles;  // bound of every mbarrier wait
};

__global__ void __launch_bounds__(256, 1)
    step2_kernel(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
                 const __grid_constant__ CUtensorMap mTh, const __grid_constant__ CUtensorMap mTl, Step2Params p) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) unsigned long long bar_full[STAGES], bar_empty[STAGES], bar_chunk, bar_drained;
    __shared__ uint32_t tmem_slot;
    __shared__ volatile int abort_flag;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int2 tile = p.tiles[blockIdx.x];
    const int i0 = tile.x * BM, j0 = tile.y * BN;
    const int nk = p.Npad / BK;
    const int chunk = p.chunk > 0 ? p.chunk : 1;
    const int nchunks = (nk + chunk - 1) / chunk;

    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int s = 0; s < STAGES; s++) {
            mbar_init(smem_u32(&bar_full[s]), 1);
            mbar_init(smem_u32(&bar_empty[s]), 1);
        }
        mbar_init(smem_u32(&bar_chunk), 1);
        mbar_init(smem_u32(&bar_drained), 4);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(smem_u32(&tmem_slot));
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    auto A_hi = [&](int s) { return smem + s * STAGE_BYTES; };
    auto A_lo = [&](int s) { return smem + s * STAGE_BYTES + A_BYTES; };
    auto B_hi = [&](int s) { return smem + s * STAGE_BYTES + 2 * A_BYTES; };
    auto B_lo = [&](int s) { return smem + s * STAGE_BYTES + 2 * A_BYTES + B_BYTES; };

    if (warp == 0) {
        if (lane == 0) {
            for (int k = 0; k < nk; k++) {
                const int s = k % STAGES, n = k / STAGES;
                if (n > 0 && !mbar_wait(smem_u32(&bar_empty[s]), (n - 1) & 1, &abort_flag, p.err, p.wait_cycles)) break;
                const uint32_t fb = smem_u32(&bar_full[s]);
                mbar_arrive_tx(fb, STAGE_BYTES);
                tma_load_2d(smem_u32(A_hi(s)), &mAh, fb, k * BK, i0);
                tma_load_2d(smem_u32(A_lo(s)), &mAl, fb, k * BK, i0);
                tma_load_2d(smem_u32(B_hi(s)), &mTh, fb, k * BK, j0);
                tma_load_2d(smem_u32(B_lo(s)), &mTl, fb, k * BK, j0);
            }
        }
    } else if (warp == 1) {
        for (int k = 0; k < nk; k++) {
            const int s = k % STAGES, n = k / STAGES;
            const bool first = (k % chunk) == 0;
            if (first && k > 0) {
                if (!mbar_wait(smem_u32(&bar_drained), ((k / chunk) - 1) & 1, &abort_flag, p.err, p.wait_cycles)) break;
            }
            if (!mbar_wait(smem_u32(&bar_full[s]), n & 1, &abort_flag, p.err, p.wait_cycles)) break;
            tc_fence_after();
            if (lane == 0) {
                issue_slice(tmem, sdesc(smem_u32(A_hi(s))), sdesc(smem_u32(A_lo(s))), sdesc(smem_u32(B_hi(s))),
                            sdesc(smem_u32(B_lo(s))), first);
                umma_commit(smem_u32(&bar_empty[s]));
                if ((k % chunk) == chunk - 1 || k == nk - 1) umma_commit(smem_u32(&bar_chunk));
            }
            __syncwarp();
        }
    } else if (warp >= 4) {
        const int q = warp & 3;
        const float out_scale = 1.0f / (p.sB * pow2_scale(__uint_as_float(*p.maxT)));
        const int i = i0 + 32 * q + lane;
        drain_loop(tmem, q, lane, nchunks, ChunkBars{smem_u32(&bar_chunk), smem_u32(&bar_drained), p.wait_cycles}, &abort_flag,
                   p.err, [&](int cc, const float* v) {
#pragma unroll
                       for (int t = 0; t < 32; t++) {
                           const int j = j0 + 32 * cc + t;
                           if (i <= j && j < p.M) p.Dp[(size_t)j * (j + 1) / 2 + i] = v[t] * out_scale;
                       }
                   });
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem);
    }
}

// ---------------------------------------------------------------- helpers
// Self-check of the bounded wait used by the projection kernels: an mbarrier that expects one
// arrival.  arrive = 1: a thread of the second warp arrives after `delay` cycles; arrive = 0:
// nothing arrives and the wait gives up after `limit` cycles, raising *err.  No copy or MMA is
// in flight, so the kernel simply returns either way.
__global__ void wait_probe_kernel(long long limit, int arrive, long long delay, int* err) {
    __shared__ __align__(8) unsigned long long bar;
    __shared__ volatile int abort_flag;
    if (threadIdx.x == 0) {
        abort_flag = 0;
        mbar_init(smem_u32(&bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 32 && arrive) {
        const long long t0 = clock64();
        while (clock64() - t0 < delay) {
        }
        mbar_arrive(smem_u32(&bar));
    }
    if (threadIdx.x == 0) mbar_wait(smem_u32(&bar), 0, &abort_flag, err, limit);
    __syncthreads();
}

__global__ void cell_keys_kernel(KeySpace ks, int N, int Npad, const int* h, const int* f, const int* g, int4* out) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < Npad; a += gridDim.x * blockDim.x) {
        int4 k = make_int4(0, 0, 0, 0);
        if (a < N) {
            if (ks.coordsys == 1)
                k = make_int4(h[a], f[a], g[a], 1);
            else
                k = make_int4(h[a] * ks.nf, f[a], 0, 1);
        }
        out[a] = k;
    }
}

__global__ void absmax_f64_kernel(size_t n, const double* x, unsigned int* out) {
    float m = 0.f;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        m = fmaxf(m, (float)fabs(x[e]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

__global__ void absmax_f32_kernel(int ntab, size_t n, const float* x, unsigned int* out) {
    const int t = blockIdx.y;
    float m = 0.f;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[(size_t)t * n + e]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out + t, __float_as_uint(m));
}

// B'[i][a] (FP64, M x N) * scale -> hi/lo FP16 [Mpad][Npad], zero padded
__global__ void split_modes_kernel(int M, int N, int Mpad, int Npad, const double* Bs, float scale, __half* Bh,
                                   __half* Bl) {
    const size_t total = (size_t)Mpad * Npad;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e / Npad), a = (int)(e % Npad);
        float x = (i < M && a < N) ? (float)(Bs[(size_t)i * N + a] * (double)scale) : 0.f;
        // split from the FP64 value so that lo carries the bits below the FP16 head
        __half h = __float2half_rn(x);
        double rem = (i < M && a < N) ? Bs[(size_t)i * N + a] * (double)scale - (double)__half2float(h) : 0.0;
        Bh[e] = h;
        Bl[e] = __float2half_rn((float)rem);
    }
}

// Q table of one band * 2^sQ -> packed FP16 (hi | lo << 16)
__global__ void split_q_kernel(size_t n, const float* Q, float scale, uint32_t* out) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        __half h, l;
        split_half(Q[e] * scale, h, l);
        out[e] = (uint32_t)__half_as_ushort(h) | ((uint32_t)__half_as_ushort(l) << 16);
    }
}

// T^T (FP32) * pow2_scale(max|T|) -> hi/lo FP16
__global__ void split_t_kernel(size_t n, const float* Tf, const unsigned* maxT, __half* Th, __half* Tl) {
    const float sc = pow2_scale(__uint_as_float(*maxT));
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        __half h, l;
        split_half(Tf[e] * sc, h, l);
        Th[e] = h;
        Tl[e] = l;
    }
}

// 2-D FP16 tensor [rows][cols] (cols contiguous), box = 64 cols x box_rows, 128B swizzle
CUtensorMap make_map(const __half* base, int rows, int cols, int box_rows) {
    CUtensorMap m;
    std::memset(&m, 0, sizeof m);
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * sizeof(__half)};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<__half*>(base), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(OPSEC_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

struct Layout {
    int Npad, Mpad;
    size_t bh, bl, th, tl, tf, qhl, ckey, maxes, tiles, err, total;
};

Layout layout_of(const ProjectArgs& a) {
    Layout L;
    L.Npad = (a.ncells + BM - 1) / BM * BM;
    L.Mpad = (a.nmodes + BN - 1) / BN * BN;
    const size_t half_mat = (size_t)L.Mpad * L.Npad * sizeof(__half);
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t at = o;
        o += (bytes + 1023) / 1024 * 1024;
        return at;
    };
    L.bh = take(half_mat);
    L.bl = take(half_mat);
    L.th = take(half_mat);
    L.tl = take(half_mat);
    L.tf = take(2 * half_mat);
    L.qhl = take(sizeof(uint32_t) * (size_t)a.ks.nsquare);
    L.ckey = take(sizeof(int4) * L.Npad);
    L.maxes = take(sizeof(unsigned) * (1 + 2 * a.nbands));
    const int nti = L.Mpad / BM, ntj = L.Mpad / BN;
    L.tiles = take(sizeof(int2) * (size_t)nti * ntj);
    L.err = take(sizeof(int));
    L.total = o;
    return L;
}

}  // namespace

bool project_tc_supported(const ProjectArgs& a) {
    return a.ncells >= 1 && a.nmodes >= 1 && a.nbands >= 1 && a.ncells < (1 << 28);
}

size_t project_tc_work_bytes(const ProjectArgs& a) { return layout_of(a).total; }

void launch_project_tc(const ProjectArgs& a, cudaStream_t s, long long* launches) {
    const Layout L = layout_of(a);
    if (a.work_bytes < L.total) fail(OPSEC_ERR_ARG, "projection workspace too small");
    unsigned char* w = static_cast<unsigned char*>(a.work);
    __half* Bh = reinterpret_cast<__half*>(w + L.bh);
    __half* Bl = reinterpret_cast<__half*>(w + L.bl);
    __half* Th = reinterpret_cast<__half*>(w + L.th);
    __half* Tl = reinterpret_cast<__half*>(w + L.tl);
    int4* ckey = reinterpret_cast<int4*>(w + L.ckey);
    unsigned* maxes = reinterpret_cast<unsigned*>(w + L.maxes);
    int2* tiles = reinterpret_cast<int2*>(w + L.tiles);
    int* err = reinterpret_cast<int*>(w + L.err);
    float* Tf = reinterpret_cast<float*>(w + L.tf);
    uint32_t* Qhl = reinterpret_cast<uint32_t*>(w + L.qhl);
    const int N = a.ncells, M = a.nmodes, nb = a.nbands;
    unsigned* maxT = maxes + 1 + nb;  // per band

    OPSEC_CUDA(cudaMemsetAsync(maxes, 0, sizeof(unsigned) * (1 + 2 * nb), s));
    OPSEC_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    cell_keys_kernel<<<(L.Npad + 255) / 256, 256, 0, s>>>(a.ks, N, L.Npad, a.cell_h, a.cell_f, a.cell_g, ckey);
    absmax_f64_kernel<<<1024, 256, 0, s>>>((size_t)M * N, a.Bs, maxes);
    absmax_f32_kernel<<<dim3(1024, nb), 256, 0, s>>>(nb, (size_t)a.ks.nsquare, a.Qsq + a.ks.nsquare, maxes + 1);
    OPSEC_CUDA(cudaGetLastError());
    *launches += 3;
    std::vector<unsigned> hm(1 + nb);
    OPSEC_CUDA(cudaMemcpyAsync(hm.data(), maxes, sizeof(unsigned) * (1 + nb), cudaMemcpyDeviceToHost, s));
    OPSEC_CUDA(cudaStreamSynchronize(s));
    auto asf = [](unsigned u) {
        float f;
        std::memcpy(&f, &u, sizeof f);
        return f;
    };
    const float sB = pow2_scale(asf(hm[0]));

    split_modes_kernel<<<2048, 256, 0, s>>>(M, N, L.Mpad, L.Npad, a.Bs, sB, Bh, Bl);
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;

    // tiles (i-tile of 128, j-tile of 256) that hold an element with i <= j
    std::vector<int2> tl;
    for (int tj = 0; tj < L.Mpad / BN; tj++)
        for (int ti = 0; ti < L.Mpad / BM; ti++)
            if (ti * BM <= tj * BN + BN - 1 && ti * BM < M && tj * BN < M) tl.push_back(make_int2(ti, tj));
    OPSEC_CUDA(cudaMemcpyAsync(tiles, tl.data(), sizeof(int2) * tl.size(), cudaMemcpyHostToDevice, s));

    const CUtensorMap mBh256 = make_map(Bh, L.Mpad, L.Npad, BN), mBl256 = make_map(Bl, L.Mpad, L.Npad, BN);
    const CUtensorMap mBh128 = make_map(Bh, L.Mpad, L.Npad, BM), mBl128 = make_map(Bl, L.Mpad, L.Npad, BM);
    const CUtensorMap mTh256 = make_map(Th, L.Mpad, L.Npad, BN), mTl256 = make_map(Tl, L.Mpad, L.Npad, BN);

    const size_t smem = (size_t)STAGES * STAGE_BYTES + 1024 + sizeof(uint32_t) * 8 * 2 * kArcTab;
    OPSEC_CUDA(cudaFuncSetAttribute(step1_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    OPSEC_CUDA(cudaFuncSetAttribute(step1_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    OPSEC_CUDA(cudaFuncSetAttribute(step1_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    OPSEC_CUDA(cudaFuncSetAttribute(step1_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    OPSEC_CUDA(cudaFuncSetAttribute(step2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));

    const int n_at = L.Npad / BM, n_jt = L.Mpad / BN;
    const size_t nT = (size_t)L.Mpad * L.Npad;
    for (int p = 0; p < nb; p++) {
        const float sQ = pow2_scale(asf(hm[1 + p]));
        Step1Params p1;
        p1.ks = a.ks;
        p1.N = N;
        p1.Npad = L.Npad;
        p1.Mpad = L.Mpad;
        p1.n_at = n_at;
        p1.ckey = ckey;
        split_q_kernel<<<2048, 256, 0, s>>>((size_t)a.ks.nsquare, a.Qsq + (size_t)(1 + p) * a.ks.nsquare, sQ, Qhl);
        OPSEC_CUDA(cudaGetLastError());
        p1.Qhl = Qhl;
        p1.out_scale = 1.0f / (sQ * sB);
        p1.Tf = Tf;
        p1.chunk = a.chunk;
        p1.err = err;
        p1.wait_cycles = a.wait_cycles;
        p1.arcs = a.arc_run;
        if (g_clock) g_clock->begin("project_step1", s, 2.0 * N * (double)N * M);
        const unsigned g1 = (unsigned)(n_at * n_jt);
        if (p1.arcs == 16)
            step1_kernel<16><<<g1, 512, smem, s>>>(mBh256, mBl256, p1);
        else if (p1.arcs == 32)
            step1_kernel<32><<<g1, 512, smem, s>>>(mBh256, mBl256, p1);
        else if (p1.arcs == 64)
            step1_kernel<64><<<g1, 512, smem, s>>>(mBh256, mBl256, p1);
        else
            step1_kernel<0><<<g1, 512, smem, s>>>(mBh256, mBl256, p1);
        OPSEC_CUDA(cudaGetLastError());
        if (g_clock) g_clock->end(s);
        absmax_f32_kernel<<<dim3(2048, 1), 256, 0, s>>>(1, nT, Tf, maxT + p);
        split_t_kernel<<<4096, 256, 0, s>>>(nT, Tf, maxT + p, Th, Tl);
        OPSEC_CUDA(cudaGetLastError());
        Step2Params p2;
        p2.M = M;
        p2.Npad = L.Npad;
        p2.tiles = tiles;
        p2.sB = sB;
        p2.maxT = maxT + p;
        p2.chunk = a.chunk;
        p2.Dp = a.Dp + (size_t)p * ((size_t)M * (M + 1) / 2);
        p2.err = err;
        p2.wait_cycles = a.wait_cycles;
        if (g_clock) g_clock->begin("project_step2", s, (double)N * M * (double)(M + 1));
        step2_kernel<<<(unsigned)tl.size(), 256, smem, s>>>(mBh128, mBl128, mTh256, mTl256, p2);
        OPSEC_CUDA(cudaGetLastError());
        if (g_clock) g_clock->end(s);
        *launches += 5;
    }
    int herr = 0;
    OPSEC_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    OPSEC_CUDA(cudaStreamSynchronize(s));
    if (herr) fail(OPSEC_ERR_CUDA, "tensor-core projection timed out waiting on a pipeline barrier");
}

void launch_wait_probe(long long limit, int arrive, long long delay, int* err, cudaStream_t s, long long* launches) {
    wait_probe_kernel<<<1, 64, 0, s>>>(limit, arrive, delay, err);
    OPSEC_CUDA(cudaGetLastError());
    ++*launches;
}

}  // namespace opsec
