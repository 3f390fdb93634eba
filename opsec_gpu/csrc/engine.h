// engine.h -- internal declarations shared by the host code and the kernels.
#pragma once

#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/opsec_gpu.h"

#ifdef __CUDACC__
#define OPSEC_HD __host__ __device__
#else
#define OPSEC_HD
#endif

namespace opsec {

// Internal error carrier; the C ABI turns it into a status code + message.
struct Error {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg);
// Largest dynamic shared-memory size a launch of `func` may request on the current device
// (the opt-in ceiling less the kernel's static shared memory).  Kernels whose launches need
// different amounts set their attribute to this one value, so that host threads launching
// them concurrently never lower it under one another.
int max_dynamic_smem(const void* func);
void cuda_check(cudaError_t e, const char* what);
#define OPSEC_CUDA(x) ::opsec::cuda_check((x), #x)

// Survey grid geometry: the fields of the reference Survey (Survey.h:56-72).
struct Geometry {
    int coordsys = 0;   // 1 Cartesian, 2 spherical (Cell.h:58-62)
    double b[6] = {0};  // Min1, Max1, Min2, Max2, Min3, Max3
    int n[3] = {0};     // N1, N2, N3
    double L = 0;       // periodic box size; 0 = open box
    bool full_sky() const;
    bool mu_symmetric() const;  // spherical mu range symmetric about 0 (reflection z -> -z maps the grid to itself)
};

// r grid of the xi tables: n1 linear points on [0, r1), n2 log points on [r1, r2]
// (QSpline::MakeArray, QSpline.cpp:6-17).
struct XiLayout {
    int n1 = 512, n2 = 256;
    double r1 = 200, r2 = 20000;
    OPSEC_HD int n() const { return n1 + n2; }
};

// Device buffer owned by the context.
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    void alloc(size_t count);
    void release();
    ~DevBuf() { release(); }
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
};

// Symmetry-key space of the cached cell-pair integrals (sig.cpp:99-119,150-207).
struct KeySpace {
    int coordsys = 0;
    int N1 = 0, N2 = 0, N3 = 0;
    int H = 0;        // spherical: arcs (Nr*Nmu)
    int nf = 0;       // spherical: phi offsets kept (Nphi, or Nphi/2+1 folded)
    bool fold = false;
    bool mu_reflect = false;  // spherical: mu grid symmetric about 0, Q(h_a,h_b,df) = Q(P h_a,P h_b,df)
    long long nkeys = 0;     // keys integrated by the cubature kernel
    long long nsquare = 0;   // entries of the expanded table read by the projection
};

// Optional per-kernel timing: CUDA events around selected launches on the
// launching stream, accumulated per kernel name.
struct KernelClock {
    bool on = false;
    struct Rec {
        const char* name;
        cudaEvent_t a, b;
        double flops, bytes;
    };
    std::vector<Rec> pending;
    std::vector<size_t> open;  // begun, not yet ended (brackets nest)
    void begin(const char* name, cudaStream_t s, double flops = 0, double bytes = 0);
    void end(cudaStream_t s);
};
extern thread_local KernelClock* g_clock;  // set by the context around its calls
// Host-side fault injection: when >= 0, the device allocation after that many more fails as if
// cudaMalloc had (set by the context around its calls; -1 = off).
extern thread_local long long* g_fail_alloc;

// ------------------------------------------------------------- kernels
struct CubatureArgs {
    int coordsys;
    double L;            // periodic box (Cartesian), 0 = open
    KeySpace ks;
    int ng, np;          // Gauss points per axis, per cell (ng^3)
    const double* w;     // [ng] Gauss weights on [0,1]
    double wmax = 1.0;   // the largest of them (host copy)
    const double* node1; // [N1][ng]: x (Cartesian) or r (spherical) nodes
    const double* node2; // [N2][ng]: y or mu nodes
    const double* snode2;// [N2][ng]: sqrt(1-mu^2) (spherical)
    const double* node3; // [N3][ng]: z nodes (Cartesian)
    const double* cphi;  // [N3][ng]: cos(phi) nodes (spherical)
    const double* sphi;  // [N3][ng]: sin(phi) nodes (spherical)
    XiLayout xl;
    int ntab;            // tables in the whole set
    const float* tab32;  // [ntab][xl.n()]
    double* Q;           // [ntab][ks.nkeys]
    float4* pts;         // [N1 N2 N3][np][2]: point table (hi: x y z w, lo: x y z 0), filled here
    int exact = 1;       // FP32-pair separations and table index (1) or plain FP32 (0)
    int window = 1;      // exact mode: per-key bin-window histograms for the far keys (1) or table groups only (0)
    int win_key = 384;   // widest key window (bins) on the window path
    int win_flush = 8;   // Cartesian window kernel: second-cell points per loop chunk (0: all)
    int win_dot64 = 0;   // window dot products in FP64 (1) or FP32 chunks of 8 bins added in FP64 (0)
    int win_logkeys = 1;  // spherical window kernel: one-pass keys in the log section of the table take
                          // the specialised loop (1) or the general one (0); the results are the same bits
    int win_keyorder = 1;  // far keys integrated in key order (1) or by window start (0); same results
    void* work = nullptr;  // cubature_work_bytes() of scratch for the window path
    size_t work_bytes = 0;
    // list mode (set internally): integrate the keys list[0 .. *list_count) only
    const int* list = nullptr;
    const int* list_count = nullptr;
    const unsigned char* skip = nullptr;  // keys already filled (by the surrogate): not integrated
};
// float4s of the point table for a key space and ng
size_t cubature_point_count(const KeySpace& ks, int ng);
// scratch bytes for the window path
size_t cubature_work_bytes(const KeySpace& ks, int nx, int ntab, int ng);
void launch_cubature(const CubatureArgs& a, cudaStream_t s, long long* launches);

struct XiTableArgs {
    XiLayout xl;
    int nbands;
    const double* band_lo;  // [nbands]
    const double* band_hi;
    int npk;
    const double* pk_x;     // cubic spline of P(k): x, y, b, c, d
    const double *pk_y, *pk_b, *pk_c, *pk_d;
    double* r;              // [n] out
    double* xi64;           // [1+nbands][n] out
    float* xi32;            // [1+nbands][n] out
    double* scratch;        // >= 3 (32769 + nbands*8193) doubles: Simpson weights, weights / k, and
                            // weights / k as (hi, lo) float pairs
};
void launch_xi_tables(const XiTableArgs& a, cudaStream_t s, long long* launches);

// Expand Q[t][key] into the square table Qsq[t][(ha*H+hb)*nf + df] (spherical)
// or copy (Cartesian), FP32, for the projection gather.
void launch_expand_q(const KeySpace& ks, int ntab, const double* Q, float* Qsq, cudaStream_t s, long long* launches);

// S_ab = sqrt(Nbar_a Nbar_b) Q[key(a,b)] for an explicit row/col block (FP64).
struct CellKeyInfo {
    const int* d1;
    const int* d2;
    const int* d3;
    const double* nbar;
};
void launch_signal_block(const KeySpace& ks, const CellKeyInfo& ci, const double* Qtab, int nrows, const int* rows,
                         int ncols, const int* cols, double* s, int lld, cudaStream_t st, long long* launches);

// Azimuthal blocks of a full-sky S: Sm[m][ha][hb] = D_ha D_hb sum_df Q(ha,hb,df) cos(2 pi m df/Nphi)
// npar = 2 splits each order into its mu-even and mu-odd blocks (half size); block b = m npar + parity
void launch_azimuthal_blocks(const KeySpace& ks, const double* Qtab, const double* nbar_arc, int nm, int npar,
                             double* Sm, cudaStream_t st, long long* launches);
void launch_azimuthal_blocks(const KeySpace& ks, const double* Qtab, const double* nbar_arc, int nm, int npar,
                             float* Sm, cudaStream_t st, long long* launches, bool tiled = true);
// Block eigenvector columns (m, idx) gathered into Ucat[col][h]
void launch_gather_block_vectors(int H, int ncol, const int* col_m, const int* col_idx, const double* U, double* Ucat,
                                 cudaStream_t st, long long* launches);
void launch_gather_block_vectors(int H, int ncol, const int* col_m, const int* col_idx, const double* U, float* Ucat,
                                 cudaStream_t st, long long* launches);
// Packed FP32 C_p of every band from per-block products C[p][blk_off[m] + col_i + col_j K_m]
void launch_azimuthal_scatter(int M, int nbands, const int* mode_m, const int* mode_cls, const int* mode_col,
                              const long long* blk_off, const int* blk_K, long long csize, const double* C, float* Dp,
                              cudaStream_t st, long long* launches);
void launch_azimuthal_scatter(int M, int nbands, const int* mode_m, const int* mode_cls, const int* mode_col,
                              const long long* blk_off, const int* blk_K, long long csize, const float* C, float* Dp,
                              cudaStream_t st, long long* launches);
// The block projection on the tensor cores (az_tc.cu): T = S_p(m) U_m and C_m = U_m^T T for np
// bands, 3-term TF32 products.  S [np][nblk][H][H], U [ncol][H], T scratch [np][ncol][H], C
// [np][csize]; Km, base, off device tables (kmh: Km on the host); work: az_tc_work_bytes; err: a
// device word raised when a bounded wait gives up.
bool az_tc_supported(int H);
size_t az_tc_work_bytes(int nblk, int np, const std::vector<int>& kmh, int H);
void launch_az_tc(int H, int nblk, int ncol, int np, const float* S, const float* U, float* T, float* C,
                  long long csize, const int* Km, const int* base, const long long* off, const std::vector<int>& kmh,
                  void* work, size_t work_bytes, int* err, long long wait_cycles, cudaStream_t s,
                  long long* launches);
// Modes from block eigenvectors: B[mode][h*Nphi + f] = U_m[h][idx] * trig(m f)
void launch_assemble_modes(int H, int Nphi, int Nmu, int npar, int nmodes, const int* sel_b, const int* sel_idx,
                           const int* sel_kind, const double* U, double* modes, cudaStream_t st, long long* launches);

// Hand-written batched symmetric eigensolver of equal-size blocks (blockeig.cu): Householder
// tridiagonalisation (column-major blocks, lower triangle; the blocks are overwritten), every
// eigenvalue to ~1e-6 of the block scale, then FP64 eigenpairs of the top kc[b] of each block
// written as columns n-1-c of out (ascending order, as LAPACK's syevd).
bool blockeig_supported(int n);
void launch_blockeig_tridiag(int n, int nblk, double* A, double* V, double* tau, double* dg, double* eg,
                             cudaStream_t s, long long* launches);
void launch_blockeig_spectrum(int n, int nblk, const double* dg, const double* eg, double* w, double* scale,
                              cudaStream_t s, long long* launches);
struct BlockEigVectors {
    int n, nblk, ktot;
    const int* kc;        // [nblk] candidates per block
    const int* koff;      // [nblk] prefix sums of kc
    const double* dg;     // [nblk][n] diagonal of T
    const double* eg;     // [nblk][n] off-diagonal of T
    const double* scale;  // [nblk] power-of-two scale
    double* w;            // [nblk][n] eigenvalues, ascending (candidates refined in place)
    double *Z, *L, *U, *G;  // [n][ktot] each
    int* status;          // [nblk], zeroed by the caller
    const double* V;      // [nblk][n][n] reflectors
    const double* tau;    // [nblk][n]
    double* out;          // [nblk][n][n] eigenvector columns
};
void launch_blockeig_vectors(const BlockEigVectors& p, cudaStream_t s, long long* launches);

// Projection C_p = B'^T Q_p B' for all bands; B' = diag(sqrt Nbar) B.
struct ProjectArgs {
    KeySpace ks;
    int ncells, nmodes, nbands;
    const int* cell_h;     // spherical arc index h of each cell, or Cartesian dx
    const int* cell_f;     // spherical phi index, or Cartesian dy
    const int* cell_g;     // Cartesian dz (unused for spherical)
    const float* Qsq;      // [ntab][nsquare], band p at table 1+p
    const double* Bs;      // [nmodes][ncells] scaled modes B' (mode-major), FP64
    float* Dp;             // [nbands][M(M+1)/2] packed output
    void* work;            // scratch
    size_t work_bytes;
    int chunk = 1;         // tensor-core path: K-slices of 64 per FP32 accumulator chunk
    long long wait_cycles = 2000000000LL;  // bound of every mbarrier wait (~1 s at 2 GHz)
    int arc_run = 0;       // spherical cells in arc order (cell = h N3 + f): N3 when it is 16, 32 or 64
};
size_t project_work_bytes(const ProjectArgs& a);
// The projection kernels' bounded mbarrier wait on a barrier that nothing (arrive = 0) or one
// thread after `delay` cycles (arrive = 1) completes; *err (device) is raised on a timeout.
void launch_wait_probe(long long limit, int arrive, long long delay, int* err, cudaStream_t s, long long* launches);
void launch_project(const ProjectArgs& a, cudaStream_t s, long long* launches);

// ------------------------------------------------------------- learned far-field surrogate
constexpr int kSurrIn = 16;      // 12 features, zero-padded to one 16-wide MMA step
constexpr int kSurrHid = 128;
constexpr int kSurrKeyStride = 10;  // per key: 8 geometry features, d, far flag
// FP32 layout of one network: W1[128][16] b1 W2[128][128] b2 W3[128][128] b3 w4[128] b4 (padded)
constexpr int kSurrOffW1 = 0, kSurrOffB1 = 2048, kSurrOffW2 = 2176, kSurrOffB2 = 18560, kSurrOffW3 = 18688,
              kSurrOffB3 = 35072, kSurrOffW4 = 35200, kSurrOffB4 = 35328, kSurrParams = 35336;
struct SurrGrid {
    double b[6];  // survey bounds
    double d[3];  // cell spacing per axis
};
void launch_surr_key_geometry(const KeySpace& ks, const SurrGrid& g, float far_widths, float* kg, cudaStream_t s,
                              long long* launches);
void launch_surr_far_list(const KeySpace& ks, const float* kg, long long* list, int* count, cudaStream_t s,
                          long long* launches);
void launch_surr_samples(long long nsamp, const long long* keys, int ntab, const float* kg, const float4* tinfo,
                         const XiLayout& xl, const double* xi64, const double* env, const double* Q, long long nkeys,
                         float* feat, float* y, cudaStream_t s, long long* launches);
// fused BF16 tensor-core forward of one member over samples (keys x tables, or explicit features)
void launch_surr_infer(long long nsamp, const long long* keys, int ntab, const float* kg, const float4* tinfo,
                       const float* feat, const float* w, float* out, cudaStream_t s, long long* launches);
void launch_surr_combine(long long nlist, const long long* keys, int ntab, int nmem, const float* pred,
                         const float* kg, const XiLayout& xl, const double* xi64, const double* env, float ysc,
                         float tol, long long nkeys, double* Q, unsigned char* done, int* counts, cudaStream_t s,
                         long long* launches);
// training: forward (+ backward when y != null) over one batch; scratch 7 Bn 128 floats
void surr_forward_backward(int Bn, const float* x, const float* y, const float* wb, float* grad, double* loss,
                           float* out, float* scratch, cudaStream_t s, long long* launches);
void launch_surr_gather(int Bn, long long S, long long off, long long stride, const float* feat, const float* y,
                        float* xb, float* yb, cudaStream_t s, long long* launches);
void launch_surr_adam(float* w, float* wb, const float* g, float* m, float* v, float lr, int step, cudaStream_t s,
                      long long* launches);

// Fisher / bias / quadratic estimates from packed FP32 C_p, FP64 accumulation.
struct FisherArgs {
    int nmodes, nbands;
    const float* Dp;       // [nbands][K]
    const double* evals;   // [nmodes]
    const double* y;       // [nmodes]
    const double* prior;   // [nbands]
    double* partial;       // [nblocks][nbands*(nbands+2)] scratch
    int nblocks;
    double* out;           // [nbands*nbands + 2*nbands]: F, f, q
};
int fisher_blocks(int nmodes);
int fisher_blocks_for(long long entries);
void launch_fisher(const FisherArgs& a, cudaStream_t s, long long* launches);

// The Fisher sums over the same-group mode pairs of the azimuthal block
// structure, values read from the per-block matrices C_b of every band (the
// packed triangle is never formed).  Groups are (block, trig class); their
// modes ascending; entries of group g are its pairs u <= v, numbered as a
// packed triangle from g_entry[g].
struct BlockFisherArgs {
    int ngroups;
    const long long* g_entry;  // [ngroups + 1] entry prefix
    const int* g_mode;         // [ngroups + 1] prefix into modes
    const int* g_blk;          // [ngroups] block of the group
    const int* modes;          // [nmodes] mode indices, grouped
    const int* mode_col;       // [nmodes] column of mode i in its block's C_b
    const int* Km;             // [nblk] C_b is Km x Km
    const long long* off;      // [nblk] offset of C_b in one band's array
    long long csize;           // floats per band
    const float* C;            // [nbands][csize]
};
void launch_fisher_blocks(const FisherArgs& a, const BlockFisherArgs& b, long long entries, cudaStream_t s,
                          long long* launches);

// Nb x Nb epilogue: mixing, window, estimates, covariance; status word on error.
void launch_epilogue(int nb, int mixing, const double* Fqf, double* out, int* status, cudaStream_t s,
                     long long* launches);

// y_i = sum_a B_ia (N_a - Nbar_a) / sqrt(Nbar_a)
// y = B^T x with x = (N - Nbar) / sqrt(Nbar) formed in place of `counts`
// y = B^T x on the azimuthal modes of the last block eigensolve, from the block eigenvectors U
// (no mode matrix); X: 2 H (Nphi/2 + 1) doubles of scratch.  counts are read, not changed.
void launch_dot_azimuthal(int H, int Nphi, int Nmu, int npar, int nmodes, const int* sel_b, const int* sel_idx,
                          const int* sel_kind, const double* U, const double* counts, const double* nbar, double* X,
                          double* y, cudaStream_t s, long long* l);
void launch_dot(int ncells, int nmodes, const double* modes, double* counts, const double* nbar, double* y,
                cudaStream_t s, long long* launches);

// B'[i][a] = sqrt(Nbar_a) B[i][a]
void launch_scale_modes(int ncells, int nmodes, const double* modes, const double* nbar, double* Bs, cudaStream_t s,
                        long long* launches);

// packed FP32 -> FP64
void launch_widen(size_t n, const float* in, double* out, cudaStream_t s, long long* launches);

// Top-M eigenpairs of a dense symmetric FP64 matrix by Chebyshev-filtered subspace
// iteration (chfsi.cu).
struct ChfsiArgs {
    int N = 0, M = 0;
    const double* S = nullptr;  // N x N, symmetric, both triangles
    int guard = 32;             // block B = M + guard, rounded up to a multiple of 32
    int degree = 12;            // largest Chebyshev degree
    int maxit = 100;            // filter iterations at most
    double tol = 1e-5;          // |S x - theta x| <= tol |theta| for the top M
    int tc = 1;                 // products with S by the engine's tcgen05 kernel (gemm_tc.cu)
    int tile = 0;               // its output tiles: 128 or 256 columns (0: by the SMs' waves)
    int df64 = 1;               // refinement products in double-FP32 (gemm_df.cu, 1) or cuBLAS DGEMM (0)
    int cholqr = 1;             // refinement QR: CholeskyQR2 with double-FP32 products (1) or Householder (0)
    int emulate = 1;            // other FP32 GEMMs (and S products when tc = 0) as cuBLAS BF16x9 (1) or FP32 SIMT (0)
    long long wait_cycles = 2000000000LL;  // bound of the tcgen05 kernel's barrier waits
    int refine = 2;             // FP64 refinement rounds (correction solves) at most
    int cg_steps = 20;          // CG steps per correction solve at most
    unsigned long long seed = 1;
    double* modes = nullptr;    // out: M x N, mode-major
    double* evals = nullptr;    // out: M, descending
};
struct ChfsiStats {
    int iterations = 0, degree = 0, gemms = 0, block = 0, rounds = 0, cg_steps = 0;
    double lo = 0, hi = 0, resid = 0;  // spectrum bounds; largest relative FP64 residual of the top M
};
void chfsi_eigensolve(const ChfsiArgs& a, cublasHandle_t blas, cusolverDnHandle_t solver, cudaStream_t s,
                      long long* launches, ChfsiStats* stats);

// Weighted galaxy counts per cell (signal.cu); counts has ncells + 1 entries, the last
// for galaxies outside every cell.
struct GridBox {
    double lo[3], hi[3];
    int n[3];
};
void launch_galaxy_counts(long long ngal, const float4* gal, const GridBox& g, const int* cellmap, int ncells,
                          double* counts, cudaStream_t st, long long* l);

// Cell builder (basis.cu): Veff and Nbar of every grid cell.
struct BasisArgs {
    int coordsys;           // 1 Cartesian (constant nbar), 2 spherical (radial spline x map)
    int n[3];
    const double* bounds;   // [cells][6]: min1 max1 min2 max2 min3 max3, grid order
    double nbar;            // Cartesian: the constant selection
    int nrad;
    const double* rad_r;    // spherical: radial linear spline knots
    const double* rad_n;
    long long nside;        // HEALPix map (0: none)
    int nest;
    const float* mask;
    int samples;            // map points per cell axis
    int quirk3;             // 1: the reference's 3x spherical Nbar
    double* out;            // [cells][2]: Veff, Nbar
};
void launch_basis(const BasisArgs& b, cudaStream_t s, long long* launches);
void launch_ang2pix(long long nside, int nest, int n, const double* theta, const double* phi, long long* pix,
                    cudaStream_t s, long long* launches);

// Mock counts (mock.cu): white noise, FFT, P(k) shaping, inverse FFT, cell counts.
constexpr unsigned long long kMockNoiseStream = 0x6E6F697365ULL;    // Philox key word 1 of the noise
constexpr unsigned long long kMockPoissonStream = 0x706F6973ULL;    // Philox key word 1 of the counts
constexpr int kMockMaxAttempts = 64;                               // PTRS attempts per draw
struct MockArgs {
    int ngrid;             // mesh points per axis (even)
    double box;            // mesh side
    unsigned long long seed;
    double bias;
    int npk;
    const double* pk;      // cubic spline of P(k): x, y, b, c, d (npk each)
    double* grid;          // [ngrid^3] noise, then the field
    double2* spec;         // [ngrid][ngrid][ngrid/2+1]
    int ncells;
    const long long* idx;  // [ncells] mesh point of each cell centre
    const double* nbar;    // [ncells]
    double* counts;        // [ncells] out
    double* delta;         // [ncells] out: the field at the cell centres
};
struct MockPlans {
    int n = 0;
    int fwd = 0, inv = 0;  // cuFFT handles
};
void launch_mock_counts(const MockArgs& m, MockPlans& plans, cudaStream_t s, long long* launches);
void destroy_mock_plans(MockPlans& plans);

#ifdef __CUDACC__
// Cubic spline of a tabulated function (Spline.cpp:13-35 lookup, :429-434 zero outside
// [x0, x_last)); shared by the xi tables and the mock spectrum.
__device__ inline int lookup_index(double x, int N, const double* X) {
    double I = (N - 1) * (x - X[0]) / (X[N - 1] - X[0]);
    int i = (int)I;
    i = i < 0 ? 0 : (i > N - 2 ? N - 2 : i);
    int ilo = 0, ihi = N - 2;
    while (ilo < ihi) {
        if (x < X[i]) {
            ihi = i - 1;
            i = (ilo + ihi) / 2;
        } else if (x > X[i + 1]) {
            ilo = i + 1;
            i = (ilo + ihi) / 2;
        } else
            break;
    }
    return i;
}

__device__ inline double spline_eval(int N, const double* X, const double* Y, const double* b, const double* c,
                                     const double* d, double x) {
    if (x < X[0] || x >= X[N - 1]) return 0.0;
    int i = lookup_index(x, N, X);
    double u = x - X[i];
    return Y[i] + b[i] * u + c[i] * u * u + d[i] * u * u * u;
}
#endif

}  // namespace opsec
