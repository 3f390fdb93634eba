// context.h -- the engine context (struct opsec_gpu) and the host-side stages that the
// C ABI (context.cpp) drives; internal to the library.
//   config.cpp          configuration text -> context fields, the P(k) file
//   tables.cpp          xi tables, key spaces
//   stages.cpp          Q by cubature, the square table, cells
//   eigensolve.cpp      the KL eigensolve (azimuthal blocks, dense, iterative)
//   project_host.cpp    C_p = B^T S_p B (azimuthal blocks or the fused tensor-core projection)
//   surrogate_host.cpp  training and use of the far-field surrogate
//   estimate_host.cpp   band priors, Fisher sums and the estimate epilogue
//   batch.cpp           batched mock surveys
#pragma once
#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cfloat>
#include <functional>
#include <array>
#include <atomic>
#include <chrono>
#include <cerrno>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"

namespace opsec {
void launch_project_simt(const ProjectArgs& a, cudaStream_t s, long long* launches);
bool project_tc_supported(const ProjectArgs& a);
void launch_project_tc(const ProjectArgs& a, cudaStream_t s, long long* launches);
size_t project_tc_work_bytes(const ProjectArgs& a);
void launch_fisher64(const FisherArgs& a, const double* Dp64, cudaStream_t s, long long* launches);
void launch_reverse_modes(int n, int m, int lda, const double* A, const double* w, double* modes, double* evals,
                          cudaStream_t s, long long* launches);
// klt.solver = auto: the subspace iteration from this many cells on (and a block of at most
// a quarter of them); the dense FP64 syevdx below
constexpr int kChfsiMinCells = 16384;
void blas_check(cublasStatus_t st, const char* what);
void solver_check(cusolverStatus_t st, const char* what);
std::map<std::string, std::string> parse_config(const char* text);
double to_double(const std::string& key, const std::string& v);
int to_int(const std::string& key, const std::string& v);
void cspline_coeffs(const std::vector<double>& X, const std::vector<double>& Y, std::vector<double>& b,
                    std::vector<double>& c, std::vector<double>& d);
int lookup_index(double x, int N, const double* X);
void gauss_legendre01(int n, std::vector<double>& u, std::vector<double>& w);
}  // namespace opsec

using namespace opsec;

// ---------------------------------------------------------------- context
struct opsec_gpu {
    std::string err;
    int device = 0;
    cudaStream_t stream = nullptr;
    cusolverDnHandle_t solver = nullptr;
    cublasHandle_t blas = nullptr;
    // side streams for the independent azimuthal eigenproblems
    static constexpr int kSide = 16;
    cudaStream_t side[kSide] = {};
    cusolverDnHandle_t side_solver[kSide] = {};
    cudaEvent_t side_ev[kSide + 1] = {};
    // FP32 band blocks of the block projection, transformed on their own stream while the
    // eigensolve runs (they depend on the Q tables only): prefetch_band_blocks, az_blocks
    cudaStream_t band_stream = nullptr;
    cudaEvent_t band_ev[2] = {};       // [0] Q tables ready on the main stream, [1] blocks done
    bool band_pending = false;         // band_stream holds work the host has not waited for
    int band_batch = 0;                // bands prefetched into azSb for this build (0: none)
    int band_nblk = 0, band_H = 0;     // their block count and order
    long long launches = 0;
    double stage_ms[5] = {0, 0, 0, 0, 0};
    std::string warning;

    // configuration
    Geometry geo;
    XiLayout xl;
    int ng = 4;
    int nmodes_cfg = 0;
    int mixing = OPSEC_MIXING_INVERSE;
    std::string projection = "auto";
    int proj_chunk = 1;
    long long proj_wait = 2000000000LL;  // projection kernels: mbarrier wait bound in cycles
    bool proj_arcs = true;               // projection: arc-run tables for spherical cells in arc order
    bool cells_arc_order = false;        // the loaded cells are in arc order (cell = h N3 + f)
    bool modes_ok = false;               // c->modes holds the modes of the last eigensolve
    DevBuf<double> arc_x;                // per-arc trig sums of the pixel values
    long long fail_alloc = -1;           // opsec_gpu_fail_alloc: device allocations left before one fails
    int cub_exact = 1;
    int az_gemm64 = 0;
    int az_tc = 1;  // block projection GEMMs on the tensor cores (az_tc.cu); 0: cuBLAS SGEMM
    int az_tiled = 1;  // FP32 band blocks by staged tiles (1) or one thread per output (0); same bits
    int az_overlap = 1;  // FP32 band blocks transformed during the eigensolve (1) or after it (0); same bits
    bool cub_reflect = true;
    int cub_window = 1;
    int win_key = 384, win_flush = 8, win_dot64 = 0, win_logkeys = 1, win_keyorder = 1;
    bool az_parity = true;
    bool az_batched = true;
    bool az_own = true;     // the hand-written block eigensolver (blockeig.cu), else cuSOLVER
    int az_streams = 6;
    int az_split = 1;  // batched eigensolve calls in flight at once
    // the batched eigensolve as a CUDA graph, for builds that repeat the shapes and buffers
    bool eig_graph_ok = true;
    std::array<size_t, 6> eig_key{};
    cudaGraphExec_t eig_exec = nullptr;
    std::vector<unsigned char> eig_hw;  // the captured call's host workspace
    int az_npar = 1;
    std::vector<double> pk_k, pk_P;
    std::vector<double> band_lo, band_hi;

    // device state
    bool tables_ok = false, q_ok = false, qsq_ok = false;
    bool custom_xi = false;  // a table was replaced through opsec_gpu_set_xi_table
    KeySpace ks;
    DevBuf<double> xi64, r_grid, scratch, pk_dev;
    DevBuf<float> xi32;
    DevBuf<double> Q;      // [ntab][nkeys]
    DevBuf<float> Qsq;     // [ntab][nsquare]
    DevBuf<double> nodes;  // node tables for the cubature kernel
    DevBuf<float> cubpts;  // cubature point table, 8 floats per Gauss point of every cell
    DevBuf<unsigned char> cubwork;  // cubature window-path scratch
    DevBuf<int> cell_i;    // d1,d2,d3 then h,f,g per cell
    DevBuf<double> nbar;
    DevBuf<int> rc;        // rows/cols for signal blocks
    DevBuf<double> sblock;
    DevBuf<double> S;      // dense S or azimuthal blocks
    DevBuf<double> W;      // eigenvalues
    DevBuf<double> work;   // solver workspace
    DevBuf<int> info;
    DevBuf<int> sel;
    // modes of the last azimuthal eigensolve: per mode its order m, block eigenvector idx, kind
    bool az_valid = false;
    std::vector<int> az_m, az_idx, az_kind;
    std::vector<double> nbar_arc;
    DevBuf<unsigned char> azws;  // azimuthal projection workspace
    DevBuf<unsigned char> azSb;  // FP32 band blocks of one batch of bands
    DevBuf<double> nba_band;     // per-arc Nbar read by the band-block transforms
    DevBuf<double> nba_dev;      // Nbar per arc
    DevBuf<unsigned char> syev_ws;  // batched eigensolver workspace
    DevBuf<double> bev_V, bev_T, bev_vec;  // hand-written block eigensolver: reflectors, T, vectors
    DevBuf<int> bev_i;
    DevBuf<int> probe;  // opsec_gpu_wait_probe's status word
    std::string cfg_text;        // the configuration the context was created with
    // learned far-field surrogate: 4 networks (FP32 master weights) and the target scale
    static constexpr int kMembers = 4;
    bool surr_on = false;
    float surr_tol = 0.02f, surr_far = 2.0f;
    std::vector<float> surr_w;  // kMembers * kSurrParams, empty until trained or loaded
    float surr_ysc = 0.f;
    long long surr_counts[3] = {0, 0, 0};  // keys predicted, sent back to the cubature, far keys
    DevBuf<float> surr_kg, surr_wdev, surr_pred, surr_tinfo;
    DevBuf<double> surr_env;  // [ntab][n]: local envelope of every table
    DevBuf<long long> surr_list;
    DevBuf<unsigned char> surr_done;
    DevBuf<int> surr_cnt;
    DevBuf<int> az_i;
    DevBuf<long long> az_off;
    // cell builder: the selection function (Cartesian constant, spherical radial spline x map)
    double sel_nbar = 0.0;
    std::vector<double> rad_r, rad_n;
    long long mask_nside = 0;
    int mask_nest = 0;
    DevBuf<float> mask_dev;
    int basis_quirk3 = 0, basis_samples = 16;
    // dense-grid eigensolver: dense FP64 syevdx, Chebyshev-filtered subspace iteration, or by size
    std::string eig_solver = "auto";
    ChfsiArgs chfsi;  // its options (sizes and buffers set per call)
    bool chfsi_guard_set = false;
    double eig_stats[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    // mock counts: cuFFT plans for the last mesh size, mesh and per-cell buffers
    MockPlans mock_plans;
    DevBuf<double> mock_grid, mock_spec, mock_nbar, mock_out;
    DevBuf<long long> mock_idx;
    // block Fisher of the last azimuthal projection (Fisher build without the packed triangle)
    bool az_blockF = false;
    BlockFisherArgs bf{};
    long long bf_entries = 0;
    DevBuf<int> bf_i;
    DevBuf<long long> bf_l;
    DevBuf<double> evals, modes, Bs, y, counts, prior, fout, partial, est;
    DevBuf<float> Dp;
    DevBuf<double> Dp64;
    DevBuf<unsigned char> pwork;
    DevBuf<int> status;
    int ncells_loaded = 0;

    // per-kernel timing (config key profile = 1)
    KernelClock clock;
    struct Stat {
        long long count = 0;
        double ms = 0, flops = 0, bytes = 0;
    };
    std::map<std::string, Stat> stats;

    int ntab() const { return 1 + (int)band_lo.size(); }
};

// ---------------------------------------------------------------- stages (defined in the files above)
void collect_clock(opsec_gpu* c);
void sync(opsec_gpu* c);
void load_pkfile(opsec_gpu* c, const std::string& path);
void configure(opsec_gpu* c, const std::map<std::string, std::string>& kv);
void build_tables(opsec_gpu* c);
void setup_keys(opsec_gpu* c);
void surrogate_stage(opsec_gpu* c);
void surrogate_train(opsec_gpu* c, long long max_samples, int epochs, unsigned seed, double* stats);
void build_q(opsec_gpu* c);
void build_qsq(opsec_gpu* c);
void load_cells(opsec_gpu* c, int ncells, const opsec_cell* cells);
CellKeyInfo cell_info(opsec_gpu* c);
bool azimuthal_ok(opsec_gpu* c, int ncells, const opsec_cell* cells);
// the per-arc Nbar of a full-sky build (nba) and its mu-parity split of the azimuthal blocks: 2
// when the mu grid and Nbar are symmetric under mu -> -mu (each order m then splits into even and
// odd blocks), else 1
int az_parity_split(opsec_gpu* c, const opsec_cell* cells, std::vector<double>& nba);
// the FP32 band blocks of the block projection, transformed on the band stream while the
// eigensolve runs (a no-op when the build will not project by blocks in FP32); band_wait: the
// host waits for that stream
void prefetch_band_blocks(opsec_gpu* c, int ncells, const opsec_cell* cells);
void band_wait(opsec_gpu* c);
void drop_eig_graph(opsec_gpu* c);
// want_modes = false leaves the mode matrix unformed on the azimuthal path (ensure_modes forms it
// from the kept block eigenvectors when a later step needs it)
int eigensolve(opsec_gpu* c, int ncells, const opsec_cell* cells, int M, bool want_modes = true);
void ensure_modes(opsec_gpu* c);
// y = B^T (N - Nbar)/sqrt(Nbar) for the modes of the last eigensolve (counts already on the device)
void pixel_projection(opsec_gpu* c, int ncells, int n);
void project_all(opsec_gpu* c, int ncells, int M, bool own_modes, bool packed = true);
std::vector<double> priors(opsec_gpu* c);
void fisher_and_epilogue(opsec_gpu* c, int M, const float* Dp32, const double* Dp64, int mixing, double* phat,
                         double* pcov, double* F, double* W, double* Mx, double* q, double* f);
float bf16_round_host(float x);
SurrGrid surr_grid(const opsec_gpu* c);

void forget_device_state(opsec_gpu* c);

template <class F>
inline int guard(opsec_gpu* ctx, F&& f) {
    if (!ctx) return OPSEC_ERR_ARG;
    struct ClockScope {
        opsec_gpu* c;
        explicit ClockScope(opsec_gpu* cc) : c(cc) {
            g_clock = &cc->clock;
            g_fail_alloc = &cc->fail_alloc;
        }
        ~ClockScope() {
            collect_clock(c);
            g_clock = nullptr;
            g_fail_alloc = nullptr;
        }
    } scope(ctx);
    try {
        ctx->err.clear();
        ctx->band_batch = 0;  // band blocks prefetched by an earlier call (one that failed) are not this call's
        if (ctx->device >= 0) OPSEC_CUDA(cudaSetDevice(ctx->device));
        f();
        return OPSEC_OK;
    } catch (const Error& e) {
        ctx->err = e.msg;
        if (e.code == OPSEC_ERR_NOMEM) forget_device_state(ctx);
        return e.code;
    } catch (const std::bad_alloc&) {
        ctx->err = "host allocation failed";
        return OPSEC_ERR_NOMEM;
    } catch (const std::exception& e) {
        ctx->err = e.what();
        return OPSEC_ERR_ARG;
    }
}
