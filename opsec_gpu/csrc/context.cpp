// context.cpp -- host side of the engine: configuration, model and survey
// setup, device-resident pipeline, and the C ABI of include/opsec_gpu.h.
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

[[noreturn]] void fail(int code, const std::string& msg) { throw Error{code, msg}; }

thread_local KernelClock* g_clock = nullptr;
thread_local long long* g_fail_alloc = nullptr;

void KernelClock::begin(const char* name, cudaStream_t s, double flops, double bytes) {
    if (!on) return;
    Rec r{name, nullptr, nullptr, flops, bytes};
    OPSEC_CUDA(cudaEventCreate(&r.a));
    OPSEC_CUDA(cudaEventCreate(&r.b));
    OPSEC_CUDA(cudaEventRecord(r.a, s));
    open.push_back(pending.size());
    pending.push_back(r);
}

void KernelClock::end(cudaStream_t s) {
    if (!on || open.empty()) return;
    OPSEC_CUDA(cudaEventRecord(pending[open.back()].b, s));
    open.pop_back();
}

int max_dynamic_smem(const void* func) {
    static std::atomic<int> cache[64];
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64) fail(OPSEC_ERR_CUDA, "device index out of range");
    int v = cache[dev].load();
    if (v <= 0) {
        cuda_check(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev),
                   "cudaDeviceGetAttribute(MaxSharedMemoryPerBlockOptin)");
        cache[dev] = v;
    }
    // The opt-in ceiling covers static plus dynamic shared memory of one block.
    cudaFuncAttributes fa;
    cuda_check(cudaFuncGetAttributes(&fa, func), "cudaFuncGetAttributes");
    return v - (int)fa.sharedSizeBytes;
}

void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation) fail(OPSEC_ERR_NOMEM, std::string(what) + ": out of device memory");
        fail(OPSEC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

// klt.solver = auto: the subspace iteration from this many cells on (and a block of at most
// a quarter of them); the dense FP64 syevdx below
constexpr int kChfsiMinCells = 16384;

static void blas_check(cublasStatus_t st, const char* what) {
    if (st != CUBLAS_STATUS_SUCCESS) fail(OPSEC_ERR_CUDA, std::string(what) + " failed (cuBLAS status " + std::to_string((int)st) + ")");
}

static void solver_check(cusolverStatus_t st, const char* what) {
    if (st != CUSOLVER_STATUS_SUCCESS) fail(OPSEC_ERR_CUDA, std::string(what) + ": cuSOLVER status " + std::to_string((int)st));
}

template <class T>
void DevBuf<T>::alloc(size_t count) {
    if (count <= n && p) return;
    release();
    if (count == 0) return;
    if (g_fail_alloc && *g_fail_alloc >= 0 && (*g_fail_alloc)-- == 0)
        fail(OPSEC_ERR_NOMEM, "cudaMalloc of " + std::to_string(sizeof(T) * count) +
                                  " bytes failed (injected by opsec_gpu_fail_alloc)");
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), sizeof(T) * count);
    if (e != cudaSuccess) {
        p = nullptr;
        n = 0;
        cudaGetLastError();
        fail(OPSEC_ERR_NOMEM, "cudaMalloc of " + std::to_string(sizeof(T) * count) + " bytes failed");
    }
    n = count;
}

template <class T>
void DevBuf<T>::release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
}

template struct DevBuf<double>;
template struct DevBuf<float>;
template struct DevBuf<int>;
template struct DevBuf<unsigned char>;
template struct DevBuf<long long>;

bool Geometry::mu_symmetric() const {
    return coordsys == 2 && std::fabs(b[2] + b[3]) <= 1e-12 * std::fabs(b[3] - b[2]);
}

bool Geometry::full_sky() const { return coordsys == 2 && std::fabs(b[5] - b[4] - 2 * M_PI) < 1e-12; }

// ---------------------------------------------------------------- config
// key = value lines, '#' comments, C isspace trimmed, one pair of surrounding quotes stripped,
// the last value of a key kept (cfg.c:238-295).  A line that is not key = value is an error
// here: the reference stops reading its file there (cfg.c:200-214), a text handed to the
// library is refused instead.
static bool cspace(char c) { return std::isspace((unsigned char)c) != 0; }

static std::map<std::string, std::string> parse_config(const char* text) {
    std::map<std::string, std::string> kv;
    if (!text) return kv;
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
        size_t p = 0, end = line.size();
        while (p < end && cspace(line[p])) p++;
        if (p == end || line[p] == '#') continue;
        const size_t eq = line.find('=', p);
        if (eq == std::string::npos || eq == p) fail(OPSEC_ERR_CONFIG, "not a key = value line: '" + line + "'");
        size_t ke = eq;
        while (ke > p && cspace(line[ke - 1])) ke--;
        size_t vb = eq + 1;
        while (vb < end && cspace(line[vb])) vb++;
        size_t ve = end;
        while (ve > vb && cspace(line[ve - 1])) ve--;
        if (ve - vb >= 2 && ((line[vb] == '"' && line[ve - 1] == '"') || (line[vb] == '\'' && line[ve - 1] == '\''))) {
            vb++;
            ve--;
        }
        kv[line.substr(p, ke - p)] = line.substr(vb, ve - vb);
    }
    return kv;
}

static double to_double(const std::string& key, const std::string& v) {
    char* end = nullptr;
    errno = 0;
    double d = std::strtod(v.c_str(), &end);
    if (end == v.c_str() || errno == ERANGE || !std::isfinite(d)) fail(OPSEC_ERR_CONFIG, "option " + key + " = '" + v + "' is not a number");
    return d;
}

// cfg_get_int (cfg.c:430-440) reads "%i": a leading integer in decimal, octal (0...) or hex
// (0x...), whatever follows it ignored
static int to_int(const std::string& key, const std::string& v) {
    char* end = nullptr;
    long x = std::strtol(v.c_str(), &end, 0);
    if (end == v.c_str()) fail(OPSEC_ERR_CONFIG, "option " + key + " = '" + v + "' is not an integer");
    return (int)x;
}

// ---------------------------------------------------------------- host math
// fmm cubic spline coefficients (Spline.cpp:258-330).
static void cspline_coeffs(const std::vector<double>& X, const std::vector<double>& Y, std::vector<double>& b,
                           std::vector<double>& c, std::vector<double>& d) {
    const int N = (int)X.size();
    b.assign(N, 0);
    c.assign(N, 0);
    d.assign(N, 0);
    if (N == 2) {
        b[0] = b[1] = (Y[1] - Y[0]) / (X[1] - X[0]);
        return;
    }
    d[0] = X[1] - X[0];
    c[1] = (Y[1] - Y[0]) / d[0];
    for (int i = 1; i < N - 1; i++) {
        d[i] = X[i + 1] - X[i];
        b[i] = 2 * (d[i - 1] + d[i]);
        c[i + 1] = (Y[i + 1] - Y[i]) / d[i];
        c[i] = c[i + 1] - c[i];
    }
    b[0] = -d[0];
    b[N - 1] = -d[N - 2];
    c[0] = 0;
    c[N - 1] = 0;
    if (N > 3) {
        c[0] = c[2] / (X[3] - X[1]) - c[1] / (X[2] - X[0]);
        c[N - 1] = c[N - 2] / (X[N - 1] - X[N - 3]) - c[N - 3] / (X[N - 2] - X[N - 4]);
        c[0] = c[0] * d[0] * d[0] / (X[3] - X[0]);
        c[N - 1] = -c[N - 1] * d[N - 2] * d[N - 2] / (X[N - 1] - X[N - 4]);
    }
    for (int i = 1; i < N; i++) {
        double t = d[i - 1] / b[i - 1];
        b[i] -= t * d[i - 1];
        c[i] -= t * c[i - 1];
    }
    c[N - 1] = c[N - 1] / b[N - 1];
    for (int j = 0; j < N - 1; j++) {
        int i = N - j - 2;
        c[i] = (c[i] - d[i] * c[i + 1]) / b[i];
    }
    b[N - 1] = (Y[N - 1] - Y[N - 2]) / d[N - 2] + d[N - 2] * (c[N - 2] + 2 * c[N - 1]);
    for (int i = 0; i < N - 1; i++) {
        b[i] = (Y[i + 1] - Y[i]) / d[i] - d[i] * (c[i + 1] + 2 * c[i]);
        d[i] = (c[i + 1] - c[i]) / d[i];
        c[i] = 3 * c[i];
    }
    c[N - 1] = 3 * c[N - 1];
    d[N - 1] = d[N - 2];
}

static int lookup_index(double x, int N, const double* X) {
    double I = (N - 1) * (x - X[0]) / (X[N - 1] - X[0]);
    int i = std::min(std::max((int)I, 0), N - 2);
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

// Gauss-Legendre nodes and weights on [0,1] (Newton on the Legendre recurrence).
static void gauss_legendre01(int n, std::vector<double>& u, std::vector<double>& w) {
    u.assign(n, 0.5);
    w.assign(n, 1.0);
    if (n == 1) return;
    for (int i = 0; i < (n + 1) / 2; i++) {
        double x = std::cos(M_PI * (i + 0.75) / (n + 0.5));
        double p0 = 1, p1 = x, dp = 1;
        for (int it = 0; it < 100; it++) {
            p0 = 1;
            p1 = x;
            for (int k = 2; k <= n; k++) {
                double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (x * p1 - p0) / (x * x - 1);
            double dx = p1 / dp;
            x -= dx;
            if (std::fabs(dx) <= 1e-15 * std::fabs(x)) break;
        }
        p0 = 1;
        p1 = x;
        for (int k = 2; k <= n; k++) {
            double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        dp = n * (x * p1 - p0) / (x * x - 1);
        double wt = 2 / ((1 - x * x) * dp * dp);
        u[i] = 0.5 * (1 - x);
        u[n - 1 - i] = 0.5 * (1 + x);
        w[i] = w[n - 1 - i] = 0.5 * wt;
    }
}

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
    long long fail_alloc = -1;           // opsec_gpu_fail_alloc: device allocations left before one fails
    int cub_exact = 1;
    int az_gemm64 = 0;
    bool cub_reflect = true;
    int cub_window = 1;
    int win_key = 384, win_flush = 8, win_dot64 = 0;
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

namespace {

void collect_clock(opsec_gpu* c) {
    for (auto& r : c->clock.pending) {
        float ms = 0;
        if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            auto& st = c->stats[r.name];
            st.count++;
            st.ms += ms;
            st.flops += r.flops;
            st.bytes += r.bytes;
        }
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    c->clock.pending.clear();
    c->clock.open.clear();
}

void forget_device_state(opsec_gpu* c);

template <class F>
int guard(opsec_gpu* ctx, F&& f) {
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

void load_pkfile(opsec_gpu* c, const std::string& path) {
    // Spline.cpp:48-90 LoadData: skip blank and '#' lines, columns 1 and 2
    FILE* fp = std::fopen(path.c_str(), "r");
    if (!fp) fail(OPSEC_ERR_FILE, "could not read pkfile '" + path + "'");
    char buf[4096];
    std::vector<double> k, P;
    while (std::fgets(buf, sizeof buf, fp)) {
        if (buf[0] == '\0' || buf[0] == '#' || buf[0] == '\n') continue;
        char* e1 = nullptr;
        double a = std::strtod(buf, &e1);
        char* e2 = nullptr;
        double b = std::strtod(e1, &e2);
        if (e1 == buf || e2 == e1) continue;
        k.push_back(a);
        P.push_back(b);
    }
    std::fclose(fp);
    if (k.size() < 2) fail(OPSEC_ERR_FILE, "pkfile '" + path + "' holds fewer than two points");
    c->pk_k = k;
    c->pk_P = P;
}

void configure(opsec_gpu* c, const std::map<std::string, std::string>& kv) {
    auto has = [&](const std::string& k) { return kv.count(k) > 0; };
    auto get = [&](const std::string& k) -> const std::string& {
        auto it = kv.find(k);
        if (it == kv.end()) fail(OPSEC_ERR_CONFIG, "missing configuration option " + k);
        return it->second;
    };
    // survey (Survey.cpp:12-60, InitializeSurvey Survey.cpp:140-165)
    std::string type = has("survey.type") ? get("survey.type") : "";
    std::string cs = has("coordsys") ? get("coordsys") : "";
    if (type == "BoxSurvey" || (type.empty() && cs == "cartesian")) {
        c->geo.coordsys = 1;
        const char* names[6] = {"XMin", "XMax", "YMin", "YMax", "ZMin", "ZMax"};
        const char* ns[3] = {"Nx", "Ny", "Nz"};
        for (int i = 0; i < 6; i++) c->geo.b[i] = to_double(names[i], get(std::string("survey.") + names[i]));
        for (int i = 0; i < 3; i++) c->geo.n[i] = to_int(ns[i], get(std::string("survey.") + ns[i]));
        // BoxSurvey separation is periodic with period L (BoxSurvey.cpp:19-37); L <= 0 = open box
        c->geo.L = has("survey.L") ? to_double("survey.L", get("survey.L")) : 0.0;
        if (has("survey.periodic") && get("survey.periodic") == "0") c->geo.L = 0.0;
    } else if (type == "SphericalSurvey" || (type.empty() && cs == "spherical")) {
        c->geo.coordsys = 2;
        c->geo.b[0] = to_double("RMin", get("survey.RMin"));
        c->geo.b[1] = to_double("RMax", get("survey.RMax"));
        // Survey.cpp:39 reads MuMin from the key "MuMuin"; it wins when present
        c->geo.b[2] = has("survey.MuMuin") ? to_double("MuMuin", get("survey.MuMuin"))
                                           : to_double("MuMin", get("survey.MuMin"));
        c->geo.b[3] = to_double("MuMax", get("survey.MuMax"));
        c->geo.b[4] = to_double("PhiMin", get("survey.PhiMin"));
        c->geo.b[5] = to_double("PhiMax", get("survey.PhiMax"));
        c->geo.n[0] = to_int("Nr", get("survey.Nr"));
        c->geo.n[1] = to_int("Nmu", get("survey.Nmu"));
        c->geo.n[2] = to_int("Nphi", get("survey.Nphi"));
    } else {
        fail(OPSEC_ERR_CONFIG, "survey.type must be BoxSurvey or SphericalSurvey (got '" + type + "')");
    }
    for (int i = 0; i < 3; i++) {
        if (c->geo.n[i] <= 0) fail(OPSEC_ERR_CONFIG, "survey grid sizes must be positive");
        if (!(c->geo.b[2 * i] < c->geo.b[2 * i + 1])) fail(OPSEC_ERR_CONFIG, "survey bounds must satisfy Min < Max");
    }
    if (c->geo.coordsys == 2 && (c->geo.b[0] < 0 || c->geo.b[2] < -1 || c->geo.b[3] > 1))
        fail(OPSEC_ERR_CONFIG, "spherical bounds need RMin >= 0 and -1 <= MuMin < MuMax <= 1");

    // model (Model.cpp:26-51, RealModel.cpp:33-79)
    if (has("model") && get("model") != "RealModel")
        fail(OPSEC_ERR_CONFIG, "model must be RealModel (got '" + get("model") + "')");
    if (has("RealModel.pkfile")) load_pkfile(c, get("RealModel.pkfile"));
    if (has("RealModel.bands")) {
        // whitespace- or comma-separated kmin kmax pairs (cfg_get_array_double, RealModel.cpp:44-48)
        std::string text = get("RealModel.bands");
        for (char& ch : text)
            if (ch == ',') ch = ' ';
        std::istringstream in(text);
        std::vector<double> v;
        std::string tok;
        while (in >> tok) v.push_back(to_double("RealModel.bands", tok));
        if (v.size() % 2) v.pop_back();  // RealModel.cpp:49-52 drops an odd trailing value
        for (size_t i = 0; i + 1 < v.size(); i += 2) {
            c->band_lo.push_back(v[i]);
            c->band_hi.push_back(v[i + 1]);
        }
    } else if (has("RealModel.Nbands")) {
        int nb = to_int("Nbands", get("RealModel.Nbands"));
        double kmin = to_double("kmin", get("RealModel.kmin"));
        double kmax = to_double("kmax", get("RealModel.kmax"));
        if (nb <= 0) fail(OPSEC_ERR_CONFIG, "RealModel.Nbands must be positive");
        for (int n = 0; n < nb; n++) {
            c->band_lo.push_back(kmin + n * (kmax - kmin) / nb);
            c->band_hi.push_back(kmin + (n + 1) * (kmax - kmin) / nb);
        }
    } else {
        fail(OPSEC_ERR_CONFIG, "k-bands not specified (RealModel.bands or RealModel.Nbands,kmin,kmax)");
    }
    if (c->band_lo.empty()) fail(OPSEC_ERR_CONFIG, "at least one k-band is required");
    for (size_t i = 0; i < c->band_lo.size(); i++)
        if (!(c->band_lo[i] < c->band_hi[i]) || c->band_lo[i] < 0)
            fail(OPSEC_ERR_CONFIG, "band " + std::to_string(i) + " has kmin >= kmax or kmin < 0");

    if (has("Nmodes")) c->nmodes_cfg = to_int("Nmodes", get("Nmodes"));
    if (has("mixing")) {
        // cfg_get_enum (cfg.c:486-501, estimate-mpi.cpp:369-372): the first of inverse,
        // inverse-sqrt, identity that the value is a prefix of; no match is inverse
        const std::string& m = get("mixing");
        static const std::pair<const char*, int> tags[] = {{"inverse", OPSEC_MIXING_INVERSE},
                                                          {"inverse-sqrt", OPSEC_MIXING_INVERSE_SQRT},
                                                          {"identity", OPSEC_MIXING_IDENTITY}};
        c->mixing = OPSEC_MIXING_INVERSE;
        for (const auto& t : tags)
            if (std::string(t.first).compare(0, m.size(), m) == 0 && m.size() <= std::strlen(t.first)) {
                c->mixing = t.second;
                break;
            }
    }
    if (has("xi.n1")) c->xl.n1 = to_int("xi.n1", get("xi.n1"));
    if (has("xi.n2")) c->xl.n2 = to_int("xi.n2", get("xi.n2"));
    if (has("xi.r1")) c->xl.r1 = to_double("xi.r1", get("xi.r1"));
    if (has("xi.r2")) c->xl.r2 = to_double("xi.r2", get("xi.r2"));
    if (c->xl.n1 < 1 || c->xl.n2 < 2 || !(c->xl.r1 > 0) || !(c->xl.r2 > c->xl.r1))
        fail(OPSEC_ERR_CONFIG, "xi table layout needs n1 >= 1, n2 >= 2, 0 < r1 < r2");
    if (has("sig.gauss")) c->ng = to_int("sig.gauss", get("sig.gauss"));
    if (c->ng < 1 || c->ng > 6) fail(OPSEC_ERR_CONFIG, "sig.gauss must be between 1 and 6");
    if (has("projection")) c->projection = get("projection");
    if (has("projection.wait_cycles")) {
        const std::string& v = get("projection.wait_cycles");
        char* end = nullptr;
        c->proj_wait = std::strtoll(v.c_str(), &end, 10);
        if (end == v.c_str() || c->proj_wait < 10000000LL)
            fail(OPSEC_ERR_CONFIG, "projection.wait_cycles must be an integer >= 10000000");
    }
    if (has("projection.arc_tables")) {
        const std::string& v = get("projection.arc_tables");
        if (v != "0" && v != "1") fail(OPSEC_ERR_CONFIG, "projection.arc_tables must be 0 or 1");
        c->proj_arcs = v == "1";
    }
    if (has("projection.chunk")) c->proj_chunk = to_int("projection.chunk", get("projection.chunk"));
    if (c->proj_chunk < 1) fail(OPSEC_ERR_CONFIG, "projection.chunk must be >= 1");
    if (has("azimuthal.gemm")) {
        const std::string& v = get("azimuthal.gemm");
        if (v == "f64")
            c->az_gemm64 = 1;
        else if (v == "f32")
            c->az_gemm64 = 0;
        else
            fail(OPSEC_ERR_CONFIG, "azimuthal.gemm must be f64 or f32");
    }
    if (has("azimuthal.parity")) c->az_parity = get("azimuthal.parity") != "0";
    if (has("azimuthal.eig")) {
        const std::string& v = get("azimuthal.eig");
        if (v != "own" && v != "streams" && v != "batched")
            fail(OPSEC_ERR_CONFIG, "azimuthal.eig must be own, batched or streams");
        c->az_own = v == "own";
        c->az_batched = v != "streams";
    }
    if (has("klt.solver")) {
        c->eig_solver = get("klt.solver");
        if (c->eig_solver != "auto" && c->eig_solver != "dense" && c->eig_solver != "chfsi")
            fail(OPSEC_ERR_CONFIG, "klt.solver must be auto, dense or chfsi");
    }
    if (has("klt.tol")) c->chfsi.tol = to_double("klt.tol", get("klt.tol"));
    if (has("klt.degree")) c->chfsi.degree = to_int("klt.degree", get("klt.degree"));
    if (has("klt.maxit")) c->chfsi.maxit = to_int("klt.maxit", get("klt.maxit"));
    if (has("klt.guard")) {
        c->chfsi.guard = to_int("klt.guard", get("klt.guard"));
        c->chfsi_guard_set = true;
    }
    if (has("klt.refine")) c->chfsi.refine = to_int("klt.refine", get("klt.refine"));
    if (has("klt.cg")) c->chfsi.cg_steps = to_int("klt.cg", get("klt.cg"));
    if (c->chfsi.refine < 0 || c->chfsi.cg_steps < 1) fail(OPSEC_ERR_CONFIG, "klt.refine must be >= 0, klt.cg >= 1");
    if (has("klt.seed")) c->chfsi.seed = (unsigned long long)to_int("klt.seed", get("klt.seed"));
    if (has("klt.gemm")) {
        const std::string& v = get("klt.gemm");
        if (v != "bf16x9" && v != "f32") fail(OPSEC_ERR_CONFIG, "klt.gemm must be bf16x9 or f32");
        c->chfsi.emulate = v == "bf16x9";
    }
    if (!(c->chfsi.tol > 0) || c->chfsi.degree < 1 || c->chfsi.degree > 64 || c->chfsi.maxit < 1 || c->chfsi.guard < 0)
        fail(OPSEC_ERR_CONFIG, "klt.tol must be > 0, klt.degree in [1, 64], klt.maxit >= 1, klt.guard >= 0");
    if (has("survey.nbar")) c->sel_nbar = to_double("survey.nbar", get("survey.nbar"));
    if (has("basis.quirk3")) c->basis_quirk3 = to_int("basis.quirk3", get("basis.quirk3")) != 0;
    if (has("basis.samples")) {
        c->basis_samples = to_int("basis.samples", get("basis.samples"));
        if (c->basis_samples < 1 || c->basis_samples > 1024) fail(OPSEC_ERR_CONFIG, "basis.samples must be in [1, 1024]");
    }
    if (has("azimuthal.split")) {
        c->az_split = to_int("azimuthal.split", get("azimuthal.split"));
        if (c->az_split < 1 || c->az_split > opsec_gpu::kSide) fail(OPSEC_ERR_CONFIG, "azimuthal.split must be in [1, 16]");
    }
    if (has("azimuthal.streams")) {
        c->az_streams = to_int("azimuthal.streams", get("azimuthal.streams"));
        if (c->az_streams < 1 || c->az_streams > opsec_gpu::kSide) fail(OPSEC_ERR_CONFIG, "azimuthal.streams must be in [1, 16]");
    }
    if (has("surrogate")) c->surr_on = get("surrogate") == "1";
    if (has("surrogate.tol")) c->surr_tol = (float)to_double("surrogate.tol", get("surrogate.tol"));
    if (has("surrogate.far")) c->surr_far = (float)to_double("surrogate.far", get("surrogate.far"));
    if (!(c->surr_tol > 0) || !(c->surr_far >= 1)) fail(OPSEC_ERR_CONFIG, "surrogate.tol must be > 0 and surrogate.far >= 1");
    if (has("cubature.window")) c->cub_window = get("cubature.window") != "0";
    if (has("cubature.window_bins")) c->win_key = to_int("cubature.window_bins", get("cubature.window_bins"));
    if (c->win_key < 16 || c->win_key > 4096) fail(OPSEC_ERR_CONFIG, "cubature.window_bins must be in [16, 4096]");
    if (has("cubature.flush")) c->win_flush = to_int("cubature.flush", get("cubature.flush"));
    if (c->win_flush < 0) fail(OPSEC_ERR_CONFIG, "cubature.flush must be >= 0");
    if (has("cubature.dot")) c->win_dot64 = get("cubature.dot") != "f32";
    if (has("cubature.symmetry")) {
        const std::string& v = get("cubature.symmetry");
        if (v == "reflect")
            c->cub_reflect = true;
        else if (v == "none")
            c->cub_reflect = false;
        else
            fail(OPSEC_ERR_CONFIG, "cubature.symmetry must be reflect or none");
    }
    if (has("cubature.precision")) {
        const std::string& v = get("cubature.precision");
        if (v == "exact")
            c->cub_exact = 1;
        else if (v == "fast")
            c->cub_exact = 0;
        else
            fail(OPSEC_ERR_CONFIG, "cubature.precision must be exact or fast");
    }
    if (has("profile")) c->clock.on = get("profile") == "1";
}

void sync(opsec_gpu* c) { OPSEC_CUDA(cudaStreamSynchronize(c->stream)); }

// ---------------------------------------------------------------- stages
void build_tables(opsec_gpu* c) {
    if (c->tables_ok) return;
    if (c->pk_k.size() < 2) fail(OPSEC_ERR_STATE, "no P(k): set RealModel.pkfile or call opsec_gpu_set_pk");
    const int n = c->xl.n(), ntab = c->ntab(), nb = ntab - 1;
    // r grid exactly as QSpline::MakeArray (QSpline.cpp:6-17)
    std::vector<double> r(n);
    for (int i = 0; i < c->xl.n1; i++) r[i] = i * c->xl.r1 / c->xl.n1;
    for (int j = 0; j < c->xl.n2; j++) r[c->xl.n1 + j] = c->xl.r1 * std::exp(j * std::log(c->xl.r2 / c->xl.r1) / (c->xl.n2 - 1));
    std::vector<double> b, cc, d;
    cspline_coeffs(c->pk_k, c->pk_P, b, cc, d);
    const int npk = (int)c->pk_k.size();
    std::vector<double> host;
    host.insert(host.end(), c->pk_k.begin(), c->pk_k.end());
    host.insert(host.end(), c->pk_P.begin(), c->pk_P.end());
    host.insert(host.end(), b.begin(), b.end());
    host.insert(host.end(), cc.begin(), cc.end());
    host.insert(host.end(), d.begin(), d.end());
    host.insert(host.end(), c->band_lo.begin(), c->band_lo.end());
    host.insert(host.end(), c->band_hi.begin(), c->band_hi.end());
    c->pk_dev.alloc(host.size());
    OPSEC_CUDA(cudaMemcpyAsync(c->pk_dev.p, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice, c->stream));
    c->r_grid.alloc(n);
    OPSEC_CUDA(cudaMemcpyAsync(c->r_grid.p, r.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    c->xi64.alloc((size_t)ntab * n);
    c->xi32.alloc((size_t)ntab * n);
    c->scratch.alloc(2 * ((size_t)32769 + (size_t)nb * 8193));
    XiTableArgs a;
    a.xl = c->xl;
    a.nbands = nb;
    a.pk_x = c->pk_dev.p;
    a.pk_y = a.pk_x + npk;
    a.pk_b = a.pk_y + npk;
    a.pk_c = a.pk_b + npk;
    a.pk_d = a.pk_c + npk;
    a.band_lo = a.pk_d + npk;
    a.band_hi = a.band_lo + nb;
    a.npk = npk;
    a.r = c->r_grid.p;
    a.xi64 = c->xi64.p;
    a.xi32 = c->xi32.p;
    a.scratch = c->scratch.p;
    launch_xi_tables(a, c->stream, &c->launches);
    sync(c);  // host arrays above go out of scope
    c->tables_ok = true;
}

void setup_keys(opsec_gpu* c) {
    KeySpace& ks = c->ks;
    ks.coordsys = c->geo.coordsys;
    ks.N1 = c->geo.n[0];
    ks.N2 = c->geo.n[1];
    ks.N3 = c->geo.n[2];
    if (ks.coordsys == 1) {
        ks.nkeys = (long long)ks.N1 * ks.N2 * ks.N3;
        ks.nsquare = ks.nkeys;
    } else {
        ks.H = ks.N1 * ks.N2;
        ks.fold = c->geo.full_sky();
        // reflection z -> -z maps mu cell j to N_mu-1-j when the mu range is symmetric about 0
        ks.mu_reflect = c->cub_reflect && c->geo.mu_symmetric();
        ks.nf = ks.fold ? ks.N3 / 2 + 1 : ks.N3;
        ks.nkeys = (long long)ks.H * (ks.H + 1) / 2 * ks.nf;
        ks.nsquare = (long long)ks.H * ks.H * ks.nf;
    }
}

// ---------------------------------------------------------------- learned surrogate
void build_q(opsec_gpu* c);

SurrGrid surr_grid(const opsec_gpu* c) {
    const Geometry& g = c->geo;
    SurrGrid sg;
    for (int k = 0; k < 6; k++) sg.b[k] = g.b[k];
    for (int k = 0; k < 3; k++) sg.d[k] = (g.b[2 * k + 1] - g.b[2 * k]) / g.n[k];
    return sg;
}

// per table: (k_lo 5, k_hi 5, band centre k, 0); the full xi table is (0, 0, 0.02, 0)
void surr_tables(opsec_gpu* c) {
    std::vector<float4> ti(c->ntab());
    ti[0] = make_float4(0.f, 0.f, 0.02f, 0.f);  // the full xi table: scale of the peak of k^2 P(k)
    for (size_t p = 0; p < c->band_lo.size(); p++)
        ti[p + 1] = make_float4((float)(5 * c->band_lo[p]), (float)(5 * c->band_hi[p]),
                                (float)(0.5 * (c->band_lo[p] + c->band_hi[p])), 0.f);
    c->surr_tinfo.alloc(4 * ti.size());
    OPSEC_CUDA(cudaMemcpyAsync(c->surr_tinfo.p, ti.data(), sizeof(float4) * ti.size(), cudaMemcpyHostToDevice,
                               c->stream));
}

// env_t(r_i) = max |xi_t(r_j)| over r_j in [r_i / 1.25, 1.25 r_i]: the scale of
// the surrogate's target, so that its error follows the local size of a table
void surr_envelope(opsec_gpu* c) {
    const int n = c->xl.n(), ntab = c->ntab();
    std::vector<double> tab((size_t)ntab * n), env((size_t)ntab * n);
    OPSEC_CUDA(cudaMemcpyAsync(tab.data(), c->xi64.p, sizeof(double) * tab.size(), cudaMemcpyDeviceToHost, c->stream));
    std::vector<double> r(n);
    OPSEC_CUDA(cudaMemcpyAsync(r.data(), c->r_grid.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    for (int t = 0; t < ntab; t++) {
        const double* T = tab.data() + (size_t)t * n;
        int lo = 0, hi = 0;  // window [lo, hi) of r_j in [r_i / 1.25, 1.25 r_i]
        for (int i = 0; i < n; i++) {
            while (lo < i && r[lo] < r[i] / 1.25) lo++;
            if (hi < i + 1) hi = i + 1;
            while (hi < n && r[hi] <= 1.25 * r[i]) hi++;
            double m = 0;
            for (int j = lo; j < hi; j++) m = std::max(m, std::fabs(T[j]));
            env[(size_t)t * n + i] = m > 0 ? m : 1e-300;
        }
    }
    c->surr_env.alloc(env.size());
    OPSEC_CUDA(cudaMemcpyAsync(c->surr_env.p, env.data(), sizeof(double) * env.size(), cudaMemcpyHostToDevice,
                               c->stream));
    sync(c);
}

// key geometry and the canonical far keys; returns their number
long long surr_far_keys(opsec_gpu* c) {
    if (c->geo.coordsys != 2) fail(OPSEC_ERR_CONFIG, "the surrogate covers spherical grids only");
    const KeySpace& ks = c->ks;
    c->surr_kg.alloc((size_t)ks.nkeys * kSurrKeyStride);
    launch_surr_key_geometry(ks, surr_grid(c), c->surr_far, c->surr_kg.p, c->stream, &c->launches);
    c->surr_list.alloc((size_t)ks.nkeys);
    c->surr_cnt.alloc(4);
    OPSEC_CUDA(cudaMemsetAsync(c->surr_cnt.p, 0, sizeof(int) * 4, c->stream));
    launch_surr_far_list(ks, c->surr_kg.p, c->surr_list.p, c->surr_cnt.p, c->stream, &c->launches);
    int n = 0;
    OPSEC_CUDA(cudaMemcpyAsync(&n, c->surr_cnt.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    return n;
}

// Predict Q of the canonical far keys with the ensemble; keys it accepts are
// marked in surr_done and skipped by the cubature.
void surrogate_stage(opsec_gpu* c) {
    if (c->surr_w.size() != (size_t)opsec_gpu::kMembers * kSurrParams)
        fail(OPSEC_ERR_STATE, "surrogate = 1 but no trained weights: call opsec_gpu_surrogate_train or _weights");
    const KeySpace& ks = c->ks;
    const int ntab = c->ntab();
    surr_tables(c);
    surr_envelope(c);
    const long long nfar = surr_far_keys(c);
    c->surr_done.alloc((size_t)ks.nkeys);
    OPSEC_CUDA(cudaMemsetAsync(c->surr_done.p, 0, (size_t)ks.nkeys, c->stream));
    c->surr_counts[0] = c->surr_counts[1] = 0;
    c->surr_counts[2] = nfar;
    if (nfar == 0) return;
    const int nm = opsec_gpu::kMembers;
    c->surr_wdev.alloc(c->surr_w.size());
    OPSEC_CUDA(cudaMemcpyAsync(c->surr_wdev.p, c->surr_w.data(), sizeof(float) * c->surr_w.size(),
                               cudaMemcpyHostToDevice, c->stream));
    const long long nsamp = nfar * ntab;
    c->surr_pred.alloc((size_t)nm * nsamp);
    const float4* ti = reinterpret_cast<const float4*>(c->surr_tinfo.p);
    if (g_clock) g_clock->begin("surrogate", c->stream, 2.0 * nm * nsamp * (16.0 * 128 + 2 * 128.0 * 128 + 128));
    for (int m = 0; m < nm; m++)
        launch_surr_infer(nsamp, c->surr_list.p, ntab, c->surr_kg.p, ti, nullptr,
                          c->surr_wdev.p + (size_t)m * kSurrParams, c->surr_pred.p + (size_t)m * nsamp, c->stream,
                          &c->launches);
    launch_surr_combine(nfar, c->surr_list.p, ntab, nm, c->surr_pred.p, c->surr_kg.p, c->xl, c->xi64.p,
                        c->surr_env.p, c->surr_ysc, c->surr_tol, ks.nkeys, c->Q.p, c->surr_done.p, c->surr_cnt.p + 1,
                        c->stream, &c->launches);
    if (g_clock) g_clock->end(c->stream);
    int cnt[2] = {0, 0};
    OPSEC_CUDA(cudaMemcpyAsync(cnt, c->surr_cnt.p + 1, sizeof(int) * 2, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    c->surr_counts[0] = cnt[0];
    c->surr_counts[1] = cnt[1];
}

// Glorot-uniform weights (the first layer over its 12 used inputs), zero biases
void surr_init(std::vector<float>& w, unsigned seed) {
    w.assign(kSurrParams, 0.f);
    uint64_t st = 0x9E3779B97F4A7C15ull ^ ((uint64_t)seed * 0xBF58476D1CE4E5B9ull);
    auto uni = [&]() {  // splitmix64 -> [0, 1)
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) / 9007199254740992.0;
    };
    auto fill = [&](int off, int nout, int nin, int nin_used) {
        const double a = std::sqrt(6.0 / (nin_used + nout));
        for (int o = 0; o < nout; o++)
            for (int i = 0; i < nin; i++) w[off + o * nin + i] = i < nin_used ? (float)((2 * uni() - 1) * a) : 0.f;
    };
    fill(kSurrOffW1, kSurrHid, kSurrIn, 12);
    fill(kSurrOffW2, kSurrHid, kSurrHid, kSurrHid);
    fill(kSurrOffW3, kSurrHid, kSurrHid, kSurrHid);
    fill(kSurrOffW4, 1, kSurrHid, kSurrHid);
}

float bf16_round_host(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

long long gcd_ll(long long a, long long b) {
    while (b) {
        const long long t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// Train the ensemble on this context's own survey: plain cubature Q of every key,
// then up to max_samples (canonical far key, table) samples, 2 % held out.
// stats: samples, validation rms error of y (mean over members), training seconds, ysc.
void surrogate_train(opsec_gpu* c, long long max_samples, int epochs, unsigned seed, double* stats) {
    const bool was_on = c->surr_on;
    c->surr_on = false;
    c->q_ok = c->qsq_ok = false;
    build_q(c);
    c->surr_on = was_on;
    c->q_ok = c->qsq_ok = false;  // the next build recomputes Q, with the surrogate when it is on
    const KeySpace& ks = c->ks;
    const int ntab = c->ntab();
    surr_tables(c);
    surr_envelope(c);
    const long long nfar = surr_far_keys(c);
    if (nfar < 16) fail(OPSEC_ERR_ARG, "too few far keys to train the surrogate");
    std::vector<long long> keys(nfar);
    OPSEC_CUDA(cudaMemcpyAsync(keys.data(), c->surr_list.p, sizeof(long long) * nfar, cudaMemcpyDeviceToHost,
                               c->stream));
    sync(c);
    std::sort(keys.begin(), keys.end());
    uint64_t st = 0x243F6A8885A308D3ull ^ seed;
    auto rnd = [&]() {  // xorshift64
        st ^= st << 13;
        st ^= st >> 7;
        st ^= st << 17;
        return st;
    };
    for (long long i = nfar - 1; i > 0; i--) std::swap(keys[i], keys[rnd() % (uint64_t)(i + 1)]);
    const long long nk = std::max<long long>(1, std::min<long long>(nfar, max_samples / ntab));
    keys.resize(nk);
    DevBuf<long long> dkeys;
    dkeys.alloc(nk);
    OPSEC_CUDA(cudaMemcpyAsync(dkeys.p, keys.data(), sizeof(long long) * nk, cudaMemcpyHostToDevice, c->stream));
    const long long S = nk * ntab;
    DevBuf<float> feat, y;
    feat.alloc((size_t)S * kSurrIn);
    y.alloc(S);
    launch_surr_samples(S, dkeys.p, ntab, c->surr_kg.p, reinterpret_cast<const float4*>(c->surr_tinfo.p), c->xl,
                        c->xi64.p, c->surr_env.p, c->Q.p, ks.nkeys, feat.p, y.p, c->stream, &c->launches);
    std::vector<float> hy(S);
    OPSEC_CUDA(cudaMemcpyAsync(hy.data(), y.p, sizeof(float) * S, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    float ysc = 0.f;
    for (float v : hy) ysc = std::max(ysc, std::fabs(v));
    if (!(ysc > 0)) ysc = 1.f;
    for (float& v : hy) v /= ysc;
    OPSEC_CUDA(cudaMemcpyAsync(y.p, hy.data(), sizeof(float) * S, cudaMemcpyHostToDevice, c->stream));
    const long long Sval = std::max<long long>(1, S / 50), Str = S - Sval;
    const int Bn = (int)std::min<long long>(2048, Str);
    DevBuf<float> xb, yb, w, wb, g, m1, v1, scratch, out;
    xb.alloc((size_t)Bn * kSurrIn);
    yb.alloc(Bn);
    w.alloc(kSurrParams);
    wb.alloc(kSurrParams);
    g.alloc(kSurrParams);
    m1.alloc(kSurrParams);
    v1.alloc(kSurrParams);
    scratch.alloc((size_t)7 * Bn * kSurrHid);
    out.alloc(Bn);
    DevBuf<double> loss;
    loss.alloc(1);
    std::vector<float> all((size_t)opsec_gpu::kMembers * kSurrParams);
    auto t0 = std::chrono::steady_clock::now();
    double val_sum = 0;
    for (int mem = 0; mem < opsec_gpu::kMembers; mem++) {
        std::vector<float> hw;
        surr_init(hw, seed * 7919u + 101u * (unsigned)mem + 1u);
        std::vector<float> hwb(hw.size());
        for (size_t i = 0; i < hw.size(); i++) hwb[i] = bf16_round_host(hw[i]);
        OPSEC_CUDA(cudaMemcpyAsync(w.p, hw.data(), sizeof(float) * kSurrParams, cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(wb.p, hwb.data(), sizeof(float) * kSurrParams, cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemsetAsync(g.p, 0, sizeof(float) * kSurrParams, c->stream));
        OPSEC_CUDA(cudaMemsetAsync(m1.p, 0, sizeof(float) * kSurrParams, c->stream));
        OPSEC_CUDA(cudaMemsetAsync(v1.p, 0, sizeof(float) * kSurrParams, c->stream));
        const long long steps_per_epoch = std::max<long long>(1, Str / Bn);
        int step = 0;
        for (int ep = 0; ep < epochs; ep++) {
            long long stride = (long long)(rnd() % (uint64_t)Str) | 1;
            while (gcd_ll(stride, Str) != 1) stride += 2;
            const long long off = (long long)(rnd() % (uint64_t)Str);
            const float lr = 2e-3f * std::pow(0.05f, (float)ep / (float)std::max(1, epochs - 1));
            for (long long k = 0; k < steps_per_epoch; k++) {
                launch_surr_gather(Bn, Str, (off + (k * Bn % Str) * (stride % Str)) % Str, stride, feat.p, y.p, xb.p,
                                   yb.p, c->stream, &c->launches);
                surr_forward_backward(Bn, xb.p, yb.p, wb.p, g.p, nullptr, out.p, scratch.p, c->stream, &c->launches);
                launch_surr_adam(w.p, wb.p, g.p, m1.p, v1.p, lr, ++step, c->stream, &c->launches);
            }
        }
        // validation rms of y over the held-out tail
        double se = 0;
        long long nv = 0;
        for (long long i0 = Str; i0 < S; i0 += Bn) {
            const int nb = (int)std::min<long long>(Bn, S - i0);
            OPSEC_CUDA(cudaMemsetAsync(loss.p, 0, sizeof(double), c->stream));
            surr_forward_backward(nb, feat.p + (size_t)i0 * kSurrIn, y.p + i0, wb.p, g.p, loss.p, out.p, scratch.p,
                                  c->stream, &c->launches);
            double l = 0;
            OPSEC_CUDA(cudaMemcpyAsync(&l, loss.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
            sync(c);
            se += l * nb;
            nv += nb;
        }
        val_sum += std::sqrt(se / std::max<long long>(nv, 1)) * ysc;
        OPSEC_CUDA(cudaMemcpyAsync(all.data() + (size_t)mem * kSurrParams, w.p, sizeof(float) * kSurrParams,
                                   cudaMemcpyDeviceToHost, c->stream));
        sync(c);
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    c->surr_w = all;
    c->surr_ysc = ysc;
    if (stats) {
        stats[0] = (double)S;
        stats[1] = val_sum / opsec_gpu::kMembers;
        stats[2] = secs;
        stats[3] = ysc;
    }
}

void build_q(opsec_gpu* c) {
    if (c->q_ok) return;
    build_tables(c);
    setup_keys(c);
    const int ng = c->ng;
    std::vector<double> u, w;
    gauss_legendre01(ng, u, w);
    const Geometry& g = c->geo;
    // per-axis node tables, computed with the reference's cell bounds (Survey.cpp:80-97)
    auto edge_lo = [&](int ax, int dd) { return g.b[2 * ax] + dd * (g.b[2 * ax + 1] - g.b[2 * ax]) / g.n[ax]; };
    auto edge_hi = [&](int ax, int dd) { return g.b[2 * ax] + (dd + 1) * (g.b[2 * ax + 1] - g.b[2 * ax]) / g.n[ax]; };
    std::vector<double> w_h(w), n1((size_t)g.n[0] * ng), n2((size_t)g.n[1] * ng), s2((size_t)g.n[1] * ng),
        n3((size_t)g.n[2] * ng), cp((size_t)g.n[2] * ng), sp((size_t)g.n[2] * ng);
    for (int ax = 0; ax < 3; ax++)
        for (int dd = 0; dd < g.n[ax]; dd++) {
            double lo = edge_lo(ax, dd), hi = edge_hi(ax, dd);
            for (int i = 0; i < ng; i++) {
                size_t o = (size_t)dd * ng + i;
                if (g.coordsys == 1) {
                    double x = (1 - u[i]) * lo + u[i] * hi;  // sig.cpp:401-406
                    (ax == 0 ? n1 : ax == 1 ? n2 : n3)[o] = x;
                } else if (ax == 0) {
                    n1[o] = std::cbrt((1 - u[i]) * (lo * lo * lo) + u[i] * (hi * hi * hi));  // sig.cpp:453-454
                } else if (ax == 1) {
                    double mu = (1 - u[i]) * lo + u[i] * hi;
                    n2[o] = mu;
                    s2[o] = std::sqrt(std::fmax(1 - mu * mu, 0.0));
                } else {
                    double phi = (1 - u[i]) * lo + u[i] * hi;
                    n3[o] = phi;
                    cp[o] = std::cos(phi);
                    sp[o] = std::sin(phi);
                }
            }
        }
    std::vector<double> all;
    size_t off_w = all.size();
    all.insert(all.end(), w_h.begin(), w_h.end());
    size_t off1 = all.size();
    all.insert(all.end(), n1.begin(), n1.end());
    size_t off2 = all.size();
    all.insert(all.end(), n2.begin(), n2.end());
    size_t offs = all.size();
    all.insert(all.end(), s2.begin(), s2.end());
    size_t off3 = all.size();
    all.insert(all.end(), n3.begin(), n3.end());
    size_t offc = all.size();
    all.insert(all.end(), cp.begin(), cp.end());
    size_t offsn = all.size();
    all.insert(all.end(), sp.begin(), sp.end());
    c->nodes.alloc(all.size());
    OPSEC_CUDA(cudaMemcpyAsync(c->nodes.p, all.data(), sizeof(double) * all.size(), cudaMemcpyHostToDevice, c->stream));
    c->Q.alloc((size_t)c->ntab() * c->ks.nkeys);
    CubatureArgs a;
    a.coordsys = g.coordsys;
    a.L = g.coordsys == 1 ? g.L : 0.0;
    a.ks = c->ks;
    a.ng = ng;
    a.np = ng * ng * ng;
    a.w = c->nodes.p + off_w;
    a.wmax = *std::max_element(w.begin(), w.end());
    a.node1 = c->nodes.p + off1;
    a.node2 = c->nodes.p + off2;
    a.snode2 = c->nodes.p + offs;
    a.node3 = c->nodes.p + off3;
    a.cphi = c->nodes.p + offc;
    a.sphi = c->nodes.p + offsn;
    a.xl = c->xl;
    a.ntab = c->ntab();
    a.tab32 = c->xi32.p;
    a.Q = c->Q.p;
    c->cubpts.alloc(8 * cubature_point_count(c->ks, ng));
    a.pts = reinterpret_cast<float4*>(c->cubpts.p);
    a.exact = c->cub_exact;
    a.window = c->cub_window;
    a.win_key = c->win_key;
    a.win_flush = c->win_flush;
    a.win_dot64 = c->win_dot64;
    if (a.exact && a.window) {
        a.work_bytes = cubature_work_bytes(c->ks, c->xl.n(), a.ntab, a.ng);
        c->cubwork.alloc(a.work_bytes);
        a.work = c->cubwork.p;
    }
    if (c->surr_on) {
        surrogate_stage(c);
        a.skip = c->surr_done.p;
    }
    launch_cubature(a, c->stream, &c->launches);
    sync(c);
    c->q_ok = true;
}

void build_qsq(opsec_gpu* c) {
    if (c->qsq_ok) return;
    build_q(c);
    c->Qsq.alloc((size_t)c->ntab() * c->ks.nsquare);
    launch_expand_q(c->ks, c->ntab(), c->Q.p, c->Qsq.p, c->stream, &c->launches);
    c->qsq_ok = true;
}

// Validate cells against the survey grid and upload their indices and Nbar.
void load_cells(opsec_gpu* c, int ncells, const opsec_cell* cells) {
    if (ncells <= 0 || !cells) fail(OPSEC_ERR_ARG, "no cells");
    const Geometry& g = c->geo;
    std::vector<int> idx((size_t)6 * ncells);
    std::vector<double> nb(ncells);
    for (int a = 0; a < ncells; a++) {
        const opsec_cell& cl = cells[a];
        if (cl.d1 < 0 || cl.d1 >= g.n[0] || cl.d2 < 0 || cl.d2 >= g.n[1] || cl.d3 < 0 || cl.d3 >= g.n[2])
            fail(OPSEC_ERR_ARG, "cell " + std::to_string(a) + " has a grid index outside the survey grid");
        if (!(cl.Nbar > 0) || !std::isfinite(cl.Nbar))
            fail(OPSEC_ERR_NUMERIC, "cell " + std::to_string(a) + " has Nbar <= 0 or non-finite");
        const double lo1 = g.b[0] + cl.d1 * (g.b[1] - g.b[0]) / g.n[0];
        const double lo3 = g.b[4] + cl.d3 * (g.b[5] - g.b[4]) / g.n[2];
        if (std::fabs(cl.min1 - lo1) > 1e-9 * (std::fabs(lo1) + std::fabs(g.b[1] - g.b[0])) ||
            std::fabs(cl.min3 - lo3) > 1e-9 * (std::fabs(lo3) + std::fabs(g.b[5] - g.b[4])))
            fail(OPSEC_ERR_CONFIG, "cell " + std::to_string(a) + " bounds do not match the survey grid");
        idx[a] = cl.d1;
        idx[ncells + a] = cl.d2;
        idx[2 * (size_t)ncells + a] = cl.d3;
        if (g.coordsys == 2) {
            idx[3 * (size_t)ncells + a] = cl.d1 * g.n[1] + cl.d2;
            idx[4 * (size_t)ncells + a] = cl.d3;
            idx[5 * (size_t)ncells + a] = 0;
        } else {
            idx[3 * (size_t)ncells + a] = cl.d1;
            idx[4 * (size_t)ncells + a] = cl.d2;
            idx[5 * (size_t)ncells + a] = cl.d3;
        }
        nb[a] = cl.Nbar;
    }
    c->cells_arc_order = g.coordsys == 2;
    for (int a = 0; a < ncells && c->cells_arc_order; a++)
        if (idx[3 * (size_t)ncells + a] * g.n[2] + idx[4 * (size_t)ncells + a] != a) c->cells_arc_order = false;
    c->cell_i.alloc(idx.size());
    c->nbar.alloc(ncells);
    OPSEC_CUDA(cudaMemcpyAsync(c->cell_i.p, idx.data(), sizeof(int) * idx.size(), cudaMemcpyHostToDevice, c->stream));
    OPSEC_CUDA(cudaMemcpyAsync(c->nbar.p, nb.data(), sizeof(double) * ncells, cudaMemcpyHostToDevice, c->stream));
    sync(c);
    c->ncells_loaded = ncells;
}

CellKeyInfo cell_info(opsec_gpu* c) {
    const size_t n = c->ncells_loaded;
    return CellKeyInfo{c->cell_i.p, c->cell_i.p + n, c->cell_i.p + 2 * n, c->nbar.p};
}

// True when S is block-circulant in phi: full-sky spherical grid, every cell
// present in grid order, Nbar constant along each arc.
bool azimuthal_ok(opsec_gpu* c, int ncells, const opsec_cell* cells) {
    const Geometry& g = c->geo;
    if (g.coordsys != 2 || !g.full_sky()) return false;
    if ((long long)ncells != (long long)g.n[0] * g.n[1] * g.n[2]) return false;
    const int Nphi = g.n[2];
    for (int a = 0; a < ncells; a++) {
        const opsec_cell& cl = cells[a];
        if ((cl.d1 * g.n[1] + cl.d2) * Nphi + cl.d3 != a) return false;
        const double ref = cells[a - cl.d3].Nbar;
        if (std::fabs(cl.Nbar - ref) > 1e-12 * ref) return false;
    }
    return true;
}

void cusolver_stream(opsec_gpu* c) {
    if (!c->solver) solver_check(cusolverDnCreate(&c->solver), "cusolverDnCreate");
    solver_check(cusolverDnSetStream(c->solver, c->stream), "cusolverDnSetStream");
}

void check_info(opsec_gpu* c, int count) {
    std::vector<int> h(count);
    OPSEC_CUDA(cudaMemcpyAsync(h.data(), c->info.p, sizeof(int) * count, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    for (int i = 0; i < count; i++)
        if (h[i] != 0) fail(OPSEC_ERR_NUMERIC, "eigensolver failed (info " + std::to_string(h[i]) + ")");
}

// Top-M eigenpairs of S into c->evals / c->modes (mode-major).  Returns nconv.
// Forget the captured batched eigensolve: called before any other solver call on the
// context, which may move the library's internal buffers the graph refers to.
void drop_eig_graph(opsec_gpu* c) {
    if (c->eig_exec) cudaGraphExecDestroy(c->eig_exec);
    destroy_mock_plans(c->mock_plans);
    c->eig_exec = nullptr;
    c->eig_key = {};
}

// The hand-written block eigensolver (blockeig.cu) on the nblk blocks of order n in c->S:
// every eigenvalue (ascending per block) into c->W, and the eigenvectors of the block
// eigenvalues that can reach the global top-M cut as columns of c->S.  kc[b] = the number of
// top eigenpairs of block b computed.  Returns false (and leaves a warning) when a check in the
// kernels failed; the caller then solves the rebuilt blocks with the library.
bool own_block_eigensolve(opsec_gpu* c, int n, int nblk, int npar, int Nphi, int M, std::vector<int>& kc) {
    const size_t nn = (size_t)n * n;
    c->bev_V.alloc((size_t)nblk * nn);
    c->bev_T.alloc((size_t)nblk * (3 * n + 1));
    double* tau = c->bev_T.p;
    double* dg = tau + (size_t)nblk * n;
    double* eg = dg + (size_t)nblk * n;
    double* scale = eg + (size_t)nblk * n;
    if (g_clock) g_clock->begin("blockeig_tridiag", c->stream, 4.0 / 3.0 * n * nn * nblk);
    launch_blockeig_tridiag(n, nblk, c->S.p, c->bev_V.p, tau, dg, eg, c->stream, &c->launches);
    if (g_clock) g_clock->end(c->stream);
    launch_blockeig_spectrum(n, nblk, dg, eg, c->W.p, scale, c->stream, &c->launches);
    std::vector<double> w((size_t)nblk * n), sc(nblk);
    OPSEC_CUDA(cudaMemcpyAsync(w.data(), c->W.p, sizeof(double) * w.size(), cudaMemcpyDeviceToHost, c->stream));
    OPSEC_CUDA(cudaMemcpyAsync(sc.data(), scale, sizeof(double) * nblk, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    // the M-th largest approximate eigenvalue, counting the (cos, sin) pairs of 0 < m < Nphi/2 twice
    std::vector<double> all;
    all.reserve((size_t)2 * nblk * n);
    double smax = 0.0;
    for (int b = 0; b < nblk; b++) {
        const int m = b / npar, mult = (m == 0 || 2 * m == Nphi) ? 1 : 2;
        smax = std::max(smax, sc[b]);
        for (int j = 0; j < n; j++)
            for (int k = 0; k < mult; k++) all.push_back(w[(size_t)b * n + j]);
    }
    const size_t mth = std::min(all.size(), (size_t)M) - 1;
    std::nth_element(all.begin(), all.begin() + mth, all.end(), std::greater<double>());
    // the FP32 bisection places every eigenvalue within ~4 eps32 of its block's scale; a
    // candidate margin of 64 eps32 of the largest scale keeps every eigenvalue that can be
    // among the top M once refined
    const double cut = all[mth] - 64.0 * FLT_EPSILON * smax;
    kc.assign(nblk, 0);
    std::vector<int> koff(nblk);
    int ktot = 0;
    for (int b = 0; b < nblk; b++) {
        int k = 0;
        while (k < n && w[(size_t)b * n + n - 1 - k] >= cut) k++;
        kc[b] = k;
        koff[b] = ktot;
        ktot += k;
    }
    c->eig_stats[1] = 1.0;
    c->eig_stats[4] = ktot;
    if (ktot == 0) return true;
    c->bev_i.alloc((size_t)3 * nblk);
    std::vector<int> hi(kc);
    hi.insert(hi.end(), koff.begin(), koff.end());
    OPSEC_CUDA(cudaMemcpyAsync(c->bev_i.p, hi.data(), sizeof(int) * 2 * nblk, cudaMemcpyHostToDevice, c->stream));
    OPSEC_CUDA(cudaMemsetAsync(c->bev_i.p + 2 * nblk, 0, sizeof(int) * nblk, c->stream));
    const size_t per = (size_t)n * ktot;
    c->bev_vec.alloc(4 * per);
    BlockEigVectors p{};
    p.n = n;
    p.nblk = nblk;
    p.ktot = ktot;
    p.kc = c->bev_i.p;
    p.koff = c->bev_i.p + nblk;
    p.status = c->bev_i.p + 2 * nblk;
    p.dg = dg;
    p.eg = eg;
    p.scale = scale;
    p.w = c->W.p;
    p.Z = c->bev_vec.p;
    p.L = p.Z + per;
    p.U = p.L + per;
    p.G = p.U + per;
    p.V = c->bev_V.p;
    p.tau = tau;
    p.out = c->S.p;
    if (g_clock) g_clock->begin("blockeig_vectors", c->stream, 2.0 * nn * ktot);
    launch_blockeig_vectors(p, c->stream, &c->launches);
    if (g_clock) g_clock->end(c->stream);
    std::vector<int> st(nblk);
    OPSEC_CUDA(cudaMemcpyAsync(st.data(), p.status, sizeof(int) * nblk, cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    for (int b = 0; b < nblk; b++)
        if (st[b]) {
            c->warning = "block eigensolver check " + std::to_string(st[b]) + " failed on block " +
                         std::to_string(b) + "; solved by cuSOLVER instead";
            c->eig_stats[1] = 0.0;
            return false;
        }
    return true;
}

// After a failed device allocation a buffer may have been released without being replaced:
// nothing cached on the device is trusted, so the next call rebuilds what it needs.
void forget_device_state(opsec_gpu* c) {
    c->q_ok = c->qsq_ok = false;
    if (!c->xi64.p || !c->xi32.p) c->tables_ok = false;
    c->az_valid = false;
    drop_eig_graph(c);
}

int eigensolve(opsec_gpu* c, int ncells, const opsec_cell* cells, int M) {
    build_q(c);
    load_cells(c, ncells, cells);
    if (M <= 0 || M > ncells) fail(OPSEC_ERR_ARG, "Nmodes must be in [1, Ncells]");
    cusolver_stream(c);
    c->evals.alloc(M);
    c->modes.alloc((size_t)M * ncells);
    c->warning.clear();
    c->az_valid = false;
    if (azimuthal_ok(c, ncells, cells)) {
        std::fill(c->eig_stats, c->eig_stats + 10, 0.0);
        c->eig_stats[0] = 1.0;
        const KeySpace& ks = c->ks;
        const int H = ks.H, Nphi = ks.N3, Nmu = ks.N2, nm = Nphi / 2 + 1;
        std::vector<double> nba(H);
        for (int h = 0; h < H; h++) nba[h] = cells[(size_t)h * Nphi].Nbar;
        c->nbar_arc = nba;
        // mu parity split: reflection-symmetric mu grid, even N_mu, Nbar symmetric under j -> N_mu-1-j
        bool par = c->az_parity && c->geo.mu_symmetric() && Nmu % 2 == 0;
        for (int h = 0; par && h < H; h++) {
            const int ph = (h / Nmu) * Nmu + (Nmu - 1 - h % Nmu);
            if (std::fabs(nba[h] - nba[ph]) > 1e-12 * nba[h]) par = false;
        }
        const int npar = par ? 2 : 1, Hb = H / npar, nblk = nm * npar;
        c->az_npar = npar;
        DevBuf<double>& d_nba = c->nba_dev;
        d_nba.alloc(H);
        OPSEC_CUDA(cudaMemcpyAsync(d_nba.p, nba.data(), sizeof(double) * H, cudaMemcpyHostToDevice, c->stream));
        c->S.alloc((size_t)nblk * Hb * Hb);
        launch_azimuthal_blocks(ks, c->Q.p, d_nba.p, nm, npar, c->S.p, c->stream, &c->launches);
        c->W.alloc((size_t)nblk * Hb);
        c->info.alloc(nblk);
        std::vector<int> own_kc;
        const bool own_try = c->az_own && blockeig_supported(Hb);
        const bool own_done = own_try && own_block_eigensolve(c, Hb, nblk, npar, Nphi, M, own_kc);
        if (!own_done) {
            if (own_try)  // the reduction overwrote the blocks: rebuild them for the library solver
                launch_azimuthal_blocks(ks, c->Q.p, d_nba.p, nm, npar, c->S.p, c->stream, &c->launches);
            int lwork = 0;
            solver_check(cusolverDnDsyevd_bufferSize(c->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, Hb,
                                                     c->S.p, Hb, c->W.p, &lwork),
                         "syevd_bufferSize");
            bool batched_done = false;
            if (c->az_batched) {
                // Batched calls over the equal-size blocks, `azimuthal.split` of them on side
                // streams at once (each is a chain of small launches, mostly latency); streams of
                // single solves if a batched call is refused.
                const int nsplit = std::max(1, std::min(c->az_split, nblk));
                cusolverDnParams_t prm = nullptr;
                solver_check(cusolverDnCreateParams(&prm), "cusolverDnCreateParams");
                std::vector<cusolverDnHandle_t> hs(nsplit, c->solver);
                if (nsplit > 1) {
                    for (int j = 0; j < nsplit; j++) {
                        if (!c->side[j]) OPSEC_CUDA(cudaStreamCreateWithFlags(&c->side[j], cudaStreamNonBlocking));
                        if (!c->side_solver[j]) solver_check(cusolverDnCreate(&c->side_solver[j]), "cusolverDnCreate");
                        solver_check(cusolverDnSetStream(c->side_solver[j], c->side[j]), "cusolverDnSetStream");
                        hs[j] = c->side_solver[j];
                    }
                    for (int j = 0; j <= nsplit; j++)
                        if (!c->side_ev[j]) OPSEC_CUDA(cudaEventCreateWithFlags(&c->side_ev[j], cudaEventDisableTiming));
                }
                std::vector<int> b0(nsplit + 1);
                for (int j = 0; j <= nsplit; j++) b0[j] = (int)((long long)j * nblk / nsplit);
                std::vector<size_t> dbytes(nsplit, 0), hbytes(nsplit, 0), doff(nsplit + 1, 0);
                cusolverStatus_t st = CUSOLVER_STATUS_SUCCESS;
                for (int j = 0; j < nsplit && st == CUSOLVER_STATUS_SUCCESS; j++) {
                    st = cusolverDnXsyevBatched_bufferSize(hs[j], prm, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                                           Hb, CUDA_R_64F, c->S.p + (size_t)b0[j] * Hb * Hb, Hb,
                                                           CUDA_R_64F, c->W.p + (size_t)b0[j] * Hb, CUDA_R_64F,
                                                           &dbytes[j], &hbytes[j], b0[j + 1] - b0[j]);
                    doff[j + 1] = doff[j] + ((std::max<size_t>(dbytes[j], 1) + 255) & ~size_t(255));
                }
                if (st == CUSOLVER_STATUS_SUCCESS) {
                    DevBuf<unsigned char>& dw = c->syev_ws;
                    dw.alloc(doff[nsplit]);
                    std::vector<std::vector<unsigned char>> hw(nsplit);
                    if (nsplit > 1) {
                        OPSEC_CUDA(cudaEventRecord(c->side_ev[nsplit], c->stream));
                        for (int j = 0; j < nsplit; j++) OPSEC_CUDA(cudaStreamWaitEvent(c->side[j], c->side_ev[nsplit], 0));
                    }
                    auto solve = [&](int j, std::vector<unsigned char>& host) {
                        host.resize(std::max<size_t>(hbytes[j], 1));
                        return cusolverDnXsyevBatched(hs[j], prm, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, Hb,
                                                      CUDA_R_64F, c->S.p + (size_t)b0[j] * Hb * Hb, Hb, CUDA_R_64F,
                                                      c->W.p + (size_t)b0[j] * Hb, CUDA_R_64F, dw.p + doff[j], dbytes[j],
                                                      host.data(), hbytes[j], c->info.p + b0[j], b0[j + 1] - b0[j]);
                    };
                    // One call is a chain of thousands of small launches, bound by their host-side
                    // cost.  When a build repeats the previous one's shapes and buffers, the call is
                    // captured once into a CUDA graph and replayed; a capture the library refuses
                    // (a host synchronisation inside) falls back to the direct call for good.
                    const std::array<size_t, 6> key{(size_t)Hb, (size_t)nblk, (size_t)c->S.p, (size_t)c->W.p,
                                                    (size_t)c->info.p, (size_t)dw.p};
                    bool done = false;
                    if (nsplit == 1 && c->eig_graph_ok && key == c->eig_key) {
                        if (!c->eig_exec) {
                            cudaGraph_t g = nullptr;
                            cudaError_t ce = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
                            cusolverStatus_t cst = CUSOLVER_STATUS_INTERNAL_ERROR;
                            if (ce == cudaSuccess) {
                                cst = solve(0, c->eig_hw);  // kept while the graph lives: it may read it
                                ce = cudaStreamEndCapture(c->stream, &g);
                            }
                            if (ce == cudaSuccess && cst == CUSOLVER_STATUS_SUCCESS && g)
                                ce = cudaGraphInstantiate(&c->eig_exec, g, 0);
                            if (g) cudaGraphDestroy(g);
                            if (ce != cudaSuccess || cst != CUSOLVER_STATUS_SUCCESS) {
                                (void)cudaGetLastError();
                                c->eig_exec = nullptr;
                                c->eig_graph_ok = false;
                            }
                        }
                        if (c->eig_exec) {
                            OPSEC_CUDA(cudaGraphLaunch(c->eig_exec, c->stream));
                            done = true;
                        }
                    }
                    if (!done) {
                        if (key != c->eig_key) drop_eig_graph(c);
                        for (int j = 0; j < nsplit && st == CUSOLVER_STATUS_SUCCESS; j++) st = solve(j, hw[j]);
                        c->eig_key = key;
                    }
                    if (nsplit > 1)
                        for (int j = 0; j < nsplit; j++) {
                            OPSEC_CUDA(cudaEventRecord(c->side_ev[j], c->side[j]));
                            OPSEC_CUDA(cudaStreamWaitEvent(c->stream, c->side_ev[j], 0));
                        }
                    sync(c);
                }
                cusolverDnDestroyParams(prm);
                batched_done = st == CUSOLVER_STATUS_SUCCESS;
                if (!batched_done)  // the blocks may have been partly overwritten: rebuild them
                    launch_azimuthal_blocks(ks, c->Q.p, d_nba.p, nm, npar, c->S.p, c->stream, &c->launches);
            }
            // the block eigenproblems are independent: spread them over side streams
            const int ns = batched_done ? 0 : std::min(nblk, c->az_streams);
            if (ns > 0) drop_eig_graph(c);
            c->work.alloc((size_t)lwork * std::max(ns, 1));
            for (int j = 0; j < ns; j++) {
                if (!c->side[j]) OPSEC_CUDA(cudaStreamCreateWithFlags(&c->side[j], cudaStreamNonBlocking));
                if (!c->side_solver[j]) solver_check(cusolverDnCreate(&c->side_solver[j]), "cusolverDnCreate");
                solver_check(cusolverDnSetStream(c->side_solver[j], c->side[j]), "cusolverDnSetStream");
            }
            for (int j = 0; j <= ns; j++)
                if (!c->side_ev[j]) OPSEC_CUDA(cudaEventCreateWithFlags(&c->side_ev[j], cudaEventDisableTiming));
            OPSEC_CUDA(cudaEventRecord(c->side_ev[ns], c->stream));
            for (int j = 0; j < ns; j++) OPSEC_CUDA(cudaStreamWaitEvent(c->side[j], c->side_ev[ns], 0));
            for (int b = 0; b < nblk && ns > 0; b++) {
                const int j = b % ns;
                solver_check(cusolverDnDsyevd(c->side_solver[j], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, Hb,
                                              c->S.p + (size_t)b * Hb * Hb, Hb, c->W.p + (size_t)b * Hb,
                                              c->work.p + (size_t)j * lwork, lwork, c->info.p + b),
                             "syevd");
            }
            for (int j = 0; j < ns; j++) {
                OPSEC_CUDA(cudaEventRecord(c->side_ev[j], c->side[j]));
                OPSEC_CUDA(cudaStreamWaitEvent(c->stream, c->side_ev[j], 0));
            }
            check_info(c, nblk);
        }
        std::vector<double> w((size_t)nblk * Hb);
        OPSEC_CUDA(cudaMemcpyAsync(w.data(), c->W.p, sizeof(double) * w.size(), cudaMemcpyDeviceToHost, c->stream));
        sync(c);
        struct Ent {
            double lam;
            int b, idx, kind;
        };
        std::vector<Ent> ent;
        ent.reserve((size_t)H * Nphi);
        for (int b = 0; b < nblk; b++) {
            const int m = b / npar;
            for (int i = 0; i < Hb; i++) {
                double lam = w[(size_t)b * Hb + i];
                if (m == 0)
                    ent.push_back({lam, b, i, 0});
                else if (2 * m == Nphi)
                    ent.push_back({lam, b, i, 3});
                else {
                    ent.push_back({lam, b, i, 1});
                    ent.push_back({lam, b, i, 2});
                }
            }
        }
        std::stable_sort(ent.begin(), ent.end(), [](const Ent& x, const Ent& y) {
            if (x.lam != y.lam) return x.lam > y.lam;
            if (x.b != y.b) return x.b < y.b;
            if (x.idx != y.idx) return x.idx < y.idx;
            return x.kind < y.kind;
        });
        if (M < (int)ent.size() && ent[M - 1].kind == 1 && ent[M].kind == 2 && ent[M].b == ent[M - 1].b &&
            ent[M].idx == ent[M - 1].idx)
            c->warning = "Nmodes splits a degenerate (cos, sin) pair of azimuthal order m=" +
                         std::to_string(ent[M].b / npar);
        std::vector<int> sel((size_t)3 * M);
        std::vector<double> ev(M);
        for (int i = 0; i < M; i++) {
            if (own_done && ent[i].idx < Hb - own_kc[ent[i].b])
                fail(OPSEC_ERR_NUMERIC, "block eigensolver: a selected eigenpair lies outside the candidates");
            sel[i] = ent[i].b;
            sel[M + i] = ent[i].idx;
            sel[2 * M + i] = ent[i].kind;
            ev[i] = ent[i].lam;
        }
        c->sel.alloc(sel.size());
        OPSEC_CUDA(cudaMemcpyAsync(c->sel.p, sel.data(), sizeof(int) * sel.size(), cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(c->evals.p, ev.data(), sizeof(double) * M, cudaMemcpyHostToDevice, c->stream));
        launch_assemble_modes(H, Nphi, Nmu, npar, M, c->sel.p, c->sel.p + M, c->sel.p + 2 * M, c->S.p, c->modes.p,
                              c->stream, &c->launches);
        sync(c);
        c->az_m.assign(sel.begin(), sel.begin() + M);
        c->az_idx.assign(sel.begin() + M, sel.begin() + 2 * M);
        c->az_kind.assign(sel.begin() + 2 * M, sel.end());
        c->az_valid = true;
        return M;
    }
    drop_eig_graph(c);
    // dense path: S in FP64, top-M by syevdx or by subspace iteration (klt.cpp:173-248 via PARPACK there)
    const int N = ncells;
    c->S.alloc((size_t)N * N);
    std::vector<int> all(N);
    for (int i = 0; i < N; i++) all[i] = i;
    c->rc.alloc(N);
    OPSEC_CUDA(cudaMemcpyAsync(c->rc.p, all.data(), sizeof(int) * N, cudaMemcpyHostToDevice, c->stream));
    launch_signal_block(c->ks, cell_info(c), c->Q.p, N, c->rc.p, N, c->rc.p, c->S.p, N, c->stream, &c->launches);
    ChfsiArgs ca = c->chfsi;
    if (!c->chfsi_guard_set) ca.guard = std::max(32, M / 4);
    const long long blk = std::min<long long>(N, ((long long)M + ca.guard + 31) / 32 * 32);
    if (c->eig_solver == "chfsi" || (c->eig_solver == "auto" && N >= kChfsiMinCells && 4 * blk <= N)) {
        if (!c->blas) blas_check(cublasCreate(&c->blas), "cublasCreate");
        ca.N = N;
        ca.M = M;
        ca.S = c->S.p;
        ca.modes = c->modes.p;
        ca.evals = c->evals.p;
        ChfsiStats st;
        chfsi_eigensolve(ca, c->blas, c->solver, c->stream, &c->launches, &st);
        const double v[10] = {2.0,   (double)st.iterations, (double)st.degree, (double)st.gemms, (double)st.block,
                              st.lo, st.hi, st.resid, (double)st.rounds, (double)st.cg_steps};
        std::copy(v, v + 10, c->eig_stats);
        return M;
    }
    std::fill(c->eig_stats, c->eig_stats + 10, 0.0);
    c->W.alloc(N);
    c->info.alloc(1);
    // the 64-bit interface: the 32-bit one's workspace count overflows from N ~ 23,000 on
    int64_t meig = 0;
    size_t wdev = 0, whost = 0;
    double vl = 0.0, vu = 0.0;
    cusolverDnParams_t prm = nullptr;
    solver_check(cusolverDnCreateParams(&prm), "cusolverDnCreateParams");
    cusolverStatus_t sst = cusolverDnXsyevdx_bufferSize(
        c->solver, prm, CUSOLVER_EIG_MODE_VECTOR, CUSOLVER_EIG_RANGE_I, CUBLAS_FILL_MODE_LOWER, N, CUDA_R_64F, c->S.p, N,
        &vl, &vu, N - M + 1, N, &meig, CUDA_R_64F, c->W.p, CUDA_R_64F, &wdev, &whost);
    if (sst == CUSOLVER_STATUS_SUCCESS) {
        c->work.alloc((wdev + sizeof(double) - 1) / sizeof(double) + 1);
        std::vector<unsigned char> hw(whost + 1);
        sst = cusolverDnXsyevdx(c->solver, prm, CUSOLVER_EIG_MODE_VECTOR, CUSOLVER_EIG_RANGE_I, CUBLAS_FILL_MODE_LOWER,
                                N, CUDA_R_64F, c->S.p, N, &vl, &vu, N - M + 1, N, &meig, CUDA_R_64F, c->W.p,
                                CUDA_R_64F, c->work.p, wdev, hw.data(), whost, c->info.p);
        if (sst == CUSOLVER_STATUS_SUCCESS) OPSEC_CUDA(cudaStreamSynchronize(c->stream));  // host workspace in use
    }
    cusolverDnDestroyParams(prm);
    solver_check(sst, "syevdx");
    check_info(c, 1);
    if (meig < M) fail(OPSEC_ERR_NUMERIC, "eigensolver returned fewer modes than requested");
    launch_reverse_modes(N, M, N, c->S.p, c->W.p, c->modes.p, c->evals.p, c->stream, &c->launches);
    sync(c);
    return M;
}

struct AzPlan {
    int H, nm, npar, nb, ncol;  // H: block size (arcs / npar)
    long long csize;
    int Kmax;
    double flops;
    const int *col_m, *col_idx, *mode_m, *mode_cls, *mode_col, *Km_dev;
    const std::vector<int>* Km;
    const std::vector<int>* base;
    const std::vector<long long>* off;
    const double* nbar_arc;
};

// C_b = A_b op B_b over `batch` equal-shape problems at fixed strides (a stride may be 0: one
// operand shared by every problem).
template <typename T>
cublasStatus_t gemm_sb(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k, const T* A,
                       int lda, long long sa, const T* B, int ldb, long long sb, T* C, int ldc, long long sc, int batch);
template <>
cublasStatus_t gemm_sb<double>(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                               const double* A, int lda, long long sa, const double* B, int ldb, long long sb,
                               double* C, int ldc, long long sc, int batch) {
    const double one = 1.0, zero = 0.0;
    return cublasDgemmStridedBatched(h, ta, tb, m, n, k, &one, A, lda, sa, B, ldb, sb, &zero, C, ldc, sc, batch);
}
template <>
cublasStatus_t gemm_sb<float>(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                              const float* A, int lda, long long sa, const float* B, int ldb, long long sb, float* C,
                              int ldc, long long sc, int batch) {
    const float one = 1.f, zero = 0.f;
    return cublasSgemmStridedBatched(h, ta, tb, m, n, k, &one, A, lda, sa, B, ldb, sb, &zero, C, ldc, sc, batch);
}

// Band blocks and block GEMMs, in FP64 or FP32, for every band: the blocks of
// up to ~2 GB of bands at a time are transformed, then for each block one
// batched GEMM over those bands forms T = S_p(b) U_b and one more
// C_b = U_b^T T.  The C_b of all bands stay in the workspace (`Cm`, csize
// floats per band) for the scatter into the packed triangle or for the block
// Fisher sums.
template <typename T>
T* az_blocks(opsec_gpu* c, const AzPlan& a) {
    const int H = a.H;
    DevBuf<unsigned char>& ws = c->azws;
    const int nblk = a.nm * a.npar;
    const size_t nU = (size_t)a.ncol * H, nS = (size_t)nblk * H * H, nT = (size_t)H * std::max(a.Kmax, 1),
                 nC = (size_t)std::max(a.csize, 1LL) * a.nb;
    const int bpp = (int)std::max<size_t>(1, std::min<size_t>(a.nb, (size_t(2) << 30) / (sizeof(T) * nS)));
    ws.alloc(sizeof(T) * (nU + nS * bpp + nT * bpp + nC));
    T* U = reinterpret_cast<T*>(ws.p);
    T* Sb = U + nU;
    T* Tm = Sb + nS * bpp;
    T* Cm = Tm + nT * bpp;
    // the block eigenvectors the modes use
    launch_gather_block_vectors(H, a.ncol, a.col_m, a.col_idx, c->S.p, U, c->stream, &c->launches);
    for (int p0 = 0; p0 < a.nb; p0 += bpp) {
        const int np = std::min(bpp, a.nb - p0);
        for (int p = p0; p < p0 + np; p++) {
            if (g_clock) g_clock->begin("azimuthal_transform", c->stream, 2.0 * nblk * (double)H * H * c->ks.nf);
            launch_azimuthal_blocks(c->ks, c->Q.p + (size_t)(1 + p) * c->ks.nkeys, a.nbar_arc, a.nm, a.npar,
                                    Sb + (size_t)(p - p0) * nS, c->stream, &c->launches);
            if (g_clock) g_clock->end(c->stream);
        }
        if (g_clock) g_clock->begin("azimuthal_gemm", c->stream, a.flops * np);
        for (int m = 0; m < nblk; m++) {
            const int K = (*a.Km)[m];
            if (K == 0) continue;
            const T* Sm = Sb + (size_t)m * H * H;
            const T* Um = U + (size_t)(*a.base)[m] * H;
            blas_check(gemm_sb<T>(c->blas, CUBLAS_OP_N, CUBLAS_OP_N, H, K, H, Sm, H, (long long)nS, Um, H, 0, Tm, H,
                                  (long long)nT, np),
                       "gemm");
            blas_check(gemm_sb<T>(c->blas, CUBLAS_OP_T, CUBLAS_OP_N, K, K, H, Um, H, 0, Tm, H, (long long)nT,
                                  Cm + (size_t)p0 * a.csize + (*a.off)[m], K, a.csize, np),
                       "gemm");
            c->launches += 2;
        }
        if (g_clock) g_clock->end(c->stream);
    }
    return Cm;
}

// Projection of a full-sky spherical build onto its own azimuthal modes.
// S_p is block circulant in phi (Q depends on |phi_a - phi_b| only and Nbar
// does not depend on phi), and every mode is U_m[:, idx] (x) a cos or sin of
// order m.  So C_p[i][j] = U_m[:, idx_i]^T S_p(m) U_m[:, idx_j] when modes i
// and j have the same order m and the same trig class, and 0 otherwise, with
// S_p(m) the H x H cosine transform of the band table (as for the eigensolve).
// Per band the transform, then per block two GEMMs T = S_p(m) U_m and
// C_m = U_m^T T (batched over the bands), then one scatter into the packed
// triangle (or, for the Fisher build, block sums that skip the triangle).
// Work per band sum_m 2 H^2 K_m + 2 H K_m^2 (K_m distinct block vectors of
// order m), against 2 N^2 M + N M^2 for the dense projection.
void project_azimuthal(opsec_gpu* c, int ncells, int M, bool packed) {
    const KeySpace& ks = c->ks;
    const int Nphi = ks.N3, nm = Nphi / 2 + 1, npar = c->az_npar, nblk = nm * npar, H = ks.H / npar;
    const int nb = c->ntab() - 1;
    // distinct (block, idx) columns, grouped by block (block = m npar + mu parity)
    std::vector<std::vector<int>> cols(nblk);
    for (int i = 0; i < M; i++) cols[c->az_m[i]].push_back(c->az_idx[i]);
    std::vector<int> col_m, col_idx, Km(nblk), base(nblk);
    std::vector<long long> off(nblk);
    long long csize = 0;
    int Kmax = 0;
    for (int m = 0; m < nblk; m++) {
        auto& v = cols[m];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        Km[m] = (int)v.size();
        base[m] = (int)col_m.size();
        off[m] = csize;
        csize += (long long)Km[m] * Km[m];
        Kmax = std::max(Kmax, Km[m]);
        for (int idx : v) {
            col_m.push_back(m);
            col_idx.push_back(idx);
        }
    }
    const int ncol = (int)col_m.size();
    std::vector<int> mode_cls(M), mode_col(M);
    for (int i = 0; i < M; i++) {
        const int m = c->az_m[i];
        mode_cls[i] = c->az_kind[i] == 2 ? 1 : 0;
        mode_col[i] = (int)(std::lower_bound(cols[m].begin(), cols[m].end(), c->az_idx[i]) - cols[m].begin());
    }
    // device tables: col_m, col_idx, mode_m, mode_cls, mode_col, Km; offsets
    std::vector<int> ti;
    ti.insert(ti.end(), col_m.begin(), col_m.end());
    ti.insert(ti.end(), col_idx.begin(), col_idx.end());
    ti.insert(ti.end(), c->az_m.begin(), c->az_m.end());
    ti.insert(ti.end(), mode_cls.begin(), mode_cls.end());
    ti.insert(ti.end(), mode_col.begin(), mode_col.end());
    ti.insert(ti.end(), Km.begin(), Km.end());
    c->az_i.alloc(ti.size());
    OPSEC_CUDA(cudaMemcpyAsync(c->az_i.p, ti.data(), sizeof(int) * ti.size(), cudaMemcpyHostToDevice, c->stream));
    c->az_off.alloc(nblk);
    OPSEC_CUDA(cudaMemcpyAsync(c->az_off.p, off.data(), sizeof(long long) * nblk, cudaMemcpyHostToDevice, c->stream));
    const int* d_col_m = c->az_i.p;
    const int* d_col_idx = d_col_m + ncol;
    const int* d_mode_m = d_col_idx + ncol;
    const int* d_mode_cls = d_mode_m + M;
    const int* d_mode_col = d_mode_cls + M;
    const int* d_Km = d_mode_col + M;
    if (!c->blas) blas_check(cublasCreate(&c->blas), "cublasCreate");
    blas_check(cublasSetStream(c->blas, c->stream), "cublasSetStream");
    std::vector<double> nba(c->nbar_arc);
    DevBuf<double>& d_nba = c->nba_dev;
    d_nba.alloc(nba.size());
    OPSEC_CUDA(cudaMemcpyAsync(d_nba.p, nba.data(), sizeof(double) * nba.size(), cudaMemcpyHostToDevice, c->stream));
    double fl = 0;
    for (int m = 0; m < nblk; m++) fl += 2.0 * H * H * Km[m] + 2.0 * H * (double)Km[m] * Km[m];
    AzPlan plan{H, nm, npar, nb, ncol, csize, Kmax, fl, d_col_m, d_col_idx, d_mode_m, d_mode_cls, d_mode_col, d_Km, &Km,
                &base, &off, d_nba.p};
    c->az_blockF = false;
    if (!packed && !c->az_gemm64) {
        // the Fisher sums read the block matrices directly: groups (block, trig class)
        // of ascending modes and their pair counts
        std::vector<std::vector<int>> gm((size_t)nblk * 2);
        for (int i = 0; i < M; i++) gm[(size_t)c->az_m[i] * 2 + mode_cls[i]].push_back(i);
        std::vector<int> g_mode{0}, g_blk, modes;
        std::vector<long long> g_entry{0};
        for (size_t g = 0; g < gm.size(); g++) {
            if (gm[g].empty()) continue;
            const long long n = (long long)gm[g].size();
            g_entry.push_back(g_entry.back() + n * (n + 1) / 2);
            g_blk.push_back((int)(g / 2));
            modes.insert(modes.end(), gm[g].begin(), gm[g].end());
            g_mode.push_back((int)modes.size());
        }
        const int G = (int)g_blk.size();
        std::vector<int> bi;
        bi.insert(bi.end(), g_mode.begin(), g_mode.end());
        bi.insert(bi.end(), g_blk.begin(), g_blk.end());
        bi.insert(bi.end(), modes.begin(), modes.end());
        c->bf_i.alloc(bi.size());
        OPSEC_CUDA(cudaMemcpyAsync(c->bf_i.p, bi.data(), sizeof(int) * bi.size(), cudaMemcpyHostToDevice, c->stream));
        c->bf_l.alloc(g_entry.size());
        OPSEC_CUDA(cudaMemcpyAsync(c->bf_l.p, g_entry.data(), sizeof(long long) * g_entry.size(),
                                   cudaMemcpyHostToDevice, c->stream));
        BlockFisherArgs& b = c->bf;
        b.ngroups = G;
        b.g_entry = c->bf_l.p;
        b.g_mode = c->bf_i.p;
        b.g_blk = c->bf_i.p + (G + 1);
        b.modes = c->bf_i.p + (G + 1) + G;
        b.mode_col = d_mode_col;
        b.Km = d_Km;
        b.off = c->az_off.p;
        b.csize = csize;
        b.C = az_blocks<float>(c, plan);
        c->bf_entries = g_entry.back();
        c->az_blockF = true;
        return;
    }
    const size_t Kp = (size_t)M * (M + 1) / 2;
    c->Dp.alloc(Kp * nb);
    if (c->az_gemm64) {
        const double* Cm = az_blocks<double>(c, plan);
        launch_azimuthal_scatter(M, nb, d_mode_m, d_mode_cls, d_mode_col, c->az_off.p, d_Km, csize, Cm, c->Dp.p,
                                 c->stream, &c->launches);
    } else {
        const float* Cm = az_blocks<float>(c, plan);
        launch_azimuthal_scatter(M, nb, d_mode_m, d_mode_cls, d_mode_col, c->az_off.p, d_Km, csize, Cm, c->Dp.p,
                                 c->stream, &c->launches);
    }
    (void)ncells;
}

// packed = false: the caller needs only the Fisher sums, which on the azimuthal
// path then read the block matrices (az_blockF) instead of the packed triangle.
void project_all(opsec_gpu* c, int ncells, int M, bool own_modes, bool packed = true) {
    c->az_blockF = false;
    if (own_modes && c->az_valid && (c->projection == "auto" || c->projection == "azimuthal")) {
        project_azimuthal(c, ncells, M, packed);
        return;
    }
    if (c->projection == "azimuthal")
        fail(OPSEC_ERR_CONFIG, "projection=azimuthal needs a full-sky spherical build on its own modes");
    build_qsq(c);
    const int nb = c->ntab() - 1;
    c->Bs.alloc((size_t)M * ncells);
    launch_scale_modes(ncells, M, c->modes.p, c->nbar.p, c->Bs.p, c->stream, &c->launches);
    const size_t K = (size_t)M * (M + 1) / 2;
    c->Dp.alloc(K * nb);
    ProjectArgs a;
    a.ks = c->ks;
    a.ncells = ncells;
    a.nmodes = M;
    a.nbands = nb;
    a.cell_h = c->cell_i.p + 3 * (size_t)ncells;
    a.cell_f = c->cell_i.p + 4 * (size_t)ncells;
    a.cell_g = c->cell_i.p + 5 * (size_t)ncells;
    a.Qsq = c->Qsq.p;
    a.Bs = c->Bs.p;
    a.Dp = c->Dp.p;
    a.chunk = c->proj_chunk;
    a.wait_cycles = c->proj_wait;
    const int n3 = c->ks.N3;
    if (c->proj_arcs && c->cells_arc_order && (n3 == 16 || n3 == 32 || n3 == 64)) a.arc_run = n3;
    bool tc = (c->projection != "simt") && project_tc_supported(a);
    if (c->projection == "tc" && !tc) fail(OPSEC_ERR_CONFIG, "projection=tc requested but the shape is not supported");
    size_t wb = tc ? project_tc_work_bytes(a) : sizeof(float) * (size_t)M * ncells;
    c->pwork.alloc(wb);
    a.work = c->pwork.p;
    a.work_bytes = wb;
    if (tc)
        launch_project_tc(a, c->stream, &c->launches);
    else
        launch_project_simt(a, c->stream, &c->launches);
}

std::vector<double> priors(opsec_gpu* c) {
    // RealModel::GetParam: mean of P(k) on 256 midpoints of the band (RealModel.cpp:85-96)
    std::vector<double> b, cc, d;
    cspline_coeffs(c->pk_k, c->pk_P, b, cc, d);
    const int N = (int)c->pk_k.size();
    const double* X = c->pk_k.data();
    std::vector<double> p(c->band_lo.size());
    for (size_t n = 0; n < p.size(); n++) {
        double sum = 0;
        for (int i = 0; i < 256; i++) {
            double k = c->band_lo[n] + (i + 0.5) * (c->band_hi[n] - c->band_lo[n]) / 256;
            double v = 0;
            if (!(k < X[0] || k >= X[N - 1])) {
                int j = lookup_index(k, N, X);
                double u = k - X[j];
                v = c->pk_P[j] + b[j] * u + cc[j] * u * u + d[j] * u * u * u;
            }
            sum += v;
        }
        p[n] = sum / 256;
    }
    return p;
}

// F, f, q then the epilogue; records copied to the host outputs
void fisher_and_epilogue(opsec_gpu* c, int M, const float* Dp32, const double* Dp64, int mixing, double* phat,
                         double* pcov, double* F, double* W, double* Mx, double* q, double* f) {
    const int nb = c->ntab() - 1;
    std::vector<double> pr = priors(c);
    c->prior.alloc(nb);
    OPSEC_CUDA(cudaMemcpyAsync(c->prior.p, pr.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, c->stream));
    FisherArgs a;
    a.nmodes = M;
    a.nbands = nb;
    a.Dp = Dp32;
    a.evals = c->evals.p;
    a.y = c->y.p;
    a.prior = c->prior.p;
    a.nblocks = fisher_blocks(M);
    const int nout = nb * (nb + 1) / 2 + 2 * nb;
    c->partial.alloc((size_t)a.nblocks * nout);
    a.partial = c->partial.p;
    c->fout.alloc((size_t)nb * nb + 2 * nb);
    a.out = c->fout.p;
    if (Dp64) {
        launch_fisher64(a, Dp64, c->stream, &c->launches);
    } else if (Dp32) {
        launch_fisher(a, c->stream, &c->launches);
    } else {
        if (!c->az_blockF) fail(OPSEC_ERR_ARG, "no derivative matrices for the Fisher sums");
        a.nblocks = fisher_blocks_for(c->bf_entries);
        c->partial.alloc((size_t)a.nblocks * nout);
        a.partial = c->partial.p;
        launch_fisher_blocks(a, c->bf, c->bf_entries, c->stream, &c->launches);
    }
    const size_t nrec = (size_t)nb + 4 * (size_t)nb * nb + 2 * nb;
    c->est.alloc(nrec);
    c->status.alloc(1);
    launch_epilogue(nb, mixing, c->fout.p, c->est.p, c->status.p, c->stream, &c->launches);
    std::vector<double> h(nrec);
    int st = 0;
    OPSEC_CUDA(cudaMemcpyAsync(h.data(), c->est.p, sizeof(double) * nrec, cudaMemcpyDeviceToHost, c->stream));
    OPSEC_CUDA(cudaMemcpyAsync(&st, c->status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    sync(c);
    if (st != 0) fail(OPSEC_ERR_NUMERIC, "Fisher matrix is singular");
    const size_t n2 = (size_t)nb * nb;
    const double* src = h.data();
    if (phat) std::memcpy(phat, src, sizeof(double) * nb);
    src += nb;
    if (pcov) std::memcpy(pcov, src, sizeof(double) * n2);
    src += n2;
    if (F) std::memcpy(F, src, sizeof(double) * n2);
    src += n2;
    if (W) std::memcpy(W, src, sizeof(double) * n2);
    src += n2;
    if (Mx) std::memcpy(Mx, src, sizeof(double) * n2);
    src += n2;
    if (q) std::memcpy(q, src, sizeof(double) * nb);
    src += nb;
    if (f) std::memcpy(f, src, sizeof(double) * nb);
}

struct StageTimer {
    opsec_gpu* c;
    cudaEvent_t ev[6];
    int n = 0;
    explicit StageTimer(opsec_gpu* cc) : c(cc) {
        for (auto& e : ev) OPSEC_CUDA(cudaEventCreate(&e));
    }
    void mark() { OPSEC_CUDA(cudaEventRecord(ev[n++], c->stream)); }
    void finish() {
        OPSEC_CUDA(cudaEventSynchronize(ev[n - 1]));
        for (int i = 0; i + 1 < n && i < 5; i++) {
            float ms = 0;
            OPSEC_CUDA(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
            c->stage_ms[i] = ms;
        }
    }
    ~StageTimer() {
        for (auto& e : ev) cudaEventDestroy(e);
    }
};

}  // namespace

// ---------------------------------------------------------------- C ABI
extern "C" {

int opsec_gpu_create(opsec_gpu** out, const char* cfg_text) {
    if (!out) return OPSEC_ERR_ARG;
    *out = nullptr;
    opsec_gpu* c = new (std::nothrow) opsec_gpu();
    if (!c) return OPSEC_ERR_NOMEM;
    c->device = -1;
    int rc = guard(c, [&] {
        // the configuration first (host only: its errors do not depend on a device), then the device
        configure(c, parse_config(cfg_text));
        c->cfg_text = cfg_text ? cfg_text : "";
        int dev = 0;
        OPSEC_CUDA(cudaGetDevice(&dev));
        c->device = dev;
        OPSEC_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    });
    *out = c;  // returned even on error so that opsec_gpu_last_error can report it
    return rc;
}

int opsec_gpu_set_pk(opsec_gpu* c, int n, const double* k, const double* P) {
    return guard(c, [&] {
        if (n < 2 || !k || !P) fail(OPSEC_ERR_ARG, "P(k) needs at least two points");
        for (int i = 0; i < n; i++) {
            if (!std::isfinite(k[i]) || !std::isfinite(P[i])) fail(OPSEC_ERR_NUMERIC, "P(k) has non-finite values");
            if (i && !(k[i] > k[i - 1])) fail(OPSEC_ERR_ARG, "P(k) abscissae must increase");
        }
        c->pk_k.assign(k, k + n);
        c->pk_P.assign(P, P + n);
        c->tables_ok = c->q_ok = c->qsq_ok = false;
        c->custom_xi = false;
    });
}

int opsec_gpu_set_xi_table(opsec_gpu* c, int table, int n, const double* values) {
    return guard(c, [&] {
        if (table < 0 || table >= c->ntab()) fail(OPSEC_ERR_ARG, "table index out of range");
        if (n != c->xl.n() || !values) fail(OPSEC_ERR_ARG, "table length must equal xi.n1 + xi.n2");
        for (int i = 0; i < n; i++)
            if (!std::isfinite(values[i])) fail(OPSEC_ERR_NUMERIC, "non-finite xi value");
        build_tables(c);
        std::vector<float> v32(values, values + n);
        OPSEC_CUDA(cudaMemcpyAsync(c->xi64.p + (size_t)table * n, values, sizeof(double) * n, cudaMemcpyHostToDevice,
                                   c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(c->xi32.p + (size_t)table * n, v32.data(), sizeof(float) * n, cudaMemcpyHostToDevice,
                                   c->stream));
        sync(c);
        c->custom_xi = true;
        c->q_ok = c->qsq_ok = false;
    });
}

int opsec_gpu_num_params(opsec_gpu* c, int* np) {
    return guard(c, [&] {
        if (!np) fail(OPSEC_ERR_ARG, "null output");
        *np = (int)c->band_lo.size();
    });
}

int opsec_gpu_get_params(opsec_gpu* c, double* p) {
    return guard(c, [&] {
        if (!p) fail(OPSEC_ERR_ARG, "null output");
        if (c->pk_k.size() < 2) fail(OPSEC_ERR_STATE, "no P(k)");
        std::vector<double> v = priors(c);
        std::memcpy(p, v.data(), sizeof(double) * v.size());
    });
}

int opsec_gpu_xi_tables(opsec_gpu* c, int* n, double* r_out, double* xi_out) {
    return guard(c, [&] {
        build_tables(c);
        const int nx = c->xl.n();
        if (n) *n = nx;
        if (r_out) OPSEC_CUDA(cudaMemcpyAsync(r_out, c->r_grid.p, sizeof(double) * nx, cudaMemcpyDeviceToHost, c->stream));
        if (xi_out)
            OPSEC_CUDA(cudaMemcpyAsync(xi_out, c->xi64.p, sizeof(double) * nx * c->ntab(), cudaMemcpyDeviceToHost,
                                       c->stream));
        sync(c);
    });
}

int opsec_gpu_signal_block(opsec_gpu* c, int ncells, const opsec_cell* cells, int nrows, const int* rows, int ncols,
                           const int* cols, double* s, int lld, int table) {
    return guard(c, [&] {
        if (nrows < 0 || ncols < 0 || (nrows && !rows) || (ncols && !cols) || (nrows && ncols && !s))
            fail(OPSEC_ERR_ARG, "invalid block arguments");
        if (lld <= 0) lld = ncols;
        if (lld < ncols) fail(OPSEC_ERR_ARG, "lld < ncols");  // sig.cpp:57-61
        if (table < 0 || table >= c->ntab()) fail(OPSEC_ERR_ARG, "table index out of range");
        for (int i = 0; i < nrows; i++)
            if (rows[i] < 0 || rows[i] >= ncells) fail(OPSEC_ERR_ARG, "row index out of range");
        for (int j = 0; j < ncols; j++)
            if (cols[j] < 0 || cols[j] >= ncells) fail(OPSEC_ERR_ARG, "column index out of range");
        if (nrows == 0 || ncols == 0) return;
        build_q(c);
        load_cells(c, ncells, cells);
        c->rc.alloc((size_t)nrows + ncols);
        OPSEC_CUDA(cudaMemcpyAsync(c->rc.p, rows, sizeof(int) * nrows, cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(c->rc.p + nrows, cols, sizeof(int) * ncols, cudaMemcpyHostToDevice, c->stream));
        c->sblock.alloc((size_t)nrows * lld);
        launch_signal_block(c->ks, cell_info(c), c->Q.p + (size_t)table * c->ks.nkeys, nrows, c->rc.p, ncols,
                            c->rc.p + nrows, c->sblock.p, lld, c->stream, &c->launches);
        OPSEC_CUDA(cudaMemcpyAsync(s, c->sblock.p, sizeof(double) * ((size_t)(nrows - 1) * lld + ncols),
                                   cudaMemcpyDeviceToHost, c->stream));
        sync(c);
    });
}

int opsec_gpu_klt(opsec_gpu* c, int ncells, const opsec_cell* cells, int nmodes, double* evals, double* modes,
                  int* nconv) {
    return guard(c, [&] {
        int n = eigensolve(c, ncells, cells, nmodes);
        if (evals) OPSEC_CUDA(cudaMemcpyAsync(evals, c->evals.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        if (modes)
            OPSEC_CUDA(cudaMemcpyAsync(modes, c->modes.p, sizeof(double) * (size_t)n * ncells, cudaMemcpyDeviceToHost,
                                       c->stream));
        sync(c);
        if (nconv) *nconv = n;
    });
}

int opsec_gpu_comma(opsec_gpu* c, int ncells, const opsec_cell* cells, int nmodes, const double* modes,
                    double* cov_packed) {
    return guard(c, [&] {
        if (nmodes <= 0 || nmodes > ncells || !modes || !cov_packed) fail(OPSEC_ERR_ARG, "invalid comma arguments");
        build_qsq(c);
        load_cells(c, ncells, cells);
        c->modes.alloc((size_t)nmodes * ncells);
        OPSEC_CUDA(cudaMemcpyAsync(c->modes.p, modes, sizeof(double) * (size_t)nmodes * ncells, cudaMemcpyHostToDevice,
                                   c->stream));
        project_all(c, ncells, nmodes, false);
        const size_t K = (size_t)nmodes * (nmodes + 1) / 2, tot = K * (c->ntab() - 1);
        c->Dp64.alloc(tot);
        launch_widen(tot, c->Dp.p, c->Dp64.p, c->stream, &c->launches);
        OPSEC_CUDA(cudaMemcpyAsync(cov_packed, c->Dp64.p, sizeof(double) * tot, cudaMemcpyDeviceToHost, c->stream));
        sync(c);
    });
}

int opsec_gpu_dot(opsec_gpu* c, int ncells, const opsec_cell* cells, const double* counts, int nmodes,
                  const double* modes, double* y) {
    return guard(c, [&] {
        if (nmodes <= 0 || !counts || !modes || !y) fail(OPSEC_ERR_ARG, "invalid dot arguments");
        load_cells(c, ncells, cells);
        c->modes.alloc((size_t)nmodes * ncells);
        c->counts.alloc(ncells);
        c->y.alloc(nmodes);
        OPSEC_CUDA(cudaMemcpyAsync(c->modes.p, modes, sizeof(double) * (size_t)nmodes * ncells, cudaMemcpyHostToDevice,
                                   c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(c->counts.p, counts, sizeof(double) * ncells, cudaMemcpyHostToDevice, c->stream));
        launch_dot(ncells, nmodes, c->modes.p, c->counts.p, c->nbar.p, c->y.p, c->stream, &c->launches);
        OPSEC_CUDA(cudaMemcpyAsync(y, c->y.p, sizeof(double) * nmodes, cudaMemcpyDeviceToHost, c->stream));
        sync(c);
    });
}

int opsec_gpu_count_galaxies(opsec_gpu* c, int ncells, const opsec_cell* cells, long long ngal, const float* gals,
                             double* counts, double* outside) {
    return guard(c, [&] {
        const Geometry& g = c->geo;
        const long long grid = (long long)g.n[0] * g.n[1] * g.n[2];
        if (ncells <= 0 || !cells || !counts || ngal < 0 || (ngal > 0 && !gals) || grid <= 0)
            fail(OPSEC_ERR_ARG, "invalid galaxy-count arguments");
        // grid index -> cell (dot.cpp:105-117)
        std::vector<int> map((size_t)grid, -1);
        for (int a = 0; a < ncells; a++) {
            const opsec_cell& e = cells[a];
            if (e.d1 < 0 || e.d1 >= g.n[0] || e.d2 < 0 || e.d2 >= g.n[1] || e.d3 < 0 || e.d3 >= g.n[2])
                fail(OPSEC_ERR_ARG, "cell " + std::to_string(a) + " lies outside the survey grid");
            map[((size_t)e.d1 * g.n[1] + e.d2) * g.n[2] + e.d3] = a;
        }
        DevBuf<int> d_map;
        DevBuf<double> d_counts;
        DevBuf<float> d_gal;
        d_map.alloc((size_t)grid);
        d_counts.alloc((size_t)ncells + 1);
        d_gal.alloc((size_t)4 * std::max<long long>(ngal, 1));
        OPSEC_CUDA(cudaMemcpyAsync(d_map.p, map.data(), sizeof(int) * map.size(), cudaMemcpyHostToDevice, c->stream));
        if (ngal > 0)
            OPSEC_CUDA(cudaMemcpyAsync(d_gal.p, gals, sizeof(float) * 4 * (size_t)ngal, cudaMemcpyHostToDevice,
                                       c->stream));
        GridBox box;
        for (int ax = 0; ax < 3; ax++) {
            box.lo[ax] = g.b[2 * ax];
            box.hi[ax] = g.b[2 * ax + 1];
            box.n[ax] = g.n[ax];
        }
        launch_galaxy_counts(ngal, reinterpret_cast<const float4*>(d_gal.p), box, d_map.p, ncells, d_counts.p,
                             c->stream, &c->launches);
        OPSEC_CUDA(cudaMemcpyAsync(counts, d_counts.p, sizeof(double) * ncells, cudaMemcpyDeviceToHost, c->stream));
        double out = 0.0;
        OPSEC_CUDA(cudaMemcpyAsync(&out, d_counts.p + ncells, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        sync(c);
        if (outside) *outside = out;
    });
}

int opsec_gpu_set_radial(opsec_gpu* c, int n, const double* r, const double* nbar) {
    return guard(c, [&] {
        if (n < 2 || !r || !nbar) fail(OPSEC_ERR_ARG, "the radial selection needs at least two points");
        for (int i = 0; i < n; i++) {
            if (!std::isfinite(r[i]) || !std::isfinite(nbar[i])) fail(OPSEC_ERR_NUMERIC, "non-finite radial selection");
            if (i && !(r[i] > r[i - 1])) fail(OPSEC_ERR_ARG, "radial selection abscissae must increase");
        }
        c->rad_r.assign(r, r + n);
        c->rad_n.assign(nbar, nbar + n);
    });
}

int opsec_gpu_set_mask(opsec_gpu* c, long long nside, int nest, const float* mask) {
    return guard(c, [&] {
        if (nside == 0) {
            c->mask_nside = 0;
            return;
        }
        if (nside < 1 || nside > 8192 || (nest && (nside & (nside - 1)))) fail(OPSEC_ERR_ARG, "invalid HEALPix nside");
        if (!mask) fail(OPSEC_ERR_ARG, "no map");
        const size_t npix = (size_t)12 * nside * nside;
        for (size_t i = 0; i < npix; i++)
            if (!std::isfinite(mask[i])) fail(OPSEC_ERR_NUMERIC, "non-finite map value");
        c->mask_dev.alloc(npix);
        OPSEC_CUDA(cudaMemcpyAsync(c->mask_dev.p, mask, sizeof(float) * npix, cudaMemcpyHostToDevice, c->stream));
        sync(c);
        c->mask_nside = nside;
        c->mask_nest = nest ? 1 : 0;
    });
}

int opsec_gpu_ang2pix(opsec_gpu* c, long long nside, int nest, int n, const double* theta, const double* phi,
                      long long* pix) {
    return guard(c, [&] {
        if (nside < 1 || nside > 8192 || (nest && (nside & (nside - 1))) || n < 0 || (n && (!theta || !phi || !pix)))
            fail(OPSEC_ERR_ARG, "invalid ang2pix arguments");
        if (n == 0) return;
        DevBuf<double> in;
        DevBuf<long long> out;
        in.alloc((size_t)2 * n);
        out.alloc(n);
        OPSEC_CUDA(cudaMemcpyAsync(in.p, theta, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(in.p + n, phi, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        launch_ang2pix(nside, nest, n, in.p, in.p + n, out.p, c->stream, &c->launches);
        OPSEC_CUDA(cudaMemcpyAsync(pix, out.p, sizeof(long long) * n, cudaMemcpyDeviceToHost, c->stream));
        sync(c);
    });
}

int opsec_gpu_basis(opsec_gpu* c, int capacity, opsec_cell* cells, int* ncells) {
    return guard(c, [&] {
        const Geometry& g = c->geo;
        const long long total = (long long)g.n[0] * g.n[1] * g.n[2];
        if (!ncells || (capacity > 0 && !cells) || total <= 0 || total > (1LL << 31) - 1)
            fail(OPSEC_ERR_ARG, "invalid basis arguments");
        if (g.coordsys == 1 && !(c->sel_nbar > 0)) fail(OPSEC_ERR_CONFIG, "survey.nbar must be > 0 (constant selection)");
        if (g.coordsys == 2 && c->rad_r.size() < 2) fail(OPSEC_ERR_STATE, "no radial selection: call opsec_gpu_set_radial");
        // cell bounds as Survey::CreateEmptyCell (Survey.cpp:80-97), grid order d1, d2, d3
        std::vector<double> bounds((size_t)6 * total);
        long long k = 0;
        for (int d1 = 0; d1 < g.n[0]; d1++)
            for (int d2 = 0; d2 < g.n[1]; d2++)
                for (int d3 = 0; d3 < g.n[2]; d3++, k++) {
                    const int dd[3] = {d1, d2, d3};
                    for (int ax = 0; ax < 3; ax++) {
                        const double lo = g.b[2 * ax], hi = g.b[2 * ax + 1];
                        bounds[6 * k + 2 * ax] = lo + dd[ax] * (hi - lo) / g.n[ax];
                        bounds[6 * k + 2 * ax + 1] = lo + (dd[ax] + 1) * (hi - lo) / g.n[ax];
                    }
                }
        DevBuf<double> dev;
        dev.alloc((size_t)6 * total + 2 * total + 2 * c->rad_r.size());
        double* d_bounds = dev.p;
        double* d_out = dev.p + 6 * total;
        double* d_rad = d_out + 2 * total;
        OPSEC_CUDA(cudaMemcpyAsync(d_bounds, bounds.data(), sizeof(double) * bounds.size(), cudaMemcpyHostToDevice,
                                   c->stream));
        const int nr = (int)c->rad_r.size();
        if (nr) {
            OPSEC_CUDA(cudaMemcpyAsync(d_rad, c->rad_r.data(), sizeof(double) * nr, cudaMemcpyHostToDevice, c->stream));
            OPSEC_CUDA(cudaMemcpyAsync(d_rad + nr, c->rad_n.data(), sizeof(double) * nr, cudaMemcpyHostToDevice,
                                       c->stream));
        }
        BasisArgs b;
        b.coordsys = g.coordsys;
        for (int ax = 0; ax < 3; ax++) b.n[ax] = g.n[ax];
        b.bounds = d_bounds;
        b.nbar = c->sel_nbar;
        b.nrad = nr;
        b.rad_r = d_rad;
        b.rad_n = d_rad + nr;
        b.nside = c->mask_nside;
        b.nest = c->mask_nest;
        b.mask = c->mask_dev.p;
        b.samples = c->basis_samples;
        b.quirk3 = c->basis_quirk3;
        b.out = d_out;
        launch_basis(b, c->stream, &c->launches);
        std::vector<double> out((size_t)2 * total);
        OPSEC_CUDA(cudaMemcpyAsync(out.data(), d_out, sizeof(double) * out.size(), cudaMemcpyDeviceToHost, c->stream));
        sync(c);
        // keep the cells whose Nbar is positive (basis.cpp:118-127), numbered in grid order
        int kept = 0;
        k = 0;
        for (int d1 = 0; d1 < g.n[0]; d1++)
            for (int d2 = 0; d2 < g.n[1]; d2++)
                for (int d3 = 0; d3 < g.n[2]; d3++, k++) {
                    if (!(out[2 * k + 1] > 0)) continue;
                    if (kept < capacity) {
                        opsec_cell& e = cells[kept];
                        e.a = kept;
                        e.d1 = d1;
                        e.d2 = d2;
                        e.d3 = d3;
                        e.min1 = bounds[6 * k];
                        e.max1 = bounds[6 * k + 1];
                        e.min2 = bounds[6 * k + 2];
                        e.max2 = bounds[6 * k + 3];
                        e.min3 = bounds[6 * k + 4];
                        e.max3 = bounds[6 * k + 5];
                        e.Veff = out[2 * k];
                        e.Nbar = out[2 * k + 1];
                    }
                    ++kept;
                }
        *ncells = kept;
        if (kept > capacity && capacity > 0) fail(OPSEC_ERR_ARG, "cell array too small: " + std::to_string(kept) + " cells");
    });
}

int opsec_gpu_mock_counts(opsec_gpu* c, int ncells, const opsec_cell* cells, int ngrid, unsigned long long seed,
                          double bias, double* counts, double* delta) {
    return guard(c, [&] {
        if (ncells <= 0 || !cells || !counts) fail(OPSEC_ERR_ARG, "invalid mock arguments");
        if (ngrid < 4 || ngrid > 1024 || ngrid % 2) fail(OPSEC_ERR_ARG, "ngrid must be even, in [4, 1024]");
        if (!std::isfinite(bias)) fail(OPSEC_ERR_ARG, "bias must be finite");
        build_tables(c);  // uploads the P(k) spline
        // cell centres (Cartesian, or (r, mu, phi) mapped to x, y, z), the enclosing periodic
        // mesh (side 1.25 x the span of the centres plus a margin of 1) and each centre's mesh point
        std::vector<double> xyz((size_t)3 * ncells), nb(ncells);
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int a = 0; a < ncells; a++) {
            const opsec_cell& e = cells[a];
            const double c1 = 0.5 * (e.min1 + e.max1), c2 = 0.5 * (e.min2 + e.max2), c3 = 0.5 * (e.min3 + e.max3);
            double x[3] = {c1, c2, c3};
            if (c->geo.coordsys == 2) {
                const double st = std::sqrt(std::fmax(1.0 - c2 * c2, 0.0));
                x[0] = c1 * st * std::cos(c3);
                x[1] = c1 * st * std::sin(c3);
                x[2] = c1 * c2;
            }
            for (int d = 0; d < 3; d++) {
                xyz[(size_t)3 * a + d] = x[d];
                lo[d] = std::fmin(lo[d], x[d]);
                hi[d] = std::fmax(hi[d], x[d]);
            }
            if (!std::isfinite(e.Nbar) || e.Nbar < 0) fail(OPSEC_ERR_NUMERIC, "Nbar must be finite and >= 0");
            nb[a] = e.Nbar;
        }
        double span = 0.0;
        for (int d = 0; d < 3; d++) {
            lo[d] -= 1.0;
            span = std::fmax(span, hi[d] - lo[d]);
        }
        const double box = (span + 1.0) * 1.25, h = box / ngrid;
        std::vector<long long> idx(ncells);
        for (int a = 0; a < ncells; a++) {
            long long m[3];
            for (int d = 0; d < 3; d++) {
                long long v = (long long)std::floor((xyz[(size_t)3 * a + d] - lo[d]) / h) % ngrid;
                m[d] = v < 0 ? v + ngrid : v;
            }
            idx[a] = (m[0] * ngrid + m[1]) * ngrid + m[2];
        }
        const long long npts = (long long)ngrid * ngrid * ngrid;
        c->mock_grid.alloc(npts);
        c->mock_spec.alloc((size_t)2 * ngrid * ngrid * (ngrid / 2 + 1));
        c->mock_idx.alloc(ncells);
        c->mock_nbar.alloc(ncells);
        c->mock_out.alloc((size_t)2 * ncells);
        OPSEC_CUDA(cudaMemcpyAsync(c->mock_idx.p, idx.data(), sizeof(long long) * ncells, cudaMemcpyHostToDevice,
                                   c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(c->mock_nbar.p, nb.data(), sizeof(double) * ncells, cudaMemcpyHostToDevice,
                                   c->stream));
        MockArgs m;
        m.ngrid = ngrid;
        m.box = box;
        m.seed = seed;
        m.bias = bias;
        m.npk = (int)c->pk_k.size();
        m.pk = c->pk_dev.p;
        m.grid = c->mock_grid.p;
        m.spec = reinterpret_cast<double2*>(c->mock_spec.p);
        m.ncells = ncells;
        m.idx = c->mock_idx.p;
        m.nbar = c->mock_nbar.p;
        m.counts = c->mock_out.p;
        m.delta = c->mock_out.p + ncells;
        launch_mock_counts(m, c->mock_plans, c->stream, &c->launches);
        OPSEC_CUDA(cudaMemcpyAsync(counts, m.counts, sizeof(double) * ncells, cudaMemcpyDeviceToHost, c->stream));
        if (delta) OPSEC_CUDA(cudaMemcpyAsync(delta, m.delta, sizeof(double) * ncells, cudaMemcpyDeviceToHost, c->stream));
        sync(c);
    });
}

int opsec_gpu_estimate(opsec_gpu* c, int nmodes, const double* evals, const double* cov_packed, const double* y,
                       int mixing, double* phat, double* pcov, double* F, double* W, double* M, double* q, double* f) {
    return guard(c, [&] {
        if (nmodes <= 0 || !evals || !cov_packed || !y) fail(OPSEC_ERR_ARG, "invalid estimate arguments");
        if (mixing < 0 || mixing > 2) fail(OPSEC_ERR_ARG, "invalid mixing");
        if (c->pk_k.size() < 2) fail(OPSEC_ERR_STATE, "no P(k): the prior band powers need it");
        const int nb = c->ntab() - 1;
        const size_t K = (size_t)nmodes * (nmodes + 1) / 2;
        c->evals.alloc(nmodes);
        c->y.alloc(nmodes);
        c->Dp64.alloc(K * nb);
        OPSEC_CUDA(cudaMemcpyAsync(c->evals.p, evals, sizeof(double) * nmodes, cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(c->y.p, y, sizeof(double) * nmodes, cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(c->Dp64.p, cov_packed, sizeof(double) * K * nb, cudaMemcpyHostToDevice, c->stream));
        fisher_and_epilogue(c, nmodes, nullptr, c->Dp64.p, mixing, phat, pcov, F, W, M, q, f);
    });
}

int opsec_gpu_fisher_build(opsec_gpu* c, int ncells, const opsec_cell* cells, const double* counts, int nmodes,
                           int mixing, double* evals, double* phat, double* pcov, double* F, double* W, double* M,
                           double* q, double* f) {
    return guard(c, [&] {
        if (!counts) fail(OPSEC_ERR_ARG, "null counts");
        if (mixing < 0 || mixing > 2) fail(OPSEC_ERR_ARG, "invalid mixing");
        for (int a = 0; a < ncells; a++)
            if (!std::isfinite(counts[a])) fail(OPSEC_ERR_NUMERIC, "non-finite count");
        // every stage is recomputed: nothing cached from an earlier call is reused
        // (tables replaced by the caller are inputs and stay)
        if (!c->custom_xi) c->tables_ok = false;
        c->q_ok = c->qsq_ok = false;
        StageTimer t(c);
        t.mark();
        build_tables(c);
        t.mark();
        build_q(c);
        t.mark();
        int n = eigensolve(c, ncells, cells, nmodes);
        t.mark();
        project_all(c, ncells, n, true, false);
        c->counts.alloc(ncells);
        c->y.alloc(n);
        OPSEC_CUDA(cudaMemcpyAsync(c->counts.p, counts, sizeof(double) * ncells, cudaMemcpyHostToDevice, c->stream));
        launch_dot(ncells, n, c->modes.p, c->counts.p, c->nbar.p, c->y.p, c->stream, &c->launches);
        t.mark();
        if (evals) OPSEC_CUDA(cudaMemcpyAsync(evals, c->evals.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        fisher_and_epilogue(c, n, c->az_blockF ? nullptr : c->Dp.p, nullptr, mixing, phat, pcov, F, W, M, q, f);
        t.mark();
        t.finish();
    });
}

// ---------------------------------------------------------------- batched mocks
namespace {
// One mock on a worker context whose xi tables are already built: the survey
// grid is replaced, every geometry-dependent stage is recomputed.
void run_mock(opsec_gpu* w, const opsec_mock& m, size_t i, int nb, double* F, double* phat, double* pcov) {
    if (m.nr <= 0 || m.nmu <= 0 || m.nphi <= 0 || (long long)m.nr * m.nmu * m.nphi != m.ncells || !m.cells ||
        !m.counts || !(m.rmin >= 0) || !(m.rmax > m.rmin))
        fail(OPSEC_ERR_ARG, "mock " + std::to_string(i) + ": invalid grid, cells or counts");
    Geometry& g = w->geo;
    g.coordsys = 2;
    g.b[0] = m.rmin;
    g.b[1] = m.rmax;
    g.b[2] = -1.0;
    g.b[3] = 1.0;
    g.b[4] = 0.0;
    g.b[5] = 2 * M_PI;
    g.n[0] = m.nr;
    g.n[1] = m.nmu;
    g.n[2] = m.nphi;
    g.L = 0.0;
    w->q_ok = w->qsq_ok = false;
    build_tables(w);  // no-op: the tables do not depend on the grid
    build_q(w);
    const int n = eigensolve(w, m.ncells, m.cells, m.nmodes);
    project_all(w, m.ncells, n, true, false);
    w->counts.alloc(m.ncells);
    w->y.alloc(n);
    OPSEC_CUDA(cudaMemcpyAsync(w->counts.p, m.counts, sizeof(double) * m.ncells, cudaMemcpyHostToDevice, w->stream));
    launch_dot(m.ncells, n, w->modes.p, w->counts.p, w->nbar.p, w->y.p, w->stream, &w->launches);
    const size_t n2 = (size_t)nb * nb;
    fisher_and_epilogue(w, n, w->az_blockF ? nullptr : w->Dp.p, nullptr, OPSEC_MIXING_INVERSE, phat ? phat + i * nb : nullptr,
                        pcov ? pcov + i * n2 : nullptr, F ? F + i * n2 : nullptr, nullptr, nullptr, nullptr, nullptr);
}
}  // namespace

int opsec_gpu_batch_fisher(opsec_gpu* c, int nmocks, const opsec_mock* mocks, int workers, double* F, double* phat,
                           double* pcov, double* stats) {
    return guard(c, [&] {
        if (nmocks <= 0 || !mocks) fail(OPSEC_ERR_ARG, "no mocks");
        if (workers > 16) fail(OPSEC_ERR_ARG, "at most 16 workers");
        const int nb = c->ntab() - 1;
        const int maxw = workers > 0 ? workers : 8;
        // worker contexts: the template's configuration and P(k), tables built once each
        std::vector<opsec_gpu*> ctx(maxw, nullptr);
        struct Cleanup {
            std::vector<opsec_gpu*>& v;
            ~Cleanup() {
                for (auto* w : v) opsec_gpu_destroy(w);
            }
        } cleanup{ctx};
        for (int k = 0; k < maxw; k++) {
            if (opsec_gpu_create(&ctx[k], c->cfg_text.c_str()) != OPSEC_OK)
                fail(OPSEC_ERR_CONFIG, std::string("worker context: ") + opsec_gpu_last_error(ctx[k]));
            ctx[k]->pk_k = c->pk_k;
            ctx[k]->pk_P = c->pk_P;
            ctx[k]->surr_on = false;
            build_tables(ctx[k]);
        }
        std::atomic<int> next{0};
        std::atomic<int> err_code{OPSEC_OK};
        std::string err_msg;
        std::mutex err_mu;
        auto run_range = [&](int nw, int end) {
            std::vector<std::thread> th;
            for (int k = 0; k < nw; k++)
                th.emplace_back([&, k] {
                    cudaSetDevice(c->device);
                    int i;
                    while (err_code.load() == OPSEC_OK && (i = next.fetch_add(1)) < end) {
                        try {
                            run_mock(ctx[k], mocks[i], (size_t)i, nb, F, phat, pcov);
                        } catch (const Error& e) {
                            std::lock_guard<std::mutex> lk(err_mu);
                            if (err_code.load() == OPSEC_OK) {
                                err_msg = e.msg;
                                err_code = e.code;
                            }
                        }
                    }
                });
            for (auto& t : th) t.join();
            if (next.load() > end) next = end;
        };
        auto now = [] { return std::chrono::steady_clock::now(); };
        const auto t0 = now();
        int best = maxw;
        if (workers <= 0) {
            // autotune the concurrency on the first mocks: 1, 2, 4, 8 workers, 2 per worker each
            const int cand[4] = {1, 2, 4, 8};
            double best_rate = 0;
            for (int ci = 0; ci < 4 && next.load() < nmocks; ci++) {
                const int start = next.load(), end = std::min(nmocks, start + 2 * cand[ci]);
                const auto ta = now();
                run_range(cand[ci], end);
                const double rate = (end - start) / std::chrono::duration<double>(now() - ta).count();
                if (stats) stats[2 + ci] = rate;
                if (rate > best_rate) {
                    best_rate = rate;
                    best = cand[ci];
                }
            }
        }
        run_range(best, nmocks);
        if (err_code.load() != OPSEC_OK) fail(err_code.load(), err_msg);
        if (stats) {
            stats[0] = std::chrono::duration<double>(now() - t0).count();
            stats[1] = best;
        }
    });
}

int opsec_gpu_surrogate_train(opsec_gpu* c, long long max_samples, int epochs, unsigned seed, double* stats) {
    return guard(c, [&] {
        if (max_samples < 64 || epochs < 1) fail(OPSEC_ERR_ARG, "max_samples must be >= 64 and epochs >= 1");
        surrogate_train(c, max_samples, epochs, seed, stats);
    });
}

int opsec_gpu_surrogate_size(void) { return opsec_gpu::kMembers * kSurrParams + 1; }

int opsec_gpu_surrogate_weights(opsec_gpu* c, float* buf, int get) {
    return guard(c, [&] {
        if (!buf) fail(OPSEC_ERR_ARG, "null buffer");
        const size_t n = (size_t)opsec_gpu::kMembers * kSurrParams;
        if (get) {
            if (c->surr_w.size() != n) fail(OPSEC_ERR_STATE, "no surrogate weights");
            std::memcpy(buf, c->surr_w.data(), sizeof(float) * n);
            buf[n] = c->surr_ysc;
        } else {
            if (!(buf[n] > 0) || !std::isfinite(buf[n])) fail(OPSEC_ERR_ARG, "invalid surrogate scale");
            c->surr_w.assign(buf, buf + n);
            c->surr_ysc = buf[n];
            c->q_ok = c->qsq_ok = false;
        }
    });
}

int opsec_gpu_surrogate_stats(const opsec_gpu* c, long long* counts) {
    if (!c || !counts) return OPSEC_ERR_ARG;
    for (int i = 0; i < 3; i++) counts[i] = c->surr_counts[i];
    return OPSEC_OK;
}

int opsec_gpu_surrogate_eval(opsec_gpu* c, const float* params, int n, const float* feats, const float* y,
                             float* out_tc, float* out_simt, double* loss, float* grad) {
    return guard(c, [&] {
        if (!params || !feats || n <= 0 || n > (1 << 20)) fail(OPSEC_ERR_ARG, "invalid surrogate evaluation arguments");
        DevBuf<float> w, wb, f, yy, g, scratch, out, o2;
        DevBuf<double> l;
        std::vector<float> hwb(params, params + kSurrParams);
        for (float& v : hwb) v = bf16_round_host(v);
        std::vector<float> hf(feats, feats + (size_t)n * kSurrIn);
        for (float& v : hf) v = bf16_round_host(v);
        w.alloc(kSurrParams);
        wb.alloc(kSurrParams);
        f.alloc((size_t)n * kSurrIn);
        g.alloc(kSurrParams);
        scratch.alloc((size_t)7 * n * kSurrHid);
        out.alloc(n);
        o2.alloc(n);
        l.alloc(1);
        OPSEC_CUDA(cudaMemcpyAsync(w.p, params, sizeof(float) * kSurrParams, cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(wb.p, hwb.data(), sizeof(float) * kSurrParams, cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(f.p, hf.data(), sizeof(float) * hf.size(), cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemsetAsync(g.p, 0, sizeof(float) * kSurrParams, c->stream));
        OPSEC_CUDA(cudaMemsetAsync(l.p, 0, sizeof(double), c->stream));
        if (y) {
            yy.alloc(n);
            OPSEC_CUDA(cudaMemcpyAsync(yy.p, y, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
        }
        surr_forward_backward(n, f.p, y ? yy.p : nullptr, wb.p, g.p, l.p, out.p, scratch.p, c->stream, &c->launches);
        launch_surr_infer(n, nullptr, 1, nullptr, nullptr, f.p, w.p, o2.p, c->stream, &c->launches);
        if (out_simt) OPSEC_CUDA(cudaMemcpyAsync(out_simt, out.p, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
        if (out_tc) OPSEC_CUDA(cudaMemcpyAsync(out_tc, o2.p, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
        if (y && grad)
            OPSEC_CUDA(cudaMemcpyAsync(grad, g.p, sizeof(float) * kSurrParams, cudaMemcpyDeviceToHost, c->stream));
        if (y && loss) OPSEC_CUDA(cudaMemcpyAsync(loss, l.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        sync(c);
    });
}

int opsec_gpu_stage_times(const opsec_gpu* c, double* times) {
    if (!c || !times) return OPSEC_ERR_ARG;
    for (int i = 0; i < 5; i++) times[i] = c->stage_ms[i];
    return OPSEC_OK;
}

long long opsec_gpu_launch_count(const opsec_gpu* c) { return c ? c->launches : 0; }

int opsec_gpu_eig_stats(const opsec_gpu* c, double* stats) {
    if (!c || !stats) return OPSEC_ERR_ARG;
    std::copy(c->eig_stats, c->eig_stats + 10, stats);
    return OPSEC_OK;
}

int opsec_gpu_fail_alloc(opsec_gpu* c, long long after) {
    if (!c || after < -1) return OPSEC_ERR_ARG;
    c->fail_alloc = after;
    return OPSEC_OK;
}

int opsec_gpu_wait_probe(opsec_gpu* c, long long limit_cycles, int arrive, long long delay_cycles, int* timed_out) {
    return guard(c, [&] {
        if (!timed_out) fail(OPSEC_ERR_ARG, "null output");
        if (limit_cycles < 1 || limit_cycles > 4000000000LL || delay_cycles < 0 || delay_cycles > 4000000000LL)
            fail(OPSEC_ERR_ARG, "wait probe: cycles must be in [1, 4e9]");
        c->probe.alloc(1);
        OPSEC_CUDA(cudaMemsetAsync(c->probe.p, 0, sizeof(int), c->stream));
        launch_wait_probe(limit_cycles, arrive ? 1 : 0, delay_cycles, c->probe.p, c->stream, &c->launches);
        int h = 0;
        OPSEC_CUDA(cudaMemcpyAsync(&h, c->probe.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        sync(c);
        *timed_out = h;
    });
}

int opsec_gpu_kernel_stats(const opsec_gpu* c, const char* name, long long* count, double* total_ms, double* flops,
                           double* bytes) {
    if (!c || !name) return OPSEC_ERR_ARG;
    auto it = c->stats.find(name);
    if (count) *count = it == c->stats.end() ? 0 : it->second.count;
    if (total_ms) *total_ms = it == c->stats.end() ? 0 : it->second.ms;
    if (flops) *flops = it == c->stats.end() ? 0 : it->second.flops;
    if (bytes) *bytes = it == c->stats.end() ? 0 : it->second.bytes;
    return OPSEC_OK;
}

const char* opsec_gpu_last_error(const opsec_gpu* c) { return c ? c->err.c_str() : "null context"; }

void opsec_gpu_destroy(opsec_gpu* c) {
    if (!c) return;
    if (c->device >= 0) cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->eig_exec) cudaGraphExecDestroy(c->eig_exec);
    destroy_mock_plans(c->mock_plans);
    if (c->solver) cusolverDnDestroy(c->solver);
    if (c->blas) cublasDestroy(c->blas);
    for (int j = 0; j < opsec_gpu::kSide; j++) {
        if (c->side[j]) cudaStreamSynchronize(c->side[j]);
        if (c->side_solver[j]) cusolverDnDestroy(c->side_solver[j]);
        if (c->side[j]) cudaStreamDestroy(c->side[j]);
    }
    for (int j = 0; j <= opsec_gpu::kSide; j++)
        if (c->side_ev[j]) cudaEventDestroy(c->side_ev[j]);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

}  // extern "C"
