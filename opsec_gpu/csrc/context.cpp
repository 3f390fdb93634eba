// context.cpp -- the engine's utilities (errors, device buffers, kernel clocks) and the C ABI of
// include/opsec_gpu.h, which drives the host-side stages that context.h lists.
#include "context.h"
#include "gemm_tc.h"

namespace opsec {

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


void blas_check(cublasStatus_t st, const char* what) {
    if (st != CUBLAS_STATUS_SUCCESS) fail(OPSEC_ERR_CUDA, std::string(what) + " failed (cuBLAS status " + std::to_string((int)st) + ")");
}

void solver_check(cusolverStatus_t st, const char* what) {
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

std::map<std::string, std::string> parse_config(const char* text) {
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

double to_double(const std::string& key, const std::string& v) {
    char* end = nullptr;
    errno = 0;
    double d = std::strtod(v.c_str(), &end);
    if (end == v.c_str() || errno == ERANGE || !std::isfinite(d)) fail(OPSEC_ERR_CONFIG, "option " + key + " = '" + v + "' is not a number");
    return d;
}

// cfg_get_int (cfg.c:430-440) reads "%i": a leading integer in decimal, octal (0...) or hex
// (0x...), whatever follows it ignored
int to_int(const std::string& key, const std::string& v) {
    char* end = nullptr;
    long x = std::strtol(v.c_str(), &end, 0);
    if (end == v.c_str()) fail(OPSEC_ERR_CONFIG, "option " + key + " = '" + v + "' is not an integer");
    return (int)x;
}

// ---------------------------------------------------------------- host math
// fmm cubic spline coefficients (Spline.cpp:258-330).
void cspline_coeffs(const std::vector<double>& X, const std::vector<double>& Y, std::vector<double>& b,
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

int lookup_index(double x, int N, const double* X) {
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
void gauss_legendre01(int n, std::vector<double>& u, std::vector<double>& w) {
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
        // the main stream at the highest priority: work overlapped on the band stream (lowest)
        // takes the SMs the main stream's kernels leave free
        int least = 0, greatest = 0;
        OPSEC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        OPSEC_CUDA(cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, greatest));
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
        c->modes_ok = false;  // the caller's modes, not the last eigensolve's
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
        c->modes_ok = false;  // the caller's modes, not the last eigensolve's
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
        prefetch_band_blocks(c, ncells, cells);
        t.mark();
        int n = eigensolve(c, ncells, cells, nmodes, false);
        t.mark();
        project_all(c, ncells, n, true, false);
        c->counts.alloc(ncells);
        OPSEC_CUDA(cudaMemcpyAsync(c->counts.p, counts, sizeof(double) * ncells, cudaMemcpyHostToDevice, c->stream));
        pixel_projection(c, ncells, n);
        t.mark();
        if (evals) OPSEC_CUDA(cudaMemcpyAsync(evals, c->evals.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        fisher_and_epilogue(c, n, c->az_blockF ? nullptr : c->Dp.p, nullptr, mixing, phat, pcov, F, W, M, q, f);
        t.mark();
        t.finish();
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

int opsec_gpu_block_product(opsec_gpu* c, int N, int ncols, const double* S, const float* X, float alpha, float beta,
                            float* C, float gamma, const float* D) {
    return guard(c, [&] {
        if (N < 1 || ncols < 1 || !S || !X || !C || (gamma != 0.f && !D))
            fail(OPSEC_ERR_ARG, "block product: N, ncols >= 1 and S, X, C (and D when gamma != 0) required");
        const size_t NN = (size_t)N * N, NX = (size_t)N * ncols;
        DevBuf<double> dS;
        DevBuf<float> dX, dC, dD;
        dS.alloc(NN);
        dX.alloc(NX);
        dC.alloc(NX);
        OPSEC_CUDA(cudaMemcpyAsync(dS.p, S, sizeof(double) * NN, cudaMemcpyHostToDevice, c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(dX.p, X, sizeof(float) * NX, cudaMemcpyHostToDevice, c->stream));
        if (beta != 0.f) OPSEC_CUDA(cudaMemcpyAsync(dC.p, C, sizeof(float) * NX, cudaMemcpyHostToDevice, c->stream));
        if (gamma != 0.f) {
            dD.alloc(NX);
            OPSEC_CUDA(cudaMemcpyAsync(dD.p, D, sizeof(float) * NX, cudaMemcpyHostToDevice, c->stream));
        }
        TcOperand a, b;
        a.shape(N, N);
        b.shape(ncols, N);
        c->probe.alloc(1);
        OPSEC_CUDA(cudaMemsetAsync(c->probe.p, 0, sizeof(int), c->stream));
        tc_split(dS.p, N, a, c->stream, &c->launches);
        tc_split(dX.p, N, b, c->stream, &c->launches);
        tc_gemm(a, b, alpha, beta, dC.p, N, gamma, dD.p, N, 1, c->chfsi.tile, c->probe.p, c->proj_wait, c->stream,
                &c->launches);
        int h = 0;
        OPSEC_CUDA(cudaMemcpyAsync(C, dC.p, sizeof(float) * NX, cudaMemcpyDeviceToHost, c->stream));
        OPSEC_CUDA(cudaMemcpyAsync(&h, c->probe.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        sync(c);
        if (h) fail(OPSEC_ERR_CUDA, "block product: tensor-core GEMM timed out waiting on a pipeline barrier");
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
    if (c->band_stream) {
        cudaStreamSynchronize(c->band_stream);
        cudaStreamDestroy(c->band_stream);
    }
    for (auto& e : c->band_ev)
        if (e) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

}  // extern "C"

