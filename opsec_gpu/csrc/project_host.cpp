// project_host.cpp -- C_p = B^T S_p B (comma-scalapack.cpp:228-265): azimuthal blocks or the fused
// tensor-core projection.
#include <type_traits>

#include "context.h"

struct AzPlan {
    int H, nm, npar, nb, ncol;  // H: block size (arcs / npar)
    long long csize;
    int Kmax;
    double flops;
    const int *col_m, *col_idx, *mode_m, *mode_cls, *mode_col, *Km_dev, *base_dev;
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

// Bands per batch of band blocks: as many as fit in ~2 GB
int band_batch_of(int nb, size_t nS, size_t elem) {
    return (int)std::max<size_t>(1, std::min<size_t>(nb, (size_t(2) << 30) / (elem * nS)));
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
    const int bpp = band_batch_of(a.nb, nS, sizeof(T));
    // FP32 band blocks live in their own buffer, whose first batch may already be under way on
    // the band stream (prefetch_band_blocks, for this build and these blocks)
    constexpr bool f32 = std::is_same<T, float>::value;
    const bool pre = f32 && c->band_batch > 0 && c->band_batch == std::min(bpp, a.nb) && c->band_nblk == nblk &&
                     c->band_H == H;
    c->band_batch = 0;
    if (f32 && !pre) {
        band_wait(c);
        c->azSb.alloc(sizeof(float) * nS * bpp);
    }
    // tensor-core products (FP32 path): T of every band of a batch, [band][ncol][H], then the
    // tiles and the error word
    const bool tcg = sizeof(T) == sizeof(float) && c->az_tc && az_tc_supported(H);
    const size_t nTb = tcg ? (size_t)a.ncol * H * bpp : nT * bpp;
    const size_t tc_bytes = tcg ? az_tc_work_bytes(nblk, bpp, *a.Km, H) : 0;
    const size_t nSw = f32 ? 0 : nS * bpp;
    ws.alloc(sizeof(T) * (nU + nSw + nTb + nC) + tc_bytes + 512);
    T* U = reinterpret_cast<T*>(ws.p);
    T* Sb = f32 ? reinterpret_cast<T*>(c->azSb.p) : U + nU;
    T* Tm = U + nU + nSw;
    T* Cm = Tm + nTb;
    unsigned char* tcw = reinterpret_cast<unsigned char*>(Cm + nC);
    tcw = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tcw) + 255) & ~uintptr_t(255));
    int* tc_err = reinterpret_cast<int*>(tcw);
    if (tcg) OPSEC_CUDA(cudaMemsetAsync(tc_err, 0, sizeof(int), c->stream));
    // the block eigenvectors the modes use
    launch_gather_block_vectors(H, a.ncol, a.col_m, a.col_idx, c->S.p, U, c->stream, &c->launches);
    for (int p0 = 0; p0 < a.nb; p0 += bpp) {
        const int np = std::min(bpp, a.nb - p0);
        if (pre && p0 == 0) {
            // the first batch was transformed on the band stream
            OPSEC_CUDA(cudaStreamWaitEvent(c->stream, c->band_ev[1], 0));
            c->band_pending = false;
        }
        for (int p = (pre && p0 == 0) ? p0 + np : p0; p < p0 + np; p++) {
            if (g_clock) g_clock->begin("azimuthal_transform", c->stream, 2.0 * nblk * (double)H * H * c->ks.nf);
            if constexpr (std::is_same<T, float>::value)
                launch_azimuthal_blocks(c->ks, c->Q.p + (size_t)(1 + p) * c->ks.nkeys, a.nbar_arc, a.nm, a.npar,
                                        Sb + (size_t)(p - p0) * nS, c->stream, &c->launches, c->az_tiled != 0);
            else
                launch_azimuthal_blocks(c->ks, c->Q.p + (size_t)(1 + p) * c->ks.nkeys, a.nbar_arc, a.nm, a.npar,
                                        Sb + (size_t)(p - p0) * nS, c->stream, &c->launches);
            if (g_clock) g_clock->end(c->stream);
        }
        if (g_clock) g_clock->begin("azimuthal_gemm", c->stream, a.flops * np);
        if (tcg) {
            launch_az_tc(H, nblk, a.ncol, np, reinterpret_cast<const float*>(Sb), reinterpret_cast<const float*>(U),
                         reinterpret_cast<float*>(Tm), reinterpret_cast<float*>(Cm + (size_t)p0 * a.csize), a.csize,
                         a.Km_dev, a.base_dev, c->az_off.p, *a.Km, tcw + 256, tc_bytes, tc_err,
                         c->proj_wait, c->stream, &c->launches);
            if (g_clock) g_clock->end(c->stream);
            continue;
        }
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
    if (tcg) {
        int e = 0;
        OPSEC_CUDA(cudaMemcpyAsync(&e, tc_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        OPSEC_CUDA(cudaStreamSynchronize(c->stream));
        if (e) fail(OPSEC_ERR_CUDA, "tensor-core block projection: a pipeline wait timed out");
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
    ti.insert(ti.end(), base.begin(), base.end());
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
    const int* d_base = d_Km + nblk;
    if (!c->blas) blas_check(cublasCreate(&c->blas), "cublasCreate");
    blas_check(cublasSetStream(c->blas, c->stream), "cublasSetStream");
    std::vector<double> nba(c->nbar_arc);
    DevBuf<double>& d_nba = c->nba_dev;
    d_nba.alloc(nba.size());
    OPSEC_CUDA(cudaMemcpyAsync(d_nba.p, nba.data(), sizeof(double) * nba.size(), cudaMemcpyHostToDevice, c->stream));
    double fl = 0;
    for (int m = 0; m < nblk; m++) fl += 2.0 * H * H * Km[m] + 2.0 * H * (double)Km[m] * Km[m];
    AzPlan plan{H,      nm,        npar,       nb,         ncol,       csize, Kmax,  fl, d_col_m,
                d_col_idx, d_mode_m, d_mode_cls, d_mode_col, d_Km, d_base, &Km, &base, &off, d_nba.p};
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
void band_wait(opsec_gpu* c) {
    if (c->band_pending && c->band_stream) OPSEC_CUDA(cudaStreamSynchronize(c->band_stream));
    c->band_pending = false;
}

void prefetch_band_blocks(opsec_gpu* c, int ncells, const opsec_cell* cells) {
    c->band_batch = 0;
    if (!c->az_overlap || c->az_gemm64 || !(c->projection == "auto" || c->projection == "azimuthal")) return;
    if (c->ntab() < 2 || !azimuthal_ok(c, ncells, cells)) return;
    const KeySpace& ks = c->ks;
    std::vector<double> nba;
    const int npar = az_parity_split(c, cells, nba);
    const int H = ks.H / npar, nm = ks.N3 / 2 + 1, nblk = nm * npar, nb = c->ntab() - 1;
    const size_t nS = (size_t)nblk * H * H;
    const int np = std::min(band_batch_of(nb, nS, sizeof(float)), nb);
    band_wait(c);
    if (!c->band_stream) {
        int least = 0, greatest = 0;
        OPSEC_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        OPSEC_CUDA(cudaStreamCreateWithPriority(&c->band_stream, cudaStreamNonBlocking, least));
        for (auto& e : c->band_ev) OPSEC_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    c->azSb.alloc(sizeof(float) * nS * band_batch_of(nb, nS, sizeof(float)));
    c->nba_band.alloc(nba.size());
    // the Q tables (and the per-arc Nbar) are complete on the main stream; the blocks depend on
    // nothing else
    OPSEC_CUDA(cudaMemcpyAsync(c->nba_band.p, nba.data(), sizeof(double) * nba.size(), cudaMemcpyHostToDevice,
                               c->stream));
    OPSEC_CUDA(cudaEventRecord(c->band_ev[0], c->stream));
    OPSEC_CUDA(cudaStreamWaitEvent(c->band_stream, c->band_ev[0], 0));
    float* Sb = reinterpret_cast<float*>(c->azSb.p);
    for (int p = 0; p < np; p++) {
        if (g_clock) g_clock->begin("azimuthal_transform", c->band_stream, 2.0 * nblk * (double)H * H * ks.nf);
        launch_azimuthal_blocks(ks, c->Q.p + (size_t)(1 + p) * ks.nkeys, c->nba_band.p, nm, npar, Sb + (size_t)p * nS,
                                c->band_stream, &c->launches, c->az_tiled != 0);
        if (g_clock) g_clock->end(c->band_stream);
    }
    OPSEC_CUDA(cudaEventRecord(c->band_ev[1], c->band_stream));
    c->band_pending = true;
    c->band_batch = np;
    c->band_nblk = nblk;
    c->band_H = H;
}

void project_all(opsec_gpu* c, int ncells, int M, bool own_modes, bool packed) {
    c->az_blockF = false;
    if (own_modes && c->az_valid && (c->projection == "auto" || c->projection == "azimuthal")) {
        project_azimuthal(c, ncells, M, packed);
        return;
    }
    if (c->projection == "azimuthal")
        fail(OPSEC_ERR_CONFIG, "projection=azimuthal needs a full-sky spherical build on its own modes");
    build_qsq(c);
    if (own_modes) ensure_modes(c);
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
    if (c->proj_arcs && c->cells_arc_order && (n3 == 16 || n3 == 32 || n3 == 64) &&
        (long long)(128 / n3) * c->ks.H * c->ks.nf < (1LL << 23))
        a.arc_run = n3;
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
