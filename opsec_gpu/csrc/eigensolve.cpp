// eigensolve.cpp -- the KL eigensolve (klt.cpp:173-248): azimuthal blocks by the hand-written
// block eigensolver or cuSOLVER, dense cuSOLVER syevdx, or the iterative solver.
#include "context.h"

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

int az_parity_split(opsec_gpu* c, const opsec_cell* cells, std::vector<double>& nba) {
    const KeySpace& ks = c->ks;
    const int H = ks.H, Nphi = ks.N3, Nmu = ks.N2;
    nba.assign(H, 0.0);
    for (int h = 0; h < H; h++) nba[h] = cells[(size_t)h * Nphi].Nbar;
    bool par = c->az_parity && c->geo.mu_symmetric() && Nmu % 2 == 0;
    for (int h = 0; par && h < H; h++) {
        const int ph = (h / Nmu) * Nmu + (Nmu - 1 - h % Nmu);
        if (std::fabs(nba[h] - nba[ph]) > 1e-12 * nba[h]) par = false;
    }
    return par ? 2 : 1;
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
    band_wait(c);
    c->band_batch = 0;
    c->q_ok = c->qsq_ok = false;
    if (!c->xi64.p || !c->xi32.p) c->tables_ok = false;
    c->az_valid = false;
    drop_eig_graph(c);
}

int eigensolve(opsec_gpu* c, int ncells, const opsec_cell* cells, int M, bool want_modes) {
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
        std::vector<double> nba;
        // mu parity split: reflection-symmetric mu grid, even N_mu, Nbar symmetric under j -> N_mu-1-j
        const int npar = az_parity_split(c, cells, nba), Hb = H / npar, nblk = nm * npar;
        c->nbar_arc = nba;
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
        c->modes_ok = false;
        if (want_modes) {
            launch_assemble_modes(H, Nphi, Nmu, npar, M, c->sel.p, c->sel.p + M, c->sel.p + 2 * M, c->S.p,
                                  c->modes.p, c->stream, &c->launches);
            c->modes_ok = true;
        }
        sync(c);
        c->az_m.assign(sel.begin(), sel.begin() + M);
        c->az_idx.assign(sel.begin() + M, sel.begin() + 2 * M);
        c->az_kind.assign(sel.begin() + 2 * M, sel.end());
        c->az_valid = true;
        return M;
    }
    drop_eig_graph(c);
    c->modes_ok = true;  // the dense and iterative solvers write the modes directly
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
        ca.wait_cycles = c->proj_wait;
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

void ensure_modes(opsec_gpu* c) {
    if (c->modes_ok) return;
    if (!c->az_valid) fail(OPSEC_ERR_STATE, "no modes: run the eigensolve first");
    const KeySpace& ks = c->ks;
    const int M = (int)c->az_m.size();
    launch_assemble_modes(ks.H, ks.N3, ks.N2, c->az_npar, M, c->sel.p, c->sel.p + M, c->sel.p + 2 * M, c->S.p,
                          c->modes.p, c->stream, &c->launches);
    c->modes_ok = true;
}

void pixel_projection(opsec_gpu* c, int ncells, int n) {
    c->y.alloc(n);
    if (!c->modes_ok && c->az_valid) {
        const KeySpace& ks = c->ks;
        c->arc_x.alloc((size_t)2 * ks.H * (ks.N3 / 2 + 1));
        launch_dot_azimuthal(ks.H, ks.N3, ks.N2, c->az_npar, n, c->sel.p, c->sel.p + n, c->sel.p + 2 * n, c->S.p,
                             c->counts.p, c->nbar.p, c->arc_x.p, c->y.p, c->stream, &c->launches);
        return;
    }
    ensure_modes(c);
    launch_dot(ncells, n, c->modes.p, c->counts.p, c->nbar.p, c->y.p, c->stream, &c->launches);
}

