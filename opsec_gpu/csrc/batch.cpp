// batch.cpp -- many independent mock surveys on worker contexts (opsec_gpu_batch_fisher).
#include "context.h"

#include <cmath>

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
    const int n = eigensolve(w, m.ncells, m.cells, m.nmodes, false);
    project_all(w, m.ncells, n, true, false);
    w->counts.alloc(m.ncells);
    OPSEC_CUDA(cudaMemcpyAsync(w->counts.p, m.counts, sizeof(double) * m.ncells, cudaMemcpyHostToDevice, w->stream));
    pixel_projection(w, m.ncells, n);
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
        const int maxw = workers > 0 ? workers : 16;
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
        // largest mocks first: a worker's buffers then reach their final size on its first mocks,
        // and later mocks reuse them (a reallocation frees device memory, which waits for the
        // whole device, every worker's work included)
        std::vector<int> order(nmocks);
        for (int i = 0; i < nmocks; i++) order[i] = i;
        std::stable_sort(order.begin(), order.end(),
                         [&](int x, int y) { return mocks[x].ncells > mocks[y].ncells; });
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
                            run_mock(ctx[k], mocks[order[i]], (size_t)order[i], nb, F, phat, pcov);
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
            // autotune the concurrency on the first mocks: 1, 2, 4, 8, 12, 16 workers, 2 mocks per
            // worker each.  The mocks run largest first, so each candidate sees smaller mocks than
            // the one before: its rate counts mocks of the batch's mean cost per second, a mock's
            // cost taken as ncells^1.5 (the cubature's key count grows as ncells^2 / nphi)
            const int cand[6] = {1, 2, 4, 8, 12, 16};
            auto cost = [&](int i) { return std::pow((double)mocks[order[i]].ncells, 1.5); };
            double mean = 0;
            for (int i = 0; i < nmocks; i++) mean += cost(i) / nmocks;
            double best_rate = 0;
            for (int ci = 0; ci < 6 && next.load() < nmocks; ci++) {
                const int start = next.load(), end = std::min(nmocks, start + 2 * cand[ci]);
                const auto ta = now();
                run_range(cand[ci], end);
                double work = 0;
                for (int i = start; i < end; i++) work += cost(i) / mean;
                const double rate = work / std::chrono::duration<double>(now() - ta).count();
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
