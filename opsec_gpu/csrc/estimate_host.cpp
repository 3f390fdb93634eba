// estimate_host.cpp -- band priors (RealModel::GetParam), Fisher sums and the estimate epilogue
// (estimate-mpi.cpp:480-641).
#include "context.h"

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
