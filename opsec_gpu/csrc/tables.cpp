// tables.cpp -- xi and band-derivative tables (Model.cpp:84-123) and the symmetry-key space.
#include "context.h"

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
    c->scratch.alloc(3 * ((size_t)32769 + (size_t)nb * 8193));  // weights, weights / k, (weights / k) as float pairs
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

SurrGrid surr_grid(const opsec_gpu* c) {
    const Geometry& g = c->geo;
    SurrGrid sg;
    for (int k = 0; k < 6; k++) sg.b[k] = g.b[k];
    for (int k = 0; k < 3; k++) sg.d[k] = (g.b[2 * k + 1] - g.b[2 * k]) / g.n[k];
    return sg;
}

// per table: (k_lo 5, k_hi 5, band centre k, 0); the full xi table is (0, 0, 0.02, 0)
