// stages.cpp -- Q by cell-pair cubature for every key and table, the square table, the cells.
#include "context.h"

void build_q(opsec_gpu* c) {
    if (c->q_ok) return;
    band_wait(c);  // band-block transforms still reading the old Q tables
    c->band_batch = 0;
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
    a.win_logkeys = c->win_logkeys;
    a.win_keyorder = c->win_keyorder;
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
