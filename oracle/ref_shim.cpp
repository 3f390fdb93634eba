// ref_shim.cpp -- C entry points into the reference's own signal-matrix code.
//
// TEST INFRASTRUCTURE ONLY.  The Makefile in this directory compiles this
// file together with the reference's unmodified sources (read in place from
// the reference checkout, never copied) into oracle/_ref/libopsecref.so.  It
// is used to pin the oracle restatement and to generate golden vectors; the
// GPU library never links it.
//
// chealpix.c (HEALPix pixelisation) is compiled from the reference too,
// against a stub fitsio.h whose map readers fail (cfitsio is absent); and
// basis.cpp, whose FinalizeCell integrates a selection function over a cell.

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "BoxSurvey.h"
#include "Cell.h"
#include "Model.h"
#include "QSpline.h"
#include "RealModel.h"
#include "SeparationFunc.h"
#include "SphericalSurvey.h"
#include "SplitFile.h"
#include "Spline.h"
#include "TestModel.h"
#include "XiFunc.h"
#include "abn.h"
#include "cfg.h"
#include "sig.h"

#include "SelectionFunc.h"
#include "chealpix.h"

bool FinalizeCell(int coordsys, Cell& c, SelectionFunc& nbar, double epsrel, double epsabs);  // basis.cpp:89

namespace {

// Same behaviour as the reference's RealSpaceXi (RealModel.cpp:19-30):
// xi(p1,p2) = F(sep.r(p1,p2)) for a QSpline F.
struct TableXi : public XiFuncImpl {
    QSpline F;
    explicit TableXi(const QSpline& f) : F(f) {}
    double xi(const Point& p1, const Point& p2, const SeparationFunc& sep) { return F(sep.r(p1, p2)); }
};

Survey* make_survey(int coordsys, const double* grid, const int* n, double L) {
    if (coordsys == CoordSysCartesian) {
        Survey* s = new BoxSurvey("none", 1.0, L);
        s->XMin = grid[0]; s->XMax = grid[1];
        s->YMin = grid[2]; s->YMax = grid[3];
        s->ZMin = grid[4]; s->ZMax = grid[5];
        s->Nx = n[0]; s->Ny = n[1]; s->Nz = n[2];
        return s;
    }
    Config cfg = cfg_new();
    cfg_set_double(cfg, "RMin", grid[0]);
    cfg_set_double(cfg, "RMax", grid[1]);
    cfg_set_double(cfg, "MuMin", grid[2]);
    cfg_set_double(cfg, "MuMuin", grid[2]);
    cfg_set_double(cfg, "MuMax", grid[3]);
    cfg_set_double(cfg, "PhiMin", grid[4]);
    cfg_set_double(cfg, "PhiMax", grid[5]);
    cfg_set_int(cfg, "Nr", n[0]);
    cfg_set_int(cfg, "Nmu", n[1]);
    cfg_set_int(cfg, "Nphi", n[2]);
    cfg_set(cfg, "galfile", "none");
    cfg_set(cfg, "maskfile", "none");
    cfg_set(cfg, "radial", "none");
    Survey* s = new SphericalSurvey(cfg);
    cfg_destroy(cfg);
    // Survey.cpp:32 requires the key MuMin but :39 reads the key MuMuin; both are set above
    s->MuMin = grid[2];
    return s;
}

// The spherical selection of SphericalSurvey.cpp:51-80 -- radial linear spline
// times a HEALPix completeness map -- built from arrays instead of its files
// (the map reader needs cfitsio); evaluate() as SphericalSurvey.cpp:70-80.
struct ArraySphericalSelection : public SelectionFuncImpl {
    long nside;
    int nest;
    std::vector<float> mask;
    Spline radial;
    double evaluate(double r, double mu, double phi) {
        double rad = radial(r);
        if (nside <= 0) return rad;
        double theta = acos(mu);
        long ip;
        if (nest)
            ang2pix_nest(nside, theta, phi, &ip);
        else
            ang2pix_ring(nside, theta, phi, &ip);
        return mask[ip] * rad;
    }
};

struct ConstantSelection : public SelectionFuncImpl {  // BoxSurvey.cpp:61-75
    double v;
    double evaluate(double, double, double) { return v; }
};

void to_cell(const double* c, Cell& cell) {
    memset(&cell, 0, sizeof(Cell));
    cell.min1 = c[0]; cell.max1 = c[1];
    cell.min2 = c[2]; cell.max2 = c[3];
    cell.min3 = c[4]; cell.max3 = c[5];
}

}  // namespace

extern "C" {

// xi(r) = RealModel::GetXi for a tabulated P(k) (RealModel.cpp:98-108), or
// the band derivative GetXiDeriv (RealModel.cpp:110-127) when band_kmax > band_kmin.
void ref_xi_table(int npk, const double* pk_k, const double* pk_P, double band_kmin, double band_kmax,
                  int n1, int n2, double r1, double r2, double* r_out, double* xi_out) {
    std::vector<double> r = QSpline::MakeArray(n1, n2, r1, r2);
    if (band_kmax > band_kmin) {
        Spline one = ConstantSpline(1, band_kmin, band_kmax);
        ComputeXiLM(0, 2, one, n1 + n2, &r[0], xi_out, 8192, band_kmin, band_kmax);
    } else {
        Spline pk = CubicSpline(npk, pk_k, pk_P);
        ComputeXiLM(0, 2, pk, n1 + n2, &r[0], xi_out);
    }
    for (int i = 0; i < n1 + n2; i++) r_out[i] = r[i];
}

double ref_cspline_eval(int npk, const double* pk_k, const double* pk_P, double k) {
    Spline pk = CubicSpline(npk, pk_k, pk_P);
    return pk(k);
}

void ref_qspline_eval(int n1, int n2, const double* x, const double* y, int m, const double* r, double* out) {
    QSpline q(n1, n2, x, y);
    for (int i = 0; i < m; i++) out[i] = q(r[i]);
}

double ref_sep(int coordsys, double L, const double* p1, const double* p2) {
    double grid[6] = {0, 1, -1, 1, 0, 2 * M_PI};
    int n[3] = {1, 1, 1};
    Survey* s = make_survey(coordsys, grid, n, L);
    SeparationFunc sep = s->GetSeparationFunction();
    Point a = {p1[0], p1[1], p1[2]};
    Point b = {p2[0], p2[1], p2[2]};
    double r = sep.r(a, b);
    delete s;
    return r;
}

// One adaptive-cubature cell-pair integral (sig.cpp:419-482) with a
// tabulated xi (kind 0) or a TestModel correlation function (kind 1
// exponential, 2 gaussian: TestModel.cpp:13-25).
double ref_signal_pair(int coordsys, double L, const double* c1, const double* c2, int kind, double A, double b,
                       int n1, int n2, const double* x, const double* y, double epsrel, double epsabs,
                       double* err) {
    double grid[6] = {0, 1, -1, 1, 0, 2 * M_PI};
    int n[3] = {1, 1, 1};
    Survey* s = make_survey(coordsys, grid, n, L);
    SeparationFunc sep = s->GetSeparationFunction();
    XiFunc xi;
    if (kind == 0)
        xi = XiFunc(new TableXi(QSpline(n1, n2, x, y)));
    else {
        TestModel m(kind == 1 ? 0 : 1, A, b);
        xi = m.GetXi();
    }
    Cell a, bb;
    to_cell(c1, a);
    to_cell(c2, bb);
    double v = (coordsys == CoordSysCartesian) ? ComputeSignalC(a, bb, xi, sep, epsrel, epsabs, err)
                                               : ComputeSignalS(a, bb, xi, sep, epsrel, epsabs, err);
    delete s;
    return v;
}

// ComputeSignalMatrixBlock (sig.cpp:50-213) over the full grid of cells,
// cells[i] = {a, d1, d2, d3, bounds..., Veff, Nbar} in the reference layout.
void ref_signal_block(int coordsys, const double* grid, const int* n, double L, int ncells, const void* cells,
                      int nrows, const int* rows, int ncols, const int* cols, double* s, int lld, int n1, int n2,
                      const double* x, const double* y, double epsrel, double epsabs) {
    Survey* sv = make_survey(coordsys, grid, n, L);
    XiFunc xi(new TableXi(QSpline(n1, n2, x, y)));
    std::vector<int> r(rows, rows + nrows), c(cols, cols + ncols);
    ComputeSignalMatrixBlock(ncells, r, c, s, lld, xi, sv, (const Cell*)cells, epsrel, epsabs);
    delete sv;
}

int ref_sizeof_cell() { return (int)sizeof(Cell); }

// A cellfile written by the reference's own ABN writer with the header basis
// puts in it (basis.cpp:195-201): survey options, then Ncells.
int ref_write_cells(const char* path, int coordsys, const double* grid, const int* n, double L, int ncells,
                    const void* cells) {
    Survey* sv = make_survey(coordsys, grid, n, L);
    Config opts = sv->GetConfigurationOptions();
    cfg_set_int(opts, "Ncells", ncells);
    FILE* f = fopen(path, "w");
    if (!f) return 1;
    abn_write(f, cells, ncells, CELL_FMT_STRING, opts);
    fclose(f);
    cfg_destroy(opts);
    delete sv;
    return 0;
}

}  // extern "C"

extern "C" {

// HEALPix pixel of each (theta, phi) by the reference's ang2pix_ring / ang2pix_nest (chealpix.c:100-246).
void ref_ang2pix(long nside, int nest, int n, const double* theta, const double* phi, long* pix) {
    for (int i = 0; i < n; i++) {
        if (nest)
            ang2pix_nest(nside, theta[i], phi[i], &pix[i]);
        else
            ang2pix_ring(nside, theta[i], phi[i], &pix[i]);
    }
}

// The reference cell builder (basis.cpp:160-190): every grid cell by Survey::CreateEmptyCell,
// Veff and Nbar by FinalizeCell (adaptive cubature, epsrel 1e-5) of the constant selection
// (coordsys 1) or the radial-spline x HEALPix-map selection (coordsys 2; nside 0 = no map).
// out[c] = (Veff, Nbar, kept) per cell in grid order.
void ref_basis(int coordsys, const double* grid, const int* n, double nbar_const, int nrad, const double* rad_r,
               const double* rad_n, long nside, int nest, const float* mask, double* out) {
    Survey* s = make_survey(coordsys, grid, n, 0.0);
    // the bounds exactly (the configuration text above keeps 6 significant digits)
    s->Min1 = grid[0]; s->Max1 = grid[1];
    s->Min2 = grid[2]; s->Max2 = grid[3];
    s->Min3 = grid[4]; s->Max3 = grid[5];
    SelectionFunc sel;
    if (coordsys == CoordSysCartesian) {
        ConstantSelection* c = new ConstantSelection;
        c->v = nbar_const;
        sel = SelectionFunc(c);
    } else {
        ArraySphericalSelection* a = new ArraySphericalSelection;
        a->nside = nside;
        a->nest = nest;
        if (nside > 0) a->mask.assign(mask, mask + 12 * nside * nside);
        a->radial = LinearSpline(nrad, rad_r, rad_n);
        sel = SelectionFunc(a);
    }
    long k = 0;
    for (int d1 = 0; d1 < n[0]; d1++)
        for (int d2 = 0; d2 < n[1]; d2++)
            for (int d3 = 0; d3 < n[2]; d3++, k++) {
                Cell c = s->CreateEmptyCell(d1, d2, d3);
                bool kept = FinalizeCell(coordsys, c, sel, 1e-5, 1e-10);
                out[3 * k] = kept ? c.Veff : 0.0;
                out[3 * k + 1] = kept ? c.Nbar : 0.0;
                out[3 * k + 2] = kept ? 1.0 : 0.0;
            }
    delete s;
}

// The reference's galaxy binning (dot.cpp:124-129): grid index of each galaxy by
// Survey::GetGridIndex (Survey.cpp:93-101), and the weighted counts per cell as dot
// accumulates them -- a galaxy goes to cellmap[e] when e > 0, else to counts[ncells].
// gals: ngal records (x1, x2, x3, w) float32; cellidx: grid index of each cell.
void ref_count_galaxies(int coordsys, const double* grid, const int* n, long ngal, const float* gals, int ncells,
                        const int* cellidx, int* index, double* counts) {
    Survey* s = make_survey(coordsys, grid, n, 0.0);
    s->Min1 = grid[0]; s->Max1 = grid[1];
    s->Min2 = grid[2]; s->Max2 = grid[3];
    s->Min3 = grid[4]; s->Max3 = grid[5];
    std::vector<int> cellmap((size_t)n[0] * n[1] * n[2], -1);
    for (int a = 0; a < ncells; a++) cellmap[cellidx[a]] = a;
    for (int a = 0; a <= ncells; a++) counts[a] = 0.0;
    for (long i = 0; i < ngal; i++) {
        const float* g = gals + 4 * i;
        const int e = s->GetGridIndex(g[0], g[1], g[2]);
        index[i] = e;
        const int a = (e > 0) ? cellmap[e] : ncells;
        if (a >= 0) counts[a] += g[3];  // a = -1 (an empty grid cell) indexes before the array there
    }
    delete s;
}

// The data of the first ABN block of a file read through the reference's SplitFile, as
// estimate reads its evalfile and covfile (estimate-mpi.cpp:152-200, SplitFile.cpp:120-175):
// the header from the first piece, the data across the pieces that follow it.  Returns the
// bytes read into out (at most cap), -1 without a header.
long ref_split_read(const char* path, char* out, long cap) {
    SplitFile f(path, "r");
    if (!f.isopen()) return -1;
    size_t n = 0, size = 0;
    char endian = 0, fmt[ABN_MAX_FORMAT_LENGTH];
    if (abn_read_header(f, &n, &size, &endian, fmt, NULL) != 0) return -1;
    size_t want = n * size;
    if ((long)want > cap) want = (size_t)cap;
    return (long)f.read(out, want);
}

// The header basis writes on its cell file (basis.cpp:195-199): the survey's
// GetConfigurationOptions (Survey.cpp:103-129, BoxSurvey.cpp:135-141,
// SphericalSurvey.cpp:172-178) plus Ncells, from the survey's sub-configuration in
// cfgpath (keys without the "survey." prefix, as InitializeSurvey hands them over).
int ref_survey_header(int coordsys, const char* cfgpath, int ncells, const char* outpath) {
    Config cfg = cfg_new();
    if (cfg_read_file(cfg, cfgpath) != 0) return 1;
    Survey* s = coordsys == CoordSysCartesian ? (Survey*)new BoxSurvey(cfg) : (Survey*)new SphericalSurvey(cfg);
    Config opts = s->GetConfigurationOptions();
    cfg_set_int(opts, "Ncells", ncells);
    FILE* f = fopen(outpath, "wb");
    abn_write_header(f, ncells, CELL_FMT_STRING, opts);
    fclose(f);
    cfg_destroy(opts);
    cfg_destroy(cfg);
    delete s;
    return 0;
}

// Model::GetParam of RealModel for every band (RealModel.cpp:33-96): P(k) from pkfile,
// Nbands regular bands on [kmin, kmax] (the values pass through cfg_set_double's "%g").
int ref_band_params(const char* pkfile, int nbands, double kmin, double kmax, double* out) {
    Config cfg = cfg_new();
    cfg_set(cfg, "pkfile", pkfile);
    cfg_set_int(cfg, "Nbands", nbands);
    cfg_set_double(cfg, "kmin", kmin);
    cfg_set_double(cfg, "kmax", kmax);
    RealModel m(cfg);
    cfg_destroy(cfg);
    if (m.NumParams() != nbands) return 1;
    for (int n = 0; n < nbands; n++) out[n] = m.GetParam(n);
    return 0;
}

}  // extern "C"
