/* oracle.c -- FP64 CPU restatement of the OPSEC signal-matrix hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  Nothing in opsec_gpu/ links against it or calls it.
 *
 * Every routine restates the reference algorithm in plain C, with the
 * reference location it follows (paths inside jwgcarlson/OPSEC):
 *   - cubic spline (Forsythe-Malcolm-Moler "fmm")   code/opsec/src/Spline.cpp:258-330
 *   - spline lookup + out-of-range zero              code/opsec/src/Spline.cpp:13-35,429-434
 *   - xi_l^m(r) by Simpson with exp(-(k/kdamp)^2)    code/opsec/src/Model.cpp:55-123
 *   - band power prior (256 midpoints)               code/opsec/src/RealModel.cpp:85-96
 *   - QSpline r-grid (linear + log sections)         code/opsec/src/QSpline.cpp:6-70
 *   - periodic box separation                        code/opsec/src/BoxSurvey.cpp:19-37
 *   - spherical separation (law of cosines)          code/opsec/src/SphericalSurvey.cpp:19-23
 *   - cell-pair integrand maps (affine / r^3)        code/opsec/src/sig.cpp:388-458
 *   - symmetry keys of the signal matrix             code/opsec/src/sig.cpp:99-119,150-207
 * The cell-pair integral itself uses the n^3 x n^3 Gauss-Legendre product
 * rule of the plain method (n = 4 by default) instead of the reference's
 * adaptive Genz-Malik cubature; genz_malik.c restates the latter.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ */
/* Spline lookup: initial guess for a uniform grid, then bisection.     */
/* Follows LookupIndex, Spline.cpp:13-35.                               */
/* ------------------------------------------------------------------ */
static int lookup_index(double x, int N, const double* X) {
    double I = (N - 1) * (x - X[0]) / (X[N - 1] - X[0]);
    int i = (int)I;
    int ilo = 0, ihi = N - 2;
    if (i < 0) i = 0;
    if (i > N - 2) i = N - 2;
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

/* fmm cubic spline coefficients, Spline.cpp:258-330.  b, c, d have n entries. */
void orc_cspline_coeffs(int N, const double* X, const double* Y, double* b, double* c, double* d) {
    if (N == 2) {
        b[0] = b[1] = (Y[1] - Y[0]) / (X[1] - X[0]);
        c[0] = c[1] = 0;
        d[0] = d[1] = 0;
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

/* Spline value; zero outside [X[0], X[N-1]) as Spline::Evaluate, Spline.cpp:429-434. */
double orc_cspline_eval(int N, const double* X, const double* Y, const double* b, const double* c,
                        const double* d, double x) {
    if (x < X[0] || x >= X[N - 1]) return 0.0;
    int i = lookup_index(x, N, X);
    double u = x - X[i];
    return Y[i] + b[i] * u + c[i] * u * u + d[i] * u * u * u;
}

/* ------------------------------------------------------------------ */
/* xi_l^m(r) for l = 0 by Simpson's rule, Model.cpp:55-123.             */
/* P(k) is supplied as its value at the Nk+1 Simpson nodes.             */
/* ------------------------------------------------------------------ */
static double sj0(double x) {
    double x2 = x * x;
    return (x2 < 1e-4) ? 1 - x2 * (1 / 6. + x2 * (1 / 120. - x2 * (1 / 5040.))) : sin(x) / x;
}

void orc_simpson_nodes(int Nk, double kmin, double kmax, double* k) {
    const double dk = (kmax - kmin) / Nk;
    for (int j = 0; j <= Nk; j++) k[j] = kmin + j * dk;
}

/* mult[j] as Model.cpp:104-112 given Pk[j] = P(k_j). */
void orc_simpson_weights(int m, int Nk, double kmin, double kmax, double kdamp, const double* Pk,
                         double* mult) {
    const double dk = (kmax - kmin) / Nk;
    for (int j = 0; j <= Nk; j++) {
        double kj = kmin + j * dk;
        mult[j] = 2 + 2 * (j % 2) - (j == 0) - (j == Nk);
        mult[j] *= Pk[j] * pow(kj, m) * exp(-kj * kj / (kdamp * kdamp));
        mult[j] *= (dk / 3) / (2 * M_PI * M_PI);
    }
}

void orc_xi_sum(int Nr, const double* r, double* xi, int Nk, const double* k, const double* mult) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < Nr; i++) {
        double s = 0;
        for (int j = 0; j <= Nk; j++) s += mult[j] * sj0(k[j] * r[i]);
        xi[i] = s;
    }
}

/* Band average of P(k) over 256 midpoints, RealModel.cpp:85-96. */
double orc_band_prior(int N, const double* X, const double* Y, const double* b, const double* c,
                      const double* d, double kmin, double kmax) {
    const int Nk = 256;
    double sum = 0;
    for (int i = 0; i < Nk; i++) {
        double k = kmin + (i + 0.5) * (kmax - kmin) / Nk;
        sum += orc_cspline_eval(N, X, Y, b, c, d, k);
    }
    return sum / Nk;
}

/* ------------------------------------------------------------------ */
/* QSpline r-grid and lookup, QSpline.cpp:6-70.                         */
/* ------------------------------------------------------------------ */
void orc_qspline_array(int n1, int n2, double x1, double x2, double* X) {
    for (int i = 0; i < n1; i++) X[i] = i * x1 / n1;
    for (int j = 0; j < n2; j++) X[n1 + j] = x1 * exp(j * log(x2 / x1) / (n2 - 1));
}

typedef struct {
    int n1, n2;
    const double* X; /* n1+n2 grid points */
    const double* U; /* log(X[n1+j]), j < n2 */
    const double* Y; /* table values, n1+n2 */
} qspline;

static double linear_eval(int N, const double* X, const double* Y, double x) {
    if (x < X[0] || x >= X[N - 1]) return 0.0;
    int i = lookup_index(x, N, X);
    double x1 = X[i], x2 = X[i + 1], y1 = Y[i], y2 = Y[i + 1];
    return y1 + (y2 - y1) * (x - x1) / (x2 - x1);
}

static double qspline_eval(const qspline* q, double x) {
    int n = q->n1 + q->n2;
    double x1 = q->X[q->n1], x2 = q->X[n - 1];
    if (x < 0) return 0;
    if (x < x1) return linear_eval(q->n1 + 1, q->X, q->Y, x);
    if (x < x2) return linear_eval(q->n2, q->U, q->Y + q->n1, log(x));
    return q->Y[n - 1];
}

double orc_qspline_eval(int n1, int n2, const double* X, const double* U, const double* Y, double x) {
    qspline q = {n1, n2, X, U, Y};
    return qspline_eval(&q, x);
}

/* ------------------------------------------------------------------ */
/* Gauss-Legendre nodes and weights mapped to [0,1] (Newton iteration   */
/* on the three-term Legendre recurrence; Abramowitz & Stegun 25.4.29). */
/* ------------------------------------------------------------------ */
void orc_gauss_legendre01(int n, double* u, double* w) {
    if (n == 1) {
        u[0] = 0.5;
        w[0] = 1.0;
        return;
    }
    for (int i = 0; i < (n + 1) / 2; i++) {
        double x = cos(M_PI * (i + 0.75) / (n + 0.5));
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
            if (fabs(dx) <= 1e-15 * fabs(x)) break;
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
        u[i] = 0.5 * (1 - x); /* ascending nodes on [0,1] */
        u[n - 1 - i] = 0.5 * (1 + x);
        w[i] = w[n - 1 - i] = 0.5 * wt;
    }
}

/* ------------------------------------------------------------------ */
/* Separation functions.                                                */
/* ------------------------------------------------------------------ */
static inline double linsep(double x1, double x2, double L) {
    double dx = x2 - x1;
    dx += L * ((dx < -L / 2) - (dx >= L / 2)); /* BoxSurvey.cpp:26-30 */
    return dx;
}

static inline double sep_box(const double* p1, const double* p2, double L) {
    double rx, ry, rz;
    if (L > 0) {
        rx = linsep(p1[0], p2[0], L);
        ry = linsep(p1[1], p2[1], L);
        rz = linsep(p1[2], p2[2], L);
    } else { /* open box: plain Euclidean separation */
        rx = p2[0] - p1[0];
        ry = p2[1] - p1[1];
        rz = p2[2] - p1[2];
    }
    return sqrt(rx * rx + ry * ry + rz * rz);
}

static inline double sep_sph(const double* p1, const double* p2) {
    /* SphericalSurvey.cpp:20-23; p = (r, mu, phi) */
    double cosgamma = sqrt((1 - p1[1] * p1[1]) * (1 - p2[1] * p2[1])) * cos(p1[2] - p2[2]) + p1[1] * p2[1];
    return sqrt(fmax(p1[0] * p1[0] + p2[0] * p2[0] - 2 * p1[0] * p2[0] * cosgamma, 0.0));
}

/* Analytic test correlation functions of TestModel.cpp:13-25 plus a
 * constant; kind 0 = tabulated QSpline. */
enum { XI_TABLE = 0, XI_CONST = 1, XI_GAUSS = 2, XI_EXP = 3 };

typedef struct {
    int kind;
    double A, b;
    qspline q;
} xifunc;

static inline double xi_eval(const xifunc* f, double r) {
    switch (f->kind) {
    case XI_CONST: return f->A;
    case XI_GAUSS: return f->A * exp(-f->b * r * r);
    case XI_EXP: return f->A * exp(-f->b * r);
    default: return qspline_eval(&f->q, r);
    }
}

static inline double cb(double x) { return x * x * x; }

/* Canonical cell bounds of grid cell (d1,d2,d3), Survey.cpp:80-97.
 * grid = {Min1,Max1,Min2,Max2,Min3,Max3} ; n = {N1,N2,N3}. */
static void grid_cell(const double* grid, const int* n, int d1, int d2, int d3, double* c) {
    c[0] = grid[0] + d1 * (grid[1] - grid[0]) / n[0];
    c[1] = grid[0] + (d1 + 1) * (grid[1] - grid[0]) / n[0];
    c[2] = grid[2] + d2 * (grid[3] - grid[2]) / n[1];
    c[3] = grid[2] + (d2 + 1) * (grid[3] - grid[2]) / n[1];
    c[4] = grid[4] + d3 * (grid[5] - grid[4]) / n[2];
    c[5] = grid[4] + (d3 + 1) * (grid[5] - grid[4]) / n[2];
}

/* Gauss product-rule cell-pair integral for several correlation functions
 * at once.  c1, c2 = {min1,max1,min2,max2,min3,max3}.  coordsys 1 =
 * Cartesian (affine map, sig.cpp:388-410), 2 = spherical (r^3 map,
 * sig.cpp:436-461).  out[t] = Q for xi[t]. */
static void q_gauss(int coordsys, double L, const double* c1, const double* c2, int ng, const double* u,
                    const double* w, int ntab, const xifunc* xi, double* out) {
    int np = ng * ng * ng;
    double* P1 = (double*)malloc(sizeof(double) * 3 * np);
    double* P2 = (double*)malloc(sizeof(double) * 3 * np);
    double* W1 = (double*)malloc(sizeof(double) * np);
    double* W2 = (double*)malloc(sizeof(double) * np);
    for (int i = 0; i < ng; i++)
        for (int j = 0; j < ng; j++)
            for (int l = 0; l < ng; l++) {
                int p = (i * ng + j) * ng + l;
                if (coordsys == 1) {
                    P1[3 * p + 0] = (1 - u[i]) * c1[0] + u[i] * c1[1];
                    P1[3 * p + 1] = (1 - u[j]) * c1[2] + u[j] * c1[3];
                    P1[3 * p + 2] = (1 - u[l]) * c1[4] + u[l] * c1[5];
                    P2[3 * p + 0] = (1 - u[i]) * c2[0] + u[i] * c2[1];
                    P2[3 * p + 1] = (1 - u[j]) * c2[2] + u[j] * c2[3];
                    P2[3 * p + 2] = (1 - u[l]) * c2[4] + u[l] * c2[5];
                } else {
                    P1[3 * p + 0] = cbrt((1 - u[i]) * cb(c1[0]) + u[i] * cb(c1[1]));
                    P1[3 * p + 1] = (1 - u[j]) * c1[2] + u[j] * c1[3];
                    P1[3 * p + 2] = (1 - u[l]) * c1[4] + u[l] * c1[5];
                    P2[3 * p + 0] = cbrt((1 - u[i]) * cb(c2[0]) + u[i] * cb(c2[1]));
                    P2[3 * p + 1] = (1 - u[j]) * c2[2] + u[j] * c2[3];
                    P2[3 * p + 2] = (1 - u[l]) * c2[4] + u[l] * c2[5];
                }
                W1[p] = W2[p] = w[i] * w[j] * w[l];
            }
    for (int t = 0; t < ntab; t++) out[t] = 0;
    double* acc = (double*)calloc((size_t)(ntab > 0 ? ntab : 1), sizeof(double));
    for (int p = 0; p < np; p++) {
        for (int t = 0; t < ntab; t++) acc[t] = 0;
        for (int q = 0; q < np; q++) {
            double r = (coordsys == 1) ? sep_box(&P1[3 * p], &P2[3 * q], L) : sep_sph(&P1[3 * p], &P2[3 * q]);
            for (int t = 0; t < ntab; t++) acc[t] += W2[q] * xi_eval(&xi[t], r);
        }
        for (int t = 0; t < ntab; t++) out[t] += W1[p] * acc[t];
    }
    free(acc);
    free(P1);
    free(P2);
    free(W1);
    free(W2);
}

/* Build xifunc descriptors: kinds[t], A[t], b[t]; tabulated ones share the
 * r-grid (n1,n2,X,U) and use Y + t*(n1+n2). */
static xifunc* make_xi(int ntab, const int* kinds, const double* A, const double* b, int n1, int n2,
                       const double* X, const double* U, const double* Y) {
    if (ntab <= 0) return NULL;
    xifunc* xi = (xifunc*)calloc((size_t)ntab, sizeof(xifunc));
    for (int t = 0; t < ntab; t++) {
        xi[t].kind = kinds ? kinds[t] : XI_TABLE;
        xi[t].A = A ? A[t] : 0;
        xi[t].b = b ? b[t] : 0;
        xi[t].q.n1 = n1;
        xi[t].q.n2 = n2;
        xi[t].q.X = X;
        xi[t].q.U = U;
        xi[t].q.Y = Y ? Y + (size_t)t * (n1 + n2) : NULL;
    }
    return xi;
}

/* Q for explicit cell pairs.  cells1/cells2: npair x 6 bounds. out: npair x ntab. */
void orc_q_pairs(int coordsys, double L, int npair, const double* cells1, const double* cells2, int ng,
                 int ntab, const int* kinds, const double* A, const double* b, int n1, int n2,
                 const double* X, const double* U, const double* Y, double* out) {
    double u[64], w[64];
    orc_gauss_legendre01(ng, u, w);
    xifunc* xi = make_xi(ntab, kinds, A, b, n1, n2, X, U, Y);
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < npair; k++)
        q_gauss(coordsys, L, &cells1[6 * k], &cells2[6 * k], ng, u, w, ntab, xi, &out[(size_t)k * ntab]);
    free(xi);
}

/* Q table entries by symmetry key, canonical grid geometry.
 * Cartesian (sig.cpp:99-119): key = (kx,ky,kz), first cell = grid (0,0,0),
 *   second = grid (kx,ky,kz).
 * Spherical (sig.cpp:150-207): key = (ha,hb,df) with h = dr*Nmu + dmu;
 *   first cell = arc min(ha,hb) at phi index 0, second = arc max(ha,hb) at
 *   phi index df.
 * keys: nkey x 3 ints.  out: nkey x ntab. */
void orc_qtable_keys(int coordsys, const double* grid, const int* n, double L, int nkey, const int* keys,
                     int ng, int ntab, const int* kinds, const double* A, const double* b, int n1, int n2,
                     const double* X, const double* U, const double* Y, double* out) {
    double u[64], w[64];
    orc_gauss_legendre01(ng, u, w);
    xifunc* xi = make_xi(ntab, kinds, A, b, n1, n2, X, U, Y);
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < nkey; k++) {
        double c1[6], c2[6];
        const int* key = &keys[3 * k];
        if (coordsys == 1) {
            grid_cell(grid, n, 0, 0, 0, c1);
            grid_cell(grid, n, key[0], key[1], key[2], c2);
        } else {
            int ha = key[0] < key[1] ? key[0] : key[1];
            int hb = key[0] < key[1] ? key[1] : key[0];
            int Nmu = n[1];
            grid_cell(grid, n, ha / Nmu, ha % Nmu, 0, c1);
            grid_cell(grid, n, hb / Nmu, hb % Nmu, key[2], c2);
        }
        q_gauss(coordsys, L, c1, c2, ng, u, w, ntab, xi, &out[(size_t)k * ntab]);
    }
    free(xi);
}

/* Separation helpers exposed for the known-answer tests. */
double orc_sep_box(const double* p1, const double* p2, double L) { return sep_box(p1, p2, L); }
double orc_sep_sph(const double* p1, const double* p2) { return sep_sph(p1, p2); }
