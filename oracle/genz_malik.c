/* genz_malik.c -- restatement of the reference's adaptive cell-pair cubature.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.c).  It times and checks the
 * reference CPU algorithm: the reference integrates every cell pair with
 * adapt_integrate_v (code/opsec/src/sig.cpp:419-482), i.e. the embedded
 * degree-7/degree-5 fully symmetric rule of
 *     A. C. Genz and A. A. Malik, "An imbedded family of fully symmetric
 *     numerical integration rules", SIAM J. Numer. Anal. 20, 580-588 (1983),
 * driven by a globally adaptive bisection loop that splits the regions of
 * largest error estimate along the axis of largest fourth difference, in
 * batches large enough to bring the error under the bound
 * (code/opsec/src/cubature.c:460-576 for the rule, :885-998 for the loop).
 *
 * The reference passes (maxeval, epsrel, epsabs) into the slots
 * (maxEval, reqAbsError, reqRelError) (sig.cpp:427-430 against
 * cubature.h:66-72), so the stop rule it actually applies is
 *     err <= epsrel  OR  |err/val| <= epsabs.
 * orc_gm_pair takes the two bounds under the names of the slots they fill.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define GM_DIM 6
#define GM_NPTS (1 + 4 * GM_DIM + 2 * GM_DIM * (GM_DIM - 1) + (1 << GM_DIM)) /* 149 */

typedef struct {
    double c[GM_DIM], h[GM_DIM];
    double vol, val, err;
    int split;
} gm_region;

/* integrand context: the two cells, the separation and xi (shared with oracle.c) */
typedef struct {
    int coordsys;
    double L;
    double lo[GM_DIM], hi[GM_DIM]; /* per-dimension map, sig.cpp:383-386 ordering */
    int xikind;
    double A, b;
    int n1, n2;
    const double *X, *U, *Y;
} gm_ctx;

double orc_qspline_eval(int n1, int n2, const double* X, const double* U, const double* Y, double x);
double orc_sep_box(const double* p1, const double* p2, double L);
double orc_sep_sph(const double* p1, const double* p2);

static double gm_xi(const gm_ctx* g, double r) {
    switch (g->xikind) {
    case 1: return g->A;
    case 2: return g->A * exp(-g->b * r * r);
    case 3: return g->A * exp(-g->b * r);
    default: return orc_qspline_eval(g->n1, g->n2, g->X, g->U, g->Y, r);
    }
}

/* The integrand at u in [0,1]^6 (sig.cpp:388-410 Cartesian: u0..2 -> cell 1,
 * u3..5 -> cell 2; sig.cpp:436-461 spherical: u0,u1 -> r^3 of cells 1,2,
 * u2,u3 -> mu, u4,u5 -> phi). */
static double gm_f(const gm_ctx* g, const double* u) {
    double p1[3], p2[3];
    if (g->coordsys == 1) {
        for (int d = 0; d < 3; d++) {
            p1[d] = (1 - u[d]) * g->lo[d] + u[d] * g->hi[d];
            p2[d] = (1 - u[3 + d]) * g->lo[3 + d] + u[3 + d] * g->hi[3 + d];
        }
        return gm_xi(g, orc_sep_box(p1, p2, g->L));
    }
    p1[0] = cbrt((1 - u[0]) * g->lo[0] + u[0] * g->hi[0]);
    p2[0] = cbrt((1 - u[1]) * g->lo[1] + u[1] * g->hi[1]);
    p1[1] = (1 - u[2]) * g->lo[2] + u[2] * g->hi[2];
    p2[1] = (1 - u[3]) * g->lo[3] + u[3] * g->hi[3];
    p1[2] = (1 - u[4]) * g->lo[4] + u[4] * g->hi[4];
    p2[2] = (1 - u[5]) * g->lo[5] + u[5] * g->hi[5];
    return gm_xi(g, orc_sep_sph(p1, p2));
}

/* Apply the degree-7 rule and its degree-5 companion to one region. */
static void gm_apply(const gm_ctx* g, gm_region* R) {
    const int D = GM_DIM;
    const double l2 = sqrt(9.0 / 70.0), l4 = sqrt(9.0 / 10.0), l5 = sqrt(9.0 / 19.0);
    const double w1 = (12824.0 - 9120.0 * D + 400.0 * D * D) / 19683.0;
    const double w2 = 980.0 / 6561.0;
    const double w3 = (1820.0 - 400.0 * D) / 19683.0;
    const double w4 = 200.0 / 19683.0;
    const double w5 = 6859.0 / 19683.0 / (double)(1 << D);
    const double e1 = (729.0 - 950.0 * D + 50.0 * D * D) / 729.0;
    const double e2 = 245.0 / 486.0;
    const double e3 = (265.0 - 100.0 * D) / 1458.0;
    const double e4 = 25.0 / 729.0;
    const double ratio = (l2 * l2) / (l4 * l4);
    double p[GM_DIM];

    memcpy(p, R->c, sizeof p);
    const double f0 = gm_f(g, p);

    /* axis points at +-l2 and +-l4; fourth differences pick the split axis */
    double s2 = 0, s3 = 0, best = 0;
    int split = 0;
    for (int k = 0; k < D; k++) {
        double a, bb, c, d;
        p[k] = R->c[k] - l2 * R->h[k]; a = gm_f(g, p);
        p[k] = R->c[k] + l2 * R->h[k]; bb = gm_f(g, p);
        p[k] = R->c[k] - l4 * R->h[k]; c = gm_f(g, p);
        p[k] = R->c[k] + l4 * R->h[k]; d = gm_f(g, p);
        p[k] = R->c[k];
        s2 += a + bb;
        s3 += c + d;
        double diff = fabs(a + bb - 2 * f0 - ratio * (c + d - 2 * f0));
        if (diff > best) { best = diff; split = k; }
    }

    /* pairs of axes at (+-l4, +-l4) */
    double s4 = 0;
    for (int i = 0; i < D - 1; i++)
        for (int j = i + 1; j < D; j++) {
            const double di = l4 * R->h[i], dj = l4 * R->h[j];
            p[i] = R->c[i] - di; p[j] = R->c[j] - dj; s4 += gm_f(g, p);
            p[i] = R->c[i] + di; s4 += gm_f(g, p);
            p[j] = R->c[j] + dj; s4 += gm_f(g, p);
            p[i] = R->c[i] - di; s4 += gm_f(g, p);
            p[i] = R->c[i]; p[j] = R->c[j];
        }

    /* the 2^D corners at +-l5 */
    double s5 = 0;
    for (unsigned m = 0; m < (1u << D); m++) {
        for (int k = 0; k < D; k++) p[k] = R->c[k] + ((m >> k) & 1 ? -l5 : l5) * R->h[k];
        s5 += gm_f(g, p);
    }

    const double r7 = R->vol * (w1 * f0 + w2 * s2 + w3 * s3 + w4 * s4 + w5 * s5);
    const double r5 = R->vol * (e1 * f0 + e2 * s2 + e3 * s3 + e4 * s4);
    R->val = r7;
    R->err = fabs(r5 - r7);
    R->split = split;
}

/* ---- max-heap of regions keyed by error ---- */
typedef struct {
    gm_region* a;
    int n, cap;
    double val, err; /* running totals */
} gm_heap;

static void heap_push(gm_heap* H, const gm_region* R) {
    if (H->n == H->cap) {
        H->cap = H->cap ? 2 * H->cap : 16;
        H->a = (gm_region*)realloc(H->a, sizeof(gm_region) * H->cap);
    }
    H->val += R->val;
    H->err += R->err;
    int i = H->n++;
    while (i > 0) {
        int parent = (i - 1) / 2;
        if (R->err <= H->a[parent].err) break;
        H->a[i] = H->a[parent];
        i = parent;
    }
    H->a[i] = *R;
}

static gm_region heap_pop(gm_heap* H) {
    gm_region top = H->a[0];
    int n = --H->n, i = 0;
    H->a[0] = H->a[n];
    for (;;) {
        int c = 2 * i + 1, big = i;
        if (c >= n) break;
        if (H->a[c].err > H->a[big].err) big = c;
        if (c + 1 < n && H->a[c + 1].err > H->a[big].err) big = c + 1;
        if (big == i) break;
        gm_region t = H->a[i];
        H->a[i] = H->a[big];
        H->a[big] = t;
        i = big;
    }
    H->val -= top.val;
    H->err -= top.err;
    return top;
}

static int converged(double val, double err, double abs_bound, double rel_bound) {
    double rel = (val == 0.0) ? HUGE_VAL : fabs(err / val);
    return err <= abs_bound || rel <= rel_bound;
}

/* Integrate one cell pair.  cell = {min1,max1,min2,max2,min3,max3}.
 * xikind: 0 tabulated QSpline (n1,n2,X,U,Y), 1 constant A, 2 A exp(-b r^2),
 * 3 A exp(-b r).  Returns the integral; *err and *neval report the final
 * error estimate and the number of integrand evaluations. */
double orc_gm_pair(int coordsys, double L, const double* c1, const double* c2, int xikind, double A, double b,
                   int n1, int n2, const double* X, const double* U, const double* Y, unsigned maxeval,
                   double abs_bound, double rel_bound, double* err, int* neval) {
    gm_ctx g;
    memset(&g, 0, sizeof g);
    g.coordsys = coordsys;
    g.L = L;
    g.xikind = xikind;
    g.A = A;
    g.b = b;
    g.n1 = n1;
    g.n2 = n2;
    g.X = X;
    g.U = U;
    g.Y = Y;
    if (coordsys == 1) {
        for (int d = 0; d < 3; d++) {
            g.lo[d] = c1[2 * d];
            g.hi[d] = c1[2 * d + 1];
            g.lo[3 + d] = c2[2 * d];
            g.hi[3 + d] = c2[2 * d + 1];
        }
    } else {
        g.lo[0] = c1[0] * c1[0] * c1[0]; g.hi[0] = c1[1] * c1[1] * c1[1];
        g.lo[1] = c2[0] * c2[0] * c2[0]; g.hi[1] = c2[1] * c2[1] * c2[1];
        g.lo[2] = c1[2]; g.hi[2] = c1[3];
        g.lo[3] = c2[2]; g.hi[3] = c2[3];
        g.lo[4] = c1[4]; g.hi[4] = c1[5];
        g.lo[5] = c2[4]; g.hi[5] = c2[5];
    }

    gm_heap H = {0};
    gm_region R0;
    for (int d = 0; d < GM_DIM; d++) {
        R0.c[d] = 0.5;
        R0.h[d] = 0.5;
    }
    R0.vol = 1.0;
    gm_apply(&g, &R0);
    heap_push(&H, &R0);
    unsigned nev = GM_NPTS;

    gm_region* batch = NULL;
    int bcap = 0;
    while (nev < maxeval || maxeval == 0) {
        if (converged(H.val, H.err, abs_bound, rel_bound)) break;
        /* pop the worst regions until the rest would meet the bound */
        double bval = H.val, berr = H.err;
        int nb = 0;
        do {
            if (nb + 2 > bcap) {
                bcap = 2 * (nb + 2);
                batch = (gm_region*)realloc(batch, sizeof(gm_region) * bcap);
            }
            gm_region R = heap_pop(&H);
            berr -= R.err;
            int d = R.split;
            R.h[d] *= 0.5;
            R.vol *= 0.5;
            gm_region R2 = R;
            R.c[d] -= R.h[d];
            R2.c[d] += R.h[d];
            batch[nb++] = R;
            batch[nb++] = R2;
            nev += 2 * GM_NPTS;
            if (converged(bval, berr, abs_bound, rel_bound)) break;
        } while (H.n > 0 && (nev < maxeval || maxeval == 0));
        for (int i = 0; i < nb; i++) gm_apply(&g, &batch[i]);
        for (int i = 0; i < nb; i++) heap_push(&H, &batch[i]);
    }
    double v = 0, e = 0;
    for (int i = 0; i < H.n; i++) {
        v += H.a[i].val;
        e += H.a[i].err;
    }
    free(batch);
    free(H.a);
    if (err) *err = e;
    if (neval) *neval = (int)nev;
    return v;
}

/* Many pairs at once (OpenMP over pairs). */
void orc_gm_pairs(int coordsys, double L, int npair, const double* cells1, const double* cells2, int xikind,
                  double A, double b, int n1, int n2, const double* X, const double* U, const double* Y,
                  unsigned maxeval, double abs_bound, double rel_bound, double* out, double* err) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int k = 0; k < npair; k++)
        out[k] = orc_gm_pair(coordsys, L, &cells1[6 * k], &cells2[6 * k], xikind, A, b, n1, n2, X, U, Y, maxeval,
                             abs_bound, rel_bound, err ? &err[k] : NULL, NULL);
}
