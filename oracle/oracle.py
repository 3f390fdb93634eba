"""FP64 CPU oracle for the Fisher-build path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this module; the GPU library never calls it.  It restates the
reference pipeline (jwgcarlson/OPSEC, paths relative to its root):

  xi / xi_p tables       code/opsec/src/Model.cpp:84-123, RealModel.cpp:85-127
  Q by symmetry key      code/opsec/src/sig.cpp:82-213 (Gauss product rule here)
  S = sqrt(Nbar Nbar) Q  code/opsec/src/sig.cpp:120,203
  top-M eigenpairs       code/opsec/src/klt.cpp:197-248 (LAPACK dsyevr via scipy)
  C_p = B^T S_p B packed code/opsec/src/comma-scalapack.cpp:228-265
  y = B^T x              code/opsec/src/dot.cpp:120-152
  F, f, q                code/opsec/src/estimate-mpi.cpp:480-546 (one rank)
  mixing, p-hat, Cov     code/opsec/src/estimate-mpi.cpp:565-641 with the
                         storage-order behaviour of MyMatrix.hpp:447-456

The C core (oracle.c, genz_malik.c) is built by oracle/Makefile into
oracle/liboracle.so.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

# Table layouts: (n1 linear points on [0, r1), n2 log points on [r1, r2])
LAYOUT_REFERENCE = (512, 256, 200.0, 20000.0)  # RealModel.cpp:99-102
LAYOUT_LOG4096 = (256, 4096, 10.0, 20000.0)    # 4096 log-spaced r beyond r = 10


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
        L = C.CDLL(path)
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        L.orc_cspline_coeffs.argtypes = [C.c_int, dp, dp, dp, dp, dp]
        L.orc_cspline_eval.argtypes = [C.c_int, dp, dp, dp, dp, dp, C.c_double]
        L.orc_cspline_eval.restype = C.c_double
        L.orc_simpson_weights.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, dp, dp]
        L.orc_simpson_nodes.argtypes = [C.c_int, C.c_double, C.c_double, dp]
        L.orc_xi_sum.argtypes = [C.c_int, dp, dp, C.c_int, dp, dp]
        L.orc_band_prior.argtypes = [C.c_int, dp, dp, dp, dp, dp, C.c_double, C.c_double]
        L.orc_band_prior.restype = C.c_double
        L.orc_qspline_array.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, dp]
        L.orc_qspline_eval.argtypes = [C.c_int, C.c_int, dp, dp, dp, C.c_double]
        L.orc_qspline_eval.restype = C.c_double
        L.orc_gauss_legendre01.argtypes = [C.c_int, dp, dp]
        vp = C.c_void_p
        L.orc_q_pairs.argtypes = [C.c_int, C.c_double, C.c_int, dp, dp, C.c_int, C.c_int, vp, vp, vp,
                                  C.c_int, C.c_int, vp, vp, vp, dp]
        L.orc_qtable_keys.argtypes = [C.c_int, dp, ip, C.c_double, C.c_int, ip, C.c_int, C.c_int, vp, vp, vp,
                                      C.c_int, C.c_int, vp, vp, vp, dp]
        L.orc_sep_box.argtypes = [dp, dp, C.c_double]
        L.orc_sep_box.restype = C.c_double
        L.orc_sep_sph.argtypes = [dp, dp]
        L.orc_sep_sph.restype = C.c_double
        L.orc_gm_pair.argtypes = [C.c_int, C.c_double, dp, dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                                  vp, vp, vp, C.c_uint, C.c_double, C.c_double, C.POINTER(C.c_double),
                                  C.POINTER(C.c_int)]
        L.orc_gm_pair.restype = C.c_double
        L.orc_gm_pairs.argtypes = [C.c_int, C.c_double, C.c_int, dp, dp, C.c_int, C.c_double, C.c_double, C.c_int,
                                   C.c_int, vp, vp, vp, C.c_uint, C.c_double, C.c_double, dp, vp]
        _LIB = L
    return _LIB


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------- splines
class CubicSpline:
    """fmm cubic spline of tabulated P(k), zero outside [k0, k_last)."""

    def __init__(self, x, y):
        self.x, self.y = _f64(x), _f64(y)
        n = self.x.size
        self.b, self.c, self.d = np.zeros(n), np.zeros(n), np.zeros(n)
        lib().orc_cspline_coeffs(n, self.x, self.y, self.b, self.c, self.d)

    def __call__(self, k):
        L = lib()
        k = np.atleast_1d(np.asarray(k, dtype=np.float64))
        return np.array([L.orc_cspline_eval(self.x.size, self.x, self.y, self.b, self.c, self.d, float(v))
                         for v in k])


def simpson_nodes(nk, kmin, kmax):
    k = np.zeros(nk + 1)
    lib().orc_simpson_nodes(nk, kmin, kmax, k)
    return k


def r_grid(layout=LAYOUT_REFERENCE):
    n1, n2, r1, r2 = layout
    X = np.zeros(n1 + n2)
    lib().orc_qspline_array(n1, n2, r1, r2, X)
    U = np.log(X[n1:])
    return X, U


def xi_tables(pk_k, pk_P, bands, layout=LAYOUT_REFERENCE):
    """Rows: xi (GetXi, Nk=32768 on [0,10]) then xi_p for each band (GetXiDeriv,
    Nk=8192 on the band with P = 1 on [kmin, kmax) and 0 elsewhere)."""
    L = lib()
    X, _ = r_grid(layout)
    n = X.size
    spl = CubicSpline(pk_k, pk_P)
    out = np.zeros((1 + len(bands), n))
    # xi
    k = simpson_nodes(32768, 0.0, 10.0)
    Pk = spl(k)
    mult = np.zeros_like(k)
    L.orc_simpson_weights(2, 32768, 0.0, 10.0, 1.0, Pk, mult)
    L.orc_xi_sum(n, X, out[0], 32768, k, mult)
    for p, (kmin, kmax) in enumerate(bands):
        k = simpson_nodes(8192, kmin, kmax)
        Pk = ((k >= kmin) & (k < kmax)).astype(np.float64)  # ConstantSpline(1,kmin,kmax)
        mult = np.zeros_like(k)
        L.orc_simpson_weights(2, 8192, kmin, kmax, 1.0, Pk, mult)
        row = np.zeros(n)
        L.orc_xi_sum(n, X, row, 8192, k, mult)
        out[1 + p] = row
    return out


def band_priors(pk_k, pk_P, bands):
    spl = CubicSpline(pk_k, pk_P)
    L = lib()
    return np.array([L.orc_band_prior(spl.x.size, spl.x, spl.y, spl.b, spl.c, spl.d, lo, hi) for lo, hi in bands])


def qspline_eval(Y, r, layout=LAYOUT_REFERENCE):
    X, U = r_grid(layout)
    n1, n2 = layout[0], layout[1]
    L = lib()
    Y = _f64(Y)
    return np.array([L.orc_qspline_eval(n1, n2, X, U, Y, float(v)) for v in np.atleast_1d(r)])


# ---------------------------------------------------------------- Q tables
def _xi_args(tables, kinds=None, A=None, b=None):
    ntab = len(kinds) if tables is None else tables.shape[0]
    k = None if kinds is None else _i32(kinds)
    a = None if A is None else _f64(A)
    bb = None if b is None else _f64(b)
    y = None if tables is None else _f64(tables)
    return ntab, k, a, bb, y


def keys_all(survey, fold=False):
    """Every symmetry key of the reference's cache (sig.cpp:99-119,150-207).

    Cartesian: (kx,ky,kz) over [0,Nx)x[0,Ny)x[0,Nz).  Spherical: (ha,hb,df)
    with ha <= hb (Q is symmetric in the two arcs) and df over [0,Nphi), or
    over [0,Nphi/2] when fold=True on a full-sky grid."""
    N1, N2, N3 = survey.n
    if survey.coordsys == 1:
        g = np.indices((N1, N2, N3)).reshape(3, -1).T
        return _i32(g)
    H = N1 * N2
    nf = N3 // 2 + 1 if fold else N3
    ha, hb = np.triu_indices(H)
    df = np.arange(nf)
    keys = np.stack([np.repeat(ha, nf), np.repeat(hb, nf), np.tile(df, ha.size)], axis=1)
    return _i32(keys)


def qtable_keys(survey, keys, tables=None, layout=LAYOUT_REFERENCE, ng=4, kinds=None, A=None, b=None):
    """Q[key, t] by the ng^3 x ng^3 Gauss rule on the canonical pair of each key."""
    ntab, k, a, bb, y = _xi_args(tables, kinds, A, b)
    X, U = r_grid(layout)
    keys = _i32(keys).reshape(-1, 3)
    out = np.zeros((keys.shape[0], ntab))
    lib().orc_qtable_keys(survey.coordsys, _f64(survey.bounds), _i32(survey.n), survey.L, keys.shape[0], keys, ng,
                          ntab, _ptr(k), _ptr(a), _ptr(bb), layout[0], layout[1], _ptr(X), _ptr(U), _ptr(y), out)
    return out


def q_pairs(coordsys, L, cells1, cells2, tables=None, layout=LAYOUT_REFERENCE, ng=4, kinds=None, A=None, b=None):
    ntab, k, a, bb, y = _xi_args(tables, kinds, A, b)
    X, U = r_grid(layout)
    c1, c2 = _f64(cells1).reshape(-1, 6), _f64(cells2).reshape(-1, 6)
    out = np.zeros((c1.shape[0], ntab))
    lib().orc_q_pairs(coordsys, L, c1.shape[0], c1, c2, ng, ntab, _ptr(k), _ptr(a), _ptr(bb), layout[0], layout[1],
                      _ptr(X), _ptr(U), _ptr(y), out)
    return out


def gm_pair(coordsys, L, c1, c2, Y=None, layout=LAYOUT_REFERENCE, kind=0, A=0.0, b=0.0, abs_bound=1e-5,
            rel_bound=1e-10, maxeval=50000000):
    """Reference adaptive cubature restated (genz_malik.c); returns (val, err, neval)."""
    X, U = r_grid(layout)
    err = C.c_double()
    nev = C.c_int()
    y = None if Y is None else _f64(Y)
    v = lib().orc_gm_pair(coordsys, L, _f64(c1), _f64(c2), kind, A, b, layout[0], layout[1], _ptr(X), _ptr(U),
                          _ptr(y), maxeval, abs_bound, rel_bound, C.byref(err), C.byref(nev))
    return v, err.value, nev.value


def gm_pairs(coordsys, L, cells1, cells2, Y, layout=LAYOUT_REFERENCE, abs_bound=1e-5, rel_bound=1e-10,
             maxeval=50000000):
    X, U = r_grid(layout)
    c1, c2 = _f64(cells1).reshape(-1, 6), _f64(cells2).reshape(-1, 6)
    out = np.zeros(c1.shape[0])
    lib().orc_gm_pairs(coordsys, L, c1.shape[0], c1, c2, 0, 0.0, 0.0, layout[0], layout[1], _ptr(X), _ptr(U),
                       _ptr(_f64(Y)), maxeval, abs_bound, rel_bound, out, None)
    return out


def cell_bounds(cells):
    return np.stack([cells["min1"], cells["max1"], cells["min2"], cells["max2"], cells["min3"], cells["max3"]],
                    axis=1)


def key_index(survey, cells, fold=False):
    """For every (a,b) cell pair, the row of keys_all(survey, fold) it reads."""
    d1, d2, d3 = cells["d1"].astype(np.int64), cells["d2"].astype(np.int64), cells["d3"].astype(np.int64)
    N1, N2, N3 = survey.n
    if survey.coordsys == 1:
        kx = np.abs(d1[:, None] - d1[None, :])
        ky = np.abs(d2[:, None] - d2[None, :])
        kz = np.abs(d3[:, None] - d3[None, :])
        return (kx * N2 + ky) * N3 + kz
    H = N1 * N2
    h = d1 * N2 + d2
    ha = np.minimum(h[:, None], h[None, :])
    hb = np.maximum(h[:, None], h[None, :])
    df = np.abs(d3[:, None] - d3[None, :])
    nf = N3 // 2 + 1 if fold else N3
    if fold:
        df = np.minimum(df, N3 - df)
    # row of (ha, hb) in the triangular enumeration of keys_all
    tri = ha * H - ha * (ha - 1) // 2 + (hb - ha)
    return tri * nf + df


def signal_matrix(survey, cells, Q, fold=False):
    """S_ab = sqrt(Nbar_a Nbar_b) Q[key(a,b)] (sig.cpp:120,203) for one table column Q."""
    idx = key_index(survey, cells, fold)
    nb = cells["Nbar"]
    return np.sqrt(nb[:, None] * nb[None, :]) * Q[idx]


# ---------------------------------------------------------------- KL, projection, Fisher
def klt(S, nmodes):
    """Top-nmodes eigenpairs of S in descending order; modes as rows (M x N)."""
    import scipy.linalg

    n = S.shape[0]
    w, V = scipy.linalg.eigh(S, subset_by_index=(n - nmodes, n - 1), driver="evr")
    order = np.argsort(w)[::-1]
    return w[order], np.ascontiguousarray(V[:, order].T)


def packed_ij(M):
    """(i, j) of packed index k = j(j+1)/2 + i, i <= j (column-major upper)."""
    j = np.repeat(np.arange(M), np.arange(1, M + 1))
    k = np.arange(M * (M + 1) // 2)
    i = k - j * (j + 1) // 2
    return i, j


def pack_upper(Cm):
    i, j = packed_ij(Cm.shape[0])
    return Cm[i, j]


def project(modes, Sp):
    """Packed C_p = B^T S_p B with B = modes^T (N x M)."""
    B = modes.T
    return pack_upper(B.T @ Sp @ B)


def dot(cells, counts, modes):
    x = (counts - cells["Nbar"]) / np.sqrt(cells["Nbar"])
    return modes @ x


def fisher(evals, Dp, y, prior):
    """F, f, q of estimate-mpi.cpp:480-546 at one rank.  Dp: [Nb, M(M+1)/2]."""
    M = evals.size
    i, j = packed_ij(M)
    C_ = 1.0 + evals
    Cinv = 1.0 / C_
    mult = np.where(i == j, 0.5, 1.0)
    R = np.where(i == j, C_[i], 0.0) - prior @ Dp
    wk = mult * Cinv[i] * Cinv[j]
    G = Dp * wk
    F = G @ Dp.T
    f = G @ R
    q = G @ (y[i] * y[j])
    return F, f, q


MIXING = {"inverse": 0, "inverse-sqrt": 1, "identity": 2}


def estimate_epilogue(F, q, f, mixing="inverse"):
    """Mixing matrix, window, estimates and covariance as estimate-mpi.cpp:565-641
    computes them.  multiply() there takes transb from A's storage order
    (MyMatrix.hpp:453-455), so with the default row-major matrices the stored
    W is (M F)^T and the stored covariance is M^T M F; the written q record is
    q - f (axpy in place, :603).  Returns the seven estfile records."""
    nb = F.shape[0]
    if mixing == "inverse":
        Mx = np.linalg.inv(F)
    elif mixing == "inverse-sqrt":
        Fi = np.linalg.inv(F)
        w, V = np.linalg.eigh(Fi)
        Mx = (V * np.sqrt(w)) @ V.T
    else:
        Mx = np.eye(nb)
    W = (Mx @ F).T
    rowsum = W.sum(axis=1)
    Mx = Mx / rowsum[:, None]
    W = (Mx @ F).T
    qmf = q - f
    phat = Mx @ qmf
    pcov = Mx.T @ Mx @ F
    return {"phat": phat, "pcov": pcov, "F": F, "W": W, "M": Mx, "q": qmf, "f": f}


def estimate_epilogue_math(F, q, f, mixing="inverse"):
    """The same quantities with the textbook algebra: W = M F, Cov = M F M^T."""
    nb = F.shape[0]
    if mixing == "inverse":
        Mx = np.linalg.inv(F)
    elif mixing == "inverse-sqrt":
        w, V = np.linalg.eigh(np.linalg.inv(F))
        Mx = (V * np.sqrt(w)) @ V.T
    else:
        Mx = np.eye(nb)
    Mx = Mx / (Mx @ F).sum(axis=1)[:, None]
    return {"phat": Mx @ (q - f), "pcov": Mx @ F @ Mx.T, "W": Mx @ F, "M": Mx}


# ---------------------------------------------------------------- whole pipeline
def fisher_build(survey, cells, counts, pk_k, pk_P, bands, nmodes, layout=LAYOUT_REFERENCE, ng=4, mixing="inverse",
                 fold=False):
    """cells + counts + P(k) -> every intermediate and the estfile records."""
    tabs = xi_tables(pk_k, pk_P, bands, layout)
    keys = keys_all(survey, fold)
    Q = qtable_keys(survey, keys, tabs, layout, ng)
    S = signal_matrix(survey, cells, Q[:, 0], fold)
    evals, modes = klt(S, nmodes)
    Dp = np.stack([project(modes, signal_matrix(survey, cells, Q[:, 1 + p], fold)) for p in range(len(bands))])
    y = dot(cells, counts, modes)
    prior = band_priors(pk_k, pk_P, bands)
    F, f, q = fisher(evals, Dp, y, prior)
    est = estimate_epilogue(F, q, f, mixing)
    return {"tables": tabs, "keys": keys, "Q": Q, "S": S, "evals": evals, "modes": modes, "cov": Dp, "y": y,
            "prior": prior, "F": F, "f": f, "q": q, "est": est}


def gap_nmodes(evals_desc, target, rel_gap=1e-6, span=16):
    """An Nmodes near target whose cut lies in a spectral gap (degenerate
    clusters are not split): the smallest M in [target, target+span] with
    lambda_{M-1} - lambda_M > rel_gap * lambda_0."""
    lam = np.asarray(evals_desc)
    for M in range(target, min(target + span, lam.size - 1) + 1):
        if lam[M - 1] - lam[M] > rel_gap * abs(lam[0]):
            return M
    return target


def subspace_sin(A, B):
    """Largest principal-angle sine between the row spaces of A and B
    (rows orthonormal)."""
    s = np.linalg.svd(A @ B.T, compute_uv=False)
    return float(np.sqrt(max(0.0, 1.0 - min(s) ** 2)))


# ---------------------------------------------------------------- full-sky shells at full size
# On a full-sky spherical grid S depends on the two cells' arcs h = (i_r, j_mu) and on
# |phi_a - phi_b| only (sig.cpp:150-207 keys it so), so S is block circulant in phi and its
# eigenvectors are u_h * cos(2 pi m phi / N_phi) and u_h * sin(...) with u an eigenvector of the
# arc-space matrix  S^(m)[h][g] = sum_d S[(h, 0), (g, d)] cos(2 pi m d / N_phi).
# The restatement below runs klt.cpp:173-248 (top-M eigenpairs), comma-scalapack.cpp:228-252
# (C_p = B^T S_p B) and estimate-mpi.cpp:480-546 (F, f, q) in that basis, in FP64, so that a
# 32,768-cell build is checked without forming or diagonalising the 32,768^2 matrix.  It is the
# same mathematics as the dense path (checked against it on small shells in tests/), not the
# engine's algorithm: one FP64 eigh per order m over all arcs (no mu-parity split), FP64 GEMMs.
def phi_basis(nphi):
    """Orders m = 0..nphi/2, the cos / sin tables [phi][m] and the unit-norm scale per order."""
    m = np.arange(nphi // 2 + 1)
    ang = 2.0 * np.pi * np.outer(np.arange(nphi), m) / nphi
    scale = np.where((m == 0) | (2 * m == nphi), 1.0 / np.sqrt(nphi), np.sqrt(2.0 / nphi))
    return m, np.cos(ang), np.sin(ang), scale


def azimuthal_blocks(srow, nphi):
    """srow: [H][H * nphi], S[(h, phi=0), (g, d)] for every arc h (cell h * nphi) and cell (g, d).
    Returns S^(m) [nm][H][H] (symmetrised)."""
    H = srow.shape[0]
    _, cosb, _, _ = phi_basis(nphi)
    B = np.tensordot(srow.reshape(H, H, nphi), cosb, axes=([2], [0]))  # [h][g][m]
    B = np.ascontiguousarray(np.moveaxis(B, 2, 0))
    return 0.5 * (B + np.transpose(B, (0, 2, 1)))


def klt_azimuthal(B0, nphi, nmodes):
    """Top-nmodes eigenpairs of S from its order blocks.  Orders 0 < m < nphi/2 carry a cos and
    a sin mode per block eigenvalue; the cos mode is ranked first (a cut inside such a pair
    keeps the cos mode).  Returns the kept eigenvalues (descending) and, per (m, trig), the
    block eigenvectors kept and their eigenvalues, and the largest eigenvalue left out."""
    nm = B0.shape[0]
    lam, mm, tt, ii, U = [], [], [], [], []
    for m in range(nm):
        w, V = np.linalg.eigh(B0[m])
        U.append(V)
        trigs = (0,) if (m == 0 or 2 * m == nphi) else (0, 1)
        for t in trigs:
            lam.append(w)
            mm.append(np.full(w.size, m))
            tt.append(np.full(w.size, t))
            ii.append(np.arange(w.size))
    lam, mm, tt, ii = (np.concatenate(a) for a in (lam, mm, tt, ii))
    full = np.lexsort((ii, mm, tt, -lam))
    order = full[:nmodes]
    nxt = float(lam[full[nmodes]]) if full.size > nmodes else None
    groups = {}
    for m in range(nm):
        for t in (0, 1):
            sel = order[(mm[order] == m) & (tt[order] == t)]
            if sel.size:
                idx = ii[sel]
                groups[(m, t)] = {"U": U[m][:, idx], "lam": lam[sel]}
    return lam[order], groups, nxt


def pixel_coefficients(x, H, nphi):
    """X[h][m][trig] = sum_phi x[(h, phi)] * unit-norm cos / sin of order m."""
    _, cosb, sinb, scale = phi_basis(nphi)
    xs = x.reshape(H, nphi)
    return np.stack([xs @ cosb * scale, xs @ sinb * scale], axis=2)


def fisher_azimuthal(srow_of_table, nphi, nbands, nmodes, x, prior):
    """F, f, q (estimate-mpi.cpp:480-546 at one rank) on the top-nmodes KL modes of a full-sky
    shell.  srow_of_table(t): the [H][H * nphi] rows of S_t at phi = 0 (t = 0: xi, 1..nbands:
    the band tables).  x: pixel values (N_a - Nbar_a)/sqrt(Nbar_a) per cell."""
    B0 = srow_of_table(0)
    H = B0.shape[0]
    evals, groups, nxt = klt_azimuthal(azimuthal_blocks(B0, nphi), nphi, nmodes)
    del B0
    X = pixel_coefficients(np.asarray(x, dtype=np.float64), H, nphi)
    keys = sorted(groups)
    C = {g: np.zeros((nbands, groups[g]["U"].shape[1], groups[g]["U"].shape[1])) for g in keys}
    for p in range(nbands):
        Bp = azimuthal_blocks(srow_of_table(1 + p), nphi)
        for (m, t) in keys:
            U = groups[(m, t)]["U"]
            if t == 1 and (m, 0) in groups and groups[(m, 0)]["U"].shape[1] >= U.shape[1]:
                k = U.shape[1]  # the sin modes of an order are the first of its cos modes
                C[(m, t)][p] = C[(m, 0)][p][:k, :k]
                continue
            C[(m, t)][p] = U.T @ Bp[m] @ U
        del Bp
    F = np.zeros((nbands, nbands))
    f = np.zeros(nbands)
    q = np.zeros(nbands)
    for (m, t) in keys:
        g = groups[(m, t)]
        lam = g["lam"]
        w = 1.0 / (1.0 + lam)
        y = g["U"].T @ X[:, m, t]
        Cg = C[(m, t)]
        ww = np.outer(w, w)
        Hg = (Cg * ww).reshape(nbands, -1)
        F += 0.5 * Hg @ Cg.reshape(nbands, -1).T
        R = np.diag(1.0 + lam) - np.tensordot(prior, Cg, axes=(0, 0))
        f += 0.5 * Hg @ R.ravel()
        wy = w * y
        q += 0.5 * np.einsum("pij,i,j->p", Cg, wy, wy)
    return {"evals": evals, "F": F, "f": f, "q": q, "groups": groups, "next_eval": nxt}


def mode_projection_norms(modes, groups, H, nphi):
    """For each row of modes [k][H * nphi] (unit vectors), the squared norm of its projection
    onto the span of the kept azimuthal modes in groups."""
    _, cosb, sinb, scale = phi_basis(nphi)
    V = np.asarray(modes).reshape(-1, H, nphi)
    coef = (np.tensordot(V, cosb, axes=([2], [0])) * scale, np.tensordot(V, sinb, axes=([2], [0])) * scale)
    out = np.zeros(V.shape[0])
    for (m, t), g in groups.items():
        out += np.sum((coef[t][:, :, m] @ g["U"]) ** 2, axis=1)
    return out
