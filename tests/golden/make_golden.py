"""Generate tests/golden/reference_vectors.npz from the reference's own code.

Run where the reference checkout is present (it is absent on GPU hosts):

    make -C oracle ref REF=<checkout>/code/opsec/src   # builds oracle/_ref/libopsecref.so
    python tests/golden/make_golden.py

The library is the reference's unmodified sources (code/opsec/src: sig.cpp,
cubature.c, Spline.cpp, QSpline.cpp, Model.cpp, RealModel.cpp, TestModel.cpp,
BoxSurvey.cpp, SphericalSurvey.cpp, ...) plus oracle/ref_shim.cpp.  The
vectors pin the oracle restatement:

* xi tables of RealModel::GetXi / GetXiDeriv (RealModel.cpp:98-127);
* the fmm cubic spline of P(k) and the QSpline lookup (Spline.cpp, QSpline.cpp);
* periodic-box and spherical separations (BoxSurvey.cpp:26-37, SphericalSurvey.cpp:20-23),
  including the two cases of testBoxSurvey.cpp:15-24;
* adaptive cell-pair integrals ComputeSignalC / ComputeSignalS (sig.cpp:419-482);
* the known answer of testsig.cpp:41-66 (periodic Gaussian xi);
* full signal-matrix blocks ComputeSignalMatrixBlock (sig.cpp:50-213) on a
  4x4x4 box and a 3x4x6 spherical grid.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from opsec_gpu import synth  # noqa: E402
import oracle as O  # noqa: E402


def load_ref():
    path = os.path.join(ROOT, "oracle", "_ref", "libopsecref.so")
    R = C.CDLL(path)
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
    R.ref_xi_table.argtypes = [C.c_int, dp, dp, C.c_double, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double,
                               dp, dp]
    R.ref_cspline_eval.argtypes = [C.c_int, dp, dp, C.c_double]
    R.ref_cspline_eval.restype = C.c_double
    R.ref_qspline_eval.argtypes = [C.c_int, C.c_int, dp, dp, C.c_int, dp, dp]
    R.ref_sep.argtypes = [C.c_int, C.c_double, dp, dp]
    R.ref_sep.restype = C.c_double
    R.ref_signal_pair.argtypes = [C.c_int, C.c_double, dp, dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                                  dp, dp, C.c_double, C.c_double, C.POINTER(C.c_double)]
    R.ref_signal_pair.restype = C.c_double
    R.ref_signal_block.argtypes = [C.c_int, dp, ip, C.c_double, C.c_int, C.c_void_p, C.c_int, ip, C.c_int, ip, dp,
                                   C.c_int, C.c_int, C.c_int, dp, dp, C.c_double, C.c_double]
    R.ref_sizeof_cell.restype = C.c_int
    R.ref_write_cells.argtypes = [C.c_char_p, C.c_int, dp, ip, C.c_double, C.c_int, C.c_void_p]
    assert R.ref_sizeof_cell() == 80
    return R


def main():
    R = load_ref()
    out = {}
    k, P = synth.pk_table()
    out["pk_k"], out["pk_P"] = k, P
    bands = synth.band_edges(20, 0.0, 0.2)
    sel = [0, 7, 19]
    out["bands_sel"] = bands[sel]
    n1, n2, r1, r2 = O.LAYOUT_REFERENCE
    X = np.zeros(n1 + n2)
    tabs = np.zeros((1 + len(sel), n1 + n2))
    R.ref_xi_table(len(k), k, P, 0.0, 0.0, n1, n2, r1, r2, X, tabs[0])
    for i, p in enumerate(sel):
        R.ref_xi_table(len(k), k, P, bands[p, 0], bands[p, 1], n1, n2, r1, r2, X, tabs[1 + i])
    out["xi_r"], out["xi_tables"] = X, tabs

    ks = np.array([0.0, 5e-5, 1e-4, 3e-3, 0.0199, 0.02, 0.17, 1.3, 9.99, 10.0, 12.0])
    out["cspline_k"] = ks
    out["cspline_P"] = np.array([R.ref_cspline_eval(len(k), k, P, float(v)) for v in ks])

    rs = np.array([-1.0, 0.0, 1e-3, 0.37, 5.0, 199.999, 200.0, 200.001, 633.0, 19999.0, 20000.0, 25000.0])
    qv = np.zeros(rs.size)
    R.ref_qspline_eval(n1, n2, X, tabs[0].copy(), rs.size, rs, qv)
    out["qspline_r"], out["qspline_xi"] = rs, qv

    # separations: testBoxSurvey.cpp:15-24 plus wrapped and spherical points
    P1 = np.array([[10, 20, 30], [10, 20, 30], [1, 2, 3], [95, 5, 50]], dtype=np.float64)
    P2 = np.array([[70, 80, 90], [70, 80, 50], [99, 98, 97], [5, 95, 50]], dtype=np.float64)
    out["sep_box_p1"], out["sep_box_p2"] = P1, P2
    out["sep_box_L"] = 100.0
    out["sep_box"] = np.array([R.ref_sep(1, 100.0, a.copy(), b.copy()) for a, b in zip(P1, P2)])
    S1 = np.array([[500, 0.3, 1.0], [250, -0.9, 0.1], [999, 0.0, 6.2], [400, 0.5, 2.0]], dtype=np.float64)
    S2 = np.array([[510, 0.31, 1.02], [900, 0.9, 3.0], [998.5, 0.001, 0.05], [400, 0.5, 2.0]], dtype=np.float64)
    out["sep_sph_p1"], out["sep_sph_p2"] = S1, S2
    out["sep_sph"] = np.array([R.ref_sep(2, 0.0, a.copy(), b.copy()) for a, b in zip(S1, S2)])

    # adaptive cell-pair integrals with the RealModel xi table
    svs, cs = synth.shell_survey(8, 8, 8)
    svb, cb_ = synth.box_survey(12)
    bs, bb = O.cell_bounds(cs), O.cell_bounds(cb_)
    pairs_s = [(0, 1), (0, 9), (5, 300), (17, 400), (64, 65), (200, 511), (100, 100)]
    pairs_b = [(0, 1), (0, 13), (5, 300), (0, 1727), (700, 1000), (100, 100)]
    err = C.c_double()
    vals, errs, c1s, c2s, kinds = [], [], [], [], []
    for coordsys, L, bnds, pairs in [(2, 0.0, bs, pairs_s), (1, 600.0, bb, pairs_b)]:
        for a, b in pairs:
            v = R.ref_signal_pair(coordsys, L, bnds[a].copy(), bnds[b].copy(), 0, 0.0, 0.0, n1, n2, X,
                                  tabs[0].copy(), 1e-5, 1e-10, C.byref(err))
            vals.append(v)
            errs.append(err.value)
            c1s.append(bnds[a])
            c2s.append(bnds[b])
            kinds.append(coordsys)
    out["pair_coordsys"] = np.array(kinds, dtype=np.int32)
    out["pair_c1"], out["pair_c2"] = np.array(c1s), np.array(c2s)
    out["pair_val"], out["pair_err"] = np.array(vals), np.array(errs)

    # testsig.cpp:41-66: whole-box cell, periodic box L = 10, sigma = 1/sqrt(2)
    L = 10.0
    sigma = 1 / np.sqrt(2)
    A = (2 * np.pi * sigma ** 2) ** -1.5
    b = 1 / (2 * sigma ** 2)
    c = np.array([0, L, 0, L, 0, L], dtype=np.float64)
    out["gauss_box_L"], out["gauss_box_A"], out["gauss_box_b"] = L, A, b
    out["gauss_box_Q"] = R.ref_signal_pair(1, L, c, c.copy(), 2, A, b, n1, n2, X, tabs[0].copy(), 1e-5, 1e-12,
                                           C.byref(err))

    # whole signal-matrix blocks
    for name, (sv, cells) in {"box": synth.box_survey(4, side=200.0, scale=100.0),
                              "sph": synth.shell_survey(3, 4, 6)}.items():
        n = cells.size
        S = np.zeros((n, n))
        idx = np.arange(n, dtype=np.int32)
        R.ref_signal_block(sv.coordsys, np.array(sv.bounds, dtype=np.float64), np.array(sv.n, dtype=np.int32),
                           sv.L, n, cells.ctypes.data, n, idx, n, idx, S, n, n1, n2, X, tabs[0].copy(), 1e-5, 1e-10)
        out[f"block_{name}_cells"] = cells
        out[f"block_{name}_bounds"] = np.array(sv.bounds)
        out[f"block_{name}_n"] = np.array(sv.n, dtype=np.int32)
        out[f"block_{name}_L"] = sv.L
        out[f"block_{name}_S"] = S

    # a cellfile written by the reference's ABN writer (basis.cpp:195-201 header)
    sv, cells = synth.shell_survey(3, 4, 6)
    path = os.path.join(HERE, "cells_ref.abn")
    assert R.ref_write_cells(path.encode(), sv.coordsys, np.array(sv.bounds, dtype=np.float64),
                             np.array(sv.n, dtype=np.int32), sv.L, cells.size, cells.ctypes.data) == 0
    out["cells_ref"] = cells

    np.savez_compressed(os.path.join(HERE, "reference_vectors.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_vectors.npz"))


if __name__ == "__main__":
    main()
