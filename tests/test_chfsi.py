"""The iterative eigensolver (klt.solver = chfsi: Chebyshev-filtered subspace iteration on
the resident signal matrix, the GPU counterpart of the reference's ARPACK Lanczos,
ParpackSolver.cpp:111-123) against the dense FP64 eigensolve of the same matrix, on
Cartesian grids: eigenvalues, modes and the Fisher matrix built on them."""
import numpy as np
import pytest

from opsec_gpu import api, synth

pytestmark = pytest.mark.gpu
BANDS = synth.band_edges(6, 0.0, 0.12)


def _box(n, side, periodic, tilt=True):
    if tilt:
        return synth.tilted_box_survey(n, side, periodic=periodic)
    sv = synth.Survey(synth.COORD_CARTESIAN, (0.0, side, 0.0, side, 0.0, side), (n, n, n),
                      L=side if periodic else 0.0)

    def sel(x, y, z):  # centred and isotropic: the grid's symmetries make eigenvalues degenerate
        return 3e-4 * np.exp(-((x - side / 2) ** 2 + (y - side / 2) ** 2 + (z - side / 2) ** 2) / (side / 2) ** 2)

    return sv, synth.make_cells(sv, sel, nquad=4)


def _pair(sv, nmodes, extra=()):
    mk = lambda solver: api.Engine(api.make_config(sv, bands=BANDS, nmodes=nmodes,
                                                   extra=(f"klt.solver = {solver}",) + tuple(extra)))
    d, c = mk("dense"), mk("chfsi")
    k, P = synth.pk_table()
    d.set_pk(k, P)
    c.set_pk(k, P)
    return d, c


def _at_gap(ev, m, rel=1e-3):
    """The largest m' <= m with a relative gap of at least rel below mode m'."""
    while m > 1 and ev[m - 1] - ev[m] <= rel * ev[m - 1]:
        m -= 1
    return m


def _compare(d, c, cells, nmodes, ev_tol=1e-9):
    evd, Bd = d.klt(cells, nmodes + 1)
    assert d.eig_stats()["solver"] == "dense"
    m = _at_gap(evd, nmodes)
    evc, Bc = c.klt(cells, m)
    st = c.eig_stats()
    # the refinement takes the FP64 residuals to a tenth of klt.tol (1e-5, ARPACK's in the reference)
    assert st["solver"] == "chfsi" and st["resid"] <= 1e-6 and st["iterations"] >= 1, st
    np.testing.assert_allclose(evc, evd[:m], rtol=ev_tol, atol=0)
    # modes: the top-m subspaces agree, and so do the modes of separated eigenvalues
    P = Bd[:m] @ Bc.T
    sv = np.linalg.svd(P, compute_uv=False)
    assert sv.min() >= 1 - 1e-8, sv.min()
    gap = np.minimum(np.r_[np.inf, -np.diff(evd[:m + 1])][:m], -np.diff(evd[:m + 1]))
    sep = gap > 1e-3 * evd[:m]
    ov = np.abs(np.sum(Bd[:m] * Bc, axis=1))
    assert np.all(ov[sep] >= 1 - 1e-8), ov[sep].min()
    # the sign convention: the entry of largest magnitude is positive
    big = np.argmax(np.abs(Bc), axis=1)
    assert np.all(Bc[np.arange(m), big] > 0)
    return m, st


def test_chfsi_open_box_matches_dense():
    sv, cells = _box(12, 600.0, periodic=False)
    d, c = _pair(sv, 200)
    m, st = _compare(d, c, cells, 200)
    # the Fisher build on either eigensolve
    counts = synth.grf_counts(sv, cells)
    rd = d.fisher_build(cells, counts, m)
    rc = c.fisher_build(cells, counts, m)
    assert c.eig_stats()["solver"] == "chfsi"
    np.testing.assert_allclose(rc["F"], rd["F"], rtol=1e-6, atol=1e-6 * np.abs(rd["F"]).max())
    # the iterative modes meet the reference's ARPACK criterion, relative residual <= 1e-5
    # (ParpackSolver.cpp:111-123), not FP64 rounding: q and f, quadratic in the data projected
    # on the modes, agree to a few 1e-5 of their scale, and p = F^-1 (q - f) to 1e-4 of its own
    for k in ("q", "f"):
        np.testing.assert_allclose(rc[k], rd[k], rtol=0, atol=5e-5 * np.abs(rd[k]).max())
    np.testing.assert_allclose(rc["phat"], rd["phat"], rtol=0, atol=1e-4 * np.abs(rd["phat"]).max())
    d.close()
    c.close()


def test_chfsi_periodic_box_eigenvalues():
    """The benchmark box (12^3 periodic cells, 500 modes): its cubic symmetry makes many
    eigenvalues degenerate, so eigenvalues and the top subspace are compared."""
    sv, cells = _box(12, 600.0, periodic=True, tilt=False)
    d, c = _pair(sv, 500)
    _compare(d, c, cells, 500, ev_tol=1e-8)
    d.close()
    c.close()


def test_chfsi_larger_grid_and_fp32_simt():
    sv, cells = _box(20, 800.0, periodic=False)
    d, c = _pair(sv, 400)
    _compare(d, c, cells, 400)
    c.close()
    _, c2 = _pair(sv, 400, extra=("klt.gemm = f32", "klt.degree = 6"))
    m = _at_gap(d.klt(cells, 401)[0], 400)
    ev2, _ = c2.klt(cells, m)
    np.testing.assert_allclose(ev2, d.klt(cells, m)[0], rtol=1e-9)
    assert c2.eig_stats()["degree"] <= 6
    d.close()
    c2.close()


def test_chfsi_rejects_bad_options():
    sv, _ = _box(4, 100.0, periodic=False)
    for bad in ("klt.solver = lanczos", "klt.degree = 0", "klt.tol = -1", "klt.gemm = tf32"):
        with pytest.raises(api.OpsecError):
            api.Engine(api.make_config(sv, bands=BANDS, extra=(bad,)))


def test_block_product_tensor_cores():
    """The eigensolver's block product C = alpha S X + beta C + gamma D on the tcgen05 kernel
    against FP64 numpy: ragged N (K padding) and column counts (partial 256-column tiles),
    rows and columns of S spread over 2^+-8 (FP16 scaling and subnormal low parts).  The
    split keeps ~22 bits of each operand and the FP32 running sums round once per 64 of K,
    so the error is a few 1e-7 of sum_k |alpha S_ik X_kj| + |beta C| + |gamma D|."""
    sv, _ = _box(4, 100.0, periodic=False)
    rng = np.random.default_rng(5)
    for N, nc, tile in ((333, 37, "auto"), (1024, 300, "256"), (1500, 640, "128"), (1500, 640, "256")):
        e = api.Engine(api.make_config(sv, bands=BANDS, extra=(f"klt.tile = {tile}",)))
        A = rng.standard_normal((N, N))
        w = np.exp2(rng.uniform(-8, 8, N))
        S = (A + A.T) * w[:, None] * w[None, :]
        X = rng.standard_normal((N, nc)).astype(np.float32)
        C0 = rng.standard_normal((N, nc)).astype(np.float32)
        D = rng.standard_normal((N, nc)).astype(np.float32)
        for alpha, beta, gamma in ((1.0, 0.0, 0.0), (0.75, -0.5, 0.25)):
            out = e.block_product(S, X, alpha, beta, C0, gamma, D if gamma else None)
            X64 = X.astype(np.float64)
            ref = alpha * (S @ X64) + beta * C0 + gamma * D
            bound = abs(alpha) * (np.abs(S) @ np.abs(X64)) + abs(beta) * np.abs(C0) + abs(gamma) * np.abs(D)
            rel = np.abs(out - ref) / bound
            print(f"N {N} ncols {nc} tile {tile} beta {beta}: max {rel.max():.2e}, median {np.median(rel):.2e}")
            assert rel.max() <= 2e-6 and np.median(rel) <= 2e-7, (N, nc, rel.max(), np.median(rel))
        e.close()


def test_chfsi_cublas_route_matches_dense():
    """klt.gemm = bf16x9, klt.fp64 = native, klt.qr = householder: the products with S through
    cuBLAS (BF16x9 and DGEMM) and the refinement's QR by cuSOLVER's Householder, instead of the
    engine's tcgen05 and double-FP32 kernels and CholeskyQR2."""
    sv, cells = _box(12, 600.0, periodic=False)
    d, c = _pair(sv, 200, extra=("klt.gemm = bf16x9", "klt.fp64 = native", "klt.qr = householder"))
    _compare(d, c, cells, 200)
    d.close()
    c.close()
