"""GPU results against the FP64 oracle, through the C ABI.

Tolerances (stated per quantity):
  xi tables (FP64 Simpson on the GPU)            1e-12 relative to max |xi|
  signal matrix (FP32 cubature, FP64 totals)      5e-7 relative to max |S|
  signal matrix, top band tables, exact / fast    3e-7 / 5e-5 relative to max |S|
  KL eigenvalues                                  1e-6 relative to lambda_0
  KL modes (cut at a spectral gap)                sin(largest principal angle) <= 1e-4
  packed C_p (projection)                         1e-5 relative to max |C_p|
  Fisher matrix and estimates, end to end         1e-6 relative (the plain-form target)
"""
import math

import numpy as np
import pytest

import oracle as O
from cases import cases
from opsec_gpu import api, synth

pytestmark = pytest.mark.gpu

PK = synth.pk_table()
CASES = cases()


def engine(sv, nb=3, kmax=0.15, layout=None, nmodes=None, gauss=None, mixing=None):
    bands = synth.band_edges(nb, 0.0, kmax)
    e = api.Engine(api.make_config(sv, bands=bands, nmodes=nmodes, layout=layout, gauss=gauss, mixing=mixing))
    e.set_pk(*PK)
    return e, bands


@pytest.mark.parametrize("layout", [O.LAYOUT_REFERENCE, O.LAYOUT_LOG4096])
def test_xi_tables(layout):
    sv, _ = CASES["box4"]
    e, bands = engine(sv, nb=4, layout=layout)
    r, xi = e.xi_tables()
    X, _ = O.r_grid(layout)
    np.testing.assert_array_equal(r, X)
    ref = O.xi_tables(*PK, bands, layout)
    for t in range(ref.shape[0]):
        assert np.max(np.abs(xi[t] - ref[t])) <= 1e-12 * np.max(np.abs(ref[t]))
    np.testing.assert_allclose(e.get_params(), O.band_priors(*PK, bands), rtol=1e-14)
    e.close()


@pytest.mark.parametrize("name", list(CASES))
def test_signal_matrix(name):
    sv, cells = CASES[name]
    e, bands = engine(sv)
    tabs = O.xi_tables(*PK, bands)
    Q = O.qtable_keys(sv, O.keys_all(sv), tabs)
    for t in range(tabs.shape[0]):
        ref = O.signal_matrix(sv, cells, Q[:, t])
        got = e.signal_block(cells, table=t)
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err <= 5e-7, (name, t, err)
    # non-contiguous rows/cols and an lld larger than ncols (sig.h:16-20)
    rows = np.array([cells.size - 1, 0, 2], dtype=np.int32)
    cols = np.array([1, cells.size - 2], dtype=np.int32)
    blk = e.signal_block(cells, rows, cols, table=1, lld=5)
    ref = O.signal_matrix(sv, cells, Q[:, 1])[np.ix_(rows, cols)]
    assert np.max(np.abs(blk - ref)) <= 5e-7 * np.max(np.abs(ref))
    e.close()


HIGH_K = {
    # 12^3 periodic box of side 600, 20 bands on [0, 0.2], 4096 log-spaced xi points
    "box1728": (lambda: synth.box_survey(12), 20, 0.2),
    # 4 x 4 x 8 full-sky shell r in [200, 1000], 40 bands on [0, 0.4]
    "shell128": (lambda: synth.shell_survey(4, 4, 8), 40, 0.4),
}


@pytest.mark.parametrize("precision,tol", [("exact", 3e-7), ("fast", 5e-5)])
@pytest.mark.parametrize("name", list(HIGH_K))
def test_signal_matrix_high_k(name, precision, tol):
    """Band tables at the top of the k range oscillate with period 2 pi / k,
    so the rounding of a pair separation r enters as a phase error k dr.
    Exact mode forms r^2 and the table index from FP32 pairs (error left:
    the FP32 tables); fast mode rounds r to FP32 (error ~ k r 6e-8)."""
    make, nb, kmax = HIGH_K[name]
    sv, cells = make()
    bands = synth.band_edges(nb, 0.0, kmax)
    layout = O.LAYOUT_LOG4096
    e = api.Engine(api.make_config(sv, bands=bands, layout=layout, extra=[f"cubature.precision = {precision}"]))
    e.set_pk(*PK)
    tabs = O.xi_tables(*PK, bands, layout)
    sel = [0, nb // 2, nb - 1, nb]
    Q = O.qtable_keys(sv, O.keys_all(sv), tabs[sel], layout)
    errs = []
    for j, t in enumerate(sel):
        ref = O.signal_matrix(sv, cells, Q[:, j])
        got = e.signal_block(cells, table=t)
        errs.append(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
    print(f"{name} {precision}: max|dS|/max|S| for tables {sel}: " + " ".join(f"{x:.2e}" for x in errs))
    assert max(errs) <= tol, (name, precision, errs)
    e.close()


@pytest.mark.parametrize("name", ["shell768", "box12"])
def test_cubature_window_path(name):
    """Exact-mode far keys go through per-key bin-window histograms (one pass
    over the point pairs for all tables); near keys through the table-group
    kernel.  Both paths against the oracle and against each other."""
    if name == "shell768":
        sv, cells = synth.shell_survey(6, 8, 16)
        bands = synth.band_edges(20, 0.0, 0.4)
    else:
        sv, cells = synth.box_survey(12)
        bands = synth.band_edges(20, 0.0, 0.2)
    layout = O.LAYOUT_LOG4096
    got = {}
    for win in ("1", "0"):
        e = api.Engine(api.make_config(sv, bands=bands, layout=layout, extra=[f"cubature.window = {win}"]))
        e.set_pk(*PK)
        got[win] = [e.signal_block(cells, table=t) for t in (0, 10, 20)]
        e.close()
    tabs = O.xi_tables(*PK, bands, layout)
    Q = O.qtable_keys(sv, O.keys_all(sv), tabs[[0, 10, 20]], layout)
    for j, t in enumerate((0, 10, 20)):
        ref = O.signal_matrix(sv, cells, Q[:, j])
        sc = np.max(np.abs(ref))
        e_win = np.max(np.abs(got["1"][j] - ref)) / sc
        e_grp = np.max(np.abs(got["0"][j] - ref)) / sc
        print(f"{name} table {t}: window {e_win:.2e}, groups {e_grp:.2e}")
        assert e_win <= 3e-7 and e_grp <= 3e-7, (name, t, e_win, e_grp)


def test_cubature_window_variants_are_bitwise_equal():
    """The spherical window kernel's loop for one-pass keys above the linear section of the
    table (exponent table, floor by a rounded-down addition, no linear branch or pass filter)
    performs the general loop's operations and roundings, and every key is integrated by one
    warp whatever order the keys are taken in: the signal matrix is the same bits with the
    loop on and off and with the far keys in key order and in window-start order, on a shell
    whose far keys take the loop and whose self and neighbour keys (windows reaching below
    r1 = 10) do not."""
    sv, cells = synth.shell_survey(8, 8, 16)
    bands = synth.band_edges(20, 0.0, 0.4)
    got = {}
    for opts in (("1", "key"), ("0", "key"), ("1", "window")):
        e = api.Engine(api.make_config(sv, bands=bands, layout=O.LAYOUT_LOG4096,
                                       extra=[f"cubature.log_keys = {opts[0]}", f"cubature.order = {opts[1]}"]))
        e.set_pk(*PK)
        got[opts] = [e.signal_block(cells, table=t) for t in (0, 10, 20)]
        e.close()
    for opts in (("0", "key"), ("1", "window")):
        for j in range(3):
            assert np.array_equal(got[("1", "key")][j], got[opts][j]), (opts, j)


@pytest.mark.parametrize("gauss", [2, 3, 5])
@pytest.mark.parametrize("name", ["shell", "box"])
def test_cubature_window_gauss_orders(name, gauss):
    """The window kernels at Gauss orders other than 4: their lane maps (node pairs per lane,
    canonical mirror pairs, 2^k fixed-point scale) change with the order.  A wrong pair or
    weight would show at 1e-3 or more.  The 4^3 box has cells of 150 Mpc/h: a self pair spans
    separations 0-260 across several periods of the band tables, whose strong cancellation lifts
    the FP32-table floor to ~1e-6 of max|S| (the table-group kernel: 8e-7 at order 5)."""
    if name == "shell":
        sv, cells = synth.shell_survey(4, 4, 8)
        bands = synth.band_edges(10, 0.0, 0.4)
    else:
        sv, cells = synth.box_survey(4)
        bands = synth.band_edges(10, 0.0, 0.2)
    layout = O.LAYOUT_LOG4096
    e = api.Engine(api.make_config(sv, bands=bands, layout=layout, gauss=gauss))
    e.set_pk(*PK)
    got = [e.signal_block(cells, table=t) for t in (0, 5, 10)]
    e.close()
    tabs = O.xi_tables(*PK, bands, layout)
    Q = O.qtable_keys(sv, O.keys_all(sv), tabs[[0, 5, 10]], layout, ng=gauss)
    for j, t in enumerate((0, 5, 10)):
        ref = O.signal_matrix(sv, cells, Q[:, j])
        err = np.max(np.abs(got[j] - ref)) / np.max(np.abs(ref))
        assert err <= (3e-7 if name == "shell" else 2.5e-6), (name, gauss, t, err)


def test_cubature_precision_key_is_checked():
    sv, _ = CASES["box4"]
    with pytest.raises(api.OpsecError):
        api.Engine(api.make_config(sv, bands=synth.band_edges(2, 0.0, 0.1), extra=["cubature.precision = double"]))


def test_known_answers_on_gpu():
    """xi = 1 gives Q = 1 (testsig.cpp:19-39); a tabulated Gaussian xi in a
    periodic box matches the oracle's Gauss rule on the same table."""
    sv, cells = CASES["box4"]
    e, _ = engine(sv, nb=1)
    n = O.r_grid(O.LAYOUT_REFERENCE)[0].size
    e.set_xi_table(0, np.ones(n))
    S = e.signal_block(cells, table=0)
    ref = np.sqrt(cells["Nbar"][:, None] * cells["Nbar"][None, :])
    assert np.max(np.abs(S / ref - 1.0)) < 2e-6
    e.close()
    # whole-box cell of side L = 10 on a fine table (testsig.cpp:41-66 geometry)
    L = 10.0
    sv = synth.Survey(synth.COORD_CARTESIAN, (0, L, 0, L, 0, L), (1, 1, 1), L=L)
    cell = synth.make_cells(sv, lambda x, y, z: np.ones_like(x), nquad=4)
    layout = (2000, 64, 20.0, 100.0)
    e, _ = engine(sv, nb=1, layout=layout, gauss=6)
    X, _ = O.r_grid(layout)
    sigma = 1 / math.sqrt(2)
    A, b = (2 * math.pi * sigma ** 2) ** -1.5, 1 / (2 * sigma ** 2)
    Y = A * np.exp(-b * X ** 2)
    e.set_xi_table(0, Y)
    got = e.signal_block(cell, table=0)[0, 0] / cell["Nbar"][0]
    ref = O.qtable_keys(sv, np.zeros((1, 3), np.int32), Y[None, :], layout, ng=6)[0, 0]
    assert abs(got - ref) <= 2e-6 * abs(ref)
    # the rule itself: 6 points per axis cannot resolve sigma = 0.7 in a cell of
    # side 10 (the oracle converges to the analytic value only as the order grows)
    exact = math.erf(L / (2 * math.sqrt(2) * sigma)) ** 3 / L ** 3
    assert 0.5 < abs(ref - exact) / exact < 1.0
    e.close()


def _oracle_modes(sv, cells, bands, target):
    tabs = O.xi_tables(*PK, bands)
    Q = O.qtable_keys(sv, O.keys_all(sv), tabs)
    S = O.signal_matrix(sv, cells, Q[:, 0])
    lam = np.sort(np.linalg.eigvalsh(S))[::-1]
    M = O.gap_nmodes(lam, target)
    ev, modes = O.klt(S, M)
    return tabs, Q, M, ev, modes


@pytest.mark.parametrize("name", list(CASES))
def test_klt(name):
    sv, cells = CASES[name]
    e, bands = engine(sv)
    tabs, Q, M, ev, modes = _oracle_modes(sv, cells, bands, cells.size // 2)
    gev, gmodes = e.klt(cells, M)
    assert np.max(np.abs(gev - ev)) <= 1e-6 * ev[0]
    np.testing.assert_allclose(gmodes @ gmodes.T, np.eye(M), atol=1e-10)
    assert O.subspace_sin(gmodes, modes) <= 1e-4
    e.close()


@pytest.mark.parametrize("name", list(CASES))
def test_comma_and_dot(name):
    sv, cells = CASES[name]
    e, bands = engine(sv)
    tabs, Q, M, ev, modes = _oracle_modes(sv, cells, bands, cells.size // 2)
    cov = e.comma(cells, modes)
    for p in range(len(bands)):
        ref = O.project(modes, O.signal_matrix(sv, cells, Q[:, 1 + p]))
        assert np.max(np.abs(cov[p] - ref)) <= 1e-5 * np.max(np.abs(ref)), (name, p)
    counts = synth.grf_counts(sv, cells)
    y = e.dot(cells, counts, modes)
    np.testing.assert_allclose(y, O.dot(cells, counts, modes), rtol=1e-12, atol=1e-12 * np.max(np.abs(y)))
    e.close()


@pytest.mark.parametrize("mixing", ["inverse", "inverse-sqrt", "identity"])
def test_estimate(mixing):
    rng = np.random.default_rng(7)
    sv, cells = CASES["sph_full"]
    e, bands = engine(sv, nb=4)
    M = 30
    evals = np.sort(rng.uniform(0.05, 4.0, M))[::-1]
    Dp = np.stack([O.pack_upper((lambda A: A @ A.T / M)(rng.standard_normal((M, M)))) for _ in bands])
    y = rng.standard_normal(M)
    got = e.estimate(evals, Dp, y, mixing)
    F, f, q = O.fisher(evals, Dp, y, O.band_priors(*PK, bands))
    ref = O.estimate_epilogue(F, q, f, mixing)
    for k in ("F", "phat", "pcov", "W", "M", "q", "f"):
        scale = np.max(np.abs(ref[k]))
        assert np.max(np.abs(got[k] - ref[k])) <= 1e-6 * scale, (k, mixing)
    e.close()


@pytest.mark.parametrize("name", list(CASES))
def test_fisher_build_end_to_end(name):
    """(1) With the oracle's modes, the GPU projection + Fisher + epilogue meet
    1e-6.  (2) With the GPU's own FP64 eigensolve of its FP32-cubature S, the
    kept subspace moves by ~|dS|/gap; at a cut whose gap exceeds 1e-4 lambda_0
    the whole path also meets 1e-6 (measured at most 4.4e-7)."""
    sv, cells = CASES[name]
    e, bands = engine(sv)
    tabs, Q, _, _, _ = _oracle_modes(sv, cells, bands, cells.size // 2)
    S = O.signal_matrix(sv, cells, Q[:, 0])
    lam = np.sort(np.linalg.eigvalsh(S))[::-1]
    M = O.gap_nmodes(lam, cells.size // 2, rel_gap=1e-4, span=cells.size // 4)
    counts = synth.grf_counts(sv, cells)
    ref = O.fisher_build(sv, cells, counts, *PK, bands, M)
    # (1) identical modes
    cov = e.comma(cells, ref["modes"])
    y = e.dot(cells, counts, ref["modes"])
    got = e.estimate(ref["evals"], cov, y)
    got["evals"] = ref["evals"]
    check_estimates(got, ref, name + "/oracle-modes", tol=1e-6)
    # (2) the whole path on the GPU
    got = e.fisher_build(cells, counts, M)
    check_estimates(got, ref, name + "/end-to-end", tol=1e-6)
    assert e.launch_count() > 0
    e.close()


def test_fisher_build_azimuthal_projection():
    """Full-sky shell, 8 x 8 x 16 = 1024 cells, 10 bands: the build projects
    onto its own azimuthal modes block by block (the block GEMMs on the H x H
    cosine transforms of each band: 3-term TF32 on the tensor cores, the
    default, FP32 and FP64 by cuBLAS).  Against the dense tensor-core projection
    of the same modes (projection = tc) and against the oracle end to end."""
    sv, cells = synth.shell_survey(8, 8, 16)
    bands = synth.band_edges(10, 0.0, 0.2)
    counts = synth.grf_counts(sv, cells)
    tabs = O.xi_tables(*PK, bands)
    Q = O.qtable_keys(sv, O.keys_all(sv), tabs)
    S = O.signal_matrix(sv, cells, Q[:, 0])
    lam = np.sort(np.linalg.eigvalsh(S))[::-1]
    M = O.gap_nmodes(lam, 256, rel_gap=1e-4, span=64)
    out = {}
    for name, extra in (("aztc", ["azimuthal.gemm = tc"]), ("az32", ["azimuthal.gemm = f32"]),
                        ("az64", ["azimuthal.gemm = f64"]), ("tc", ["projection = tc"]),
                        ("simt", ["projection = simt"])):
        e = api.Engine(api.make_config(sv, bands=bands, extra=extra))
        e.set_pk(*PK)
        out[name] = e.fisher_build(cells, counts, M)
        e.close()
    scale = np.max(np.abs(out["simt"]["F"]))
    d = {k: np.max(np.abs(out[k]["F"] - out["az64"]["F"])) / scale for k in ("aztc", "az32", "tc", "simt")}
    print("F against the FP64 azimuthal projection: " + ", ".join(f"{k} {v:.2e}" for k, v in d.items()))
    assert max(d.values()) <= 1e-6, d
    ref = O.fisher_build(sv, cells, counts, *PK, bands, M)
    for k in ("aztc", "az32", "az64"):
        rel = np.max(np.abs(out[k]["F"] - ref["est"]["F"])) / np.max(np.abs(ref["est"]["F"]))
        print(f"{k}: end-to-end Fisher rel err {rel:.2e}")
        check_estimates(out[k], ref, f"shell1024/{k}/end-to-end", tol=1e-6)


def test_azimuthal_transform_tiles_are_bitwise_the_rows():
    """The FP32 band blocks by staged 16 x 32 tiles (upper triangle, mirrored) perform the
    per-output kernel's operations on the same key values: the Fisher matrix is the same bits
    with either, on a shell with both mu parities and several radial shells per tile."""
    sv, cells = synth.shell_survey(8, 8, 16)
    bands = synth.band_edges(6, 0.0, 0.2)
    counts = synth.grf_counts(sv, cells)
    out = {}
    for tr in ("tiled", "rows"):
        e = api.Engine(api.make_config(sv, bands=bands, extra=[f"azimuthal.transform = {tr}"]))
        e.set_pk(*PK)
        out[tr] = e.fisher_build(cells, counts, 200)
        e.close()
    assert np.array_equal(out["tiled"]["F"], out["rows"]["F"])
    assert np.array_equal(out["tiled"]["q"], out["rows"]["q"])


def test_band_blocks_overlapped_with_the_eigensolve_are_bitwise_equal():
    """The FP32 band blocks transformed on their own stream during the eigensolve
    (azimuthal.overlap = 1, the default) against the same transforms after it: the same bits,
    on two shells and over repeated builds in one context (the band stream's buffers and events
    are reused)."""
    sv, cells = synth.shell_survey(8, 8, 16)
    sv2, cells2 = synth.shell_survey(6, 8, 16)
    bands = synth.band_edges(6, 0.0, 0.2)
    counts = synth.grf_counts(sv, cells)
    counts2 = synth.grf_counts(sv2, cells2)
    out = {}
    for ov in (0, 1):
        e = api.Engine(api.make_config(sv, bands=bands, extra=[f"azimuthal.overlap = {ov}"]))
        e.set_pk(*PK)
        out[ov] = [e.fisher_build(cells, counts, 200)]
        e.close()
        e = api.Engine(api.make_config(sv2, bands=bands, extra=[f"azimuthal.overlap = {ov}"]))
        e.set_pk(*PK)
        out[ov].append(e.fisher_build(cells2, counts2, 150))
        out[ov].append(e.fisher_build(cells2, counts2, 150))
        e.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a["F"], b["F"]) and np.array_equal(a["q"], b["q"])
    assert np.array_equal(out[1][1]["F"], out[1][2]["F"])


def test_reflection_symmetry_paths_agree():
    """Full-sky shell with a mu range symmetric about 0: the cubature integrates
    one key of each (h_a, h_b) <-> (P h_a, P h_b) reflection pair and the
    azimuthal eigensolve splits every order into mu-even and mu-odd blocks.
    Against the same build with both symmetries switched off."""
    sv, cells = synth.shell_survey(6, 8, 16)
    bands = synth.band_edges(6, 0.0, 0.2)
    counts = synth.grf_counts(sv, cells)
    tabs = O.xi_tables(*PK, bands)
    Q = O.qtable_keys(sv, O.keys_all(sv), tabs[:1])
    lam = np.sort(np.linalg.eigvalsh(O.signal_matrix(sv, cells, Q[:, 0])))[::-1]
    M = O.gap_nmodes(lam, 200, rel_gap=1e-4, span=64)
    out = {}
    for name, extra in (("sym", []), ("plain", ["cubature.symmetry = none", "azimuthal.parity = 0"])):
        e = api.Engine(api.make_config(sv, bands=bands, extra=extra))
        e.set_pk(*PK)
        out[name] = (e.fisher_build(cells, counts, M), e.signal_block(cells, table=3))
        e.close()
    (a, Sa), (b, Sb) = out["sym"], out["plain"]
    # the two cubatures of a reflected pair agree to the exact-mode index precision, not bitwise
    assert np.max(np.abs(Sa - Sb)) <= 2e-7 * np.max(np.abs(Sb))
    assert np.max(np.abs(a["evals"] - b["evals"])) <= 1e-7 * b["evals"][0]
    assert np.max(np.abs(a["F"] - b["F"])) <= 1e-6 * np.max(np.abs(b["F"]))


def check_estimates(got, ref, name, tol=1e-6):
    """F, f and q within tol of their scale; p-hat and Cov within tol of the
    scale their own inputs propagate (p-hat = M (q - f) cancels q against f,
    and Cov ~ F^-1 amplifies by cond(F)), i.e. backward error <= tol.
    Prints and returns the measured errors in those units."""
    est = ref["est"]
    F = est["F"]
    qf_scale = max(np.max(np.abs(ref["q"])), np.max(np.abs(ref["f"])))
    Mx = est["M"]
    phat_scale = np.max(np.abs(Mx) @ (np.abs(ref["q"]) + np.abs(ref["f"])))
    cond = np.linalg.cond(F)
    err = {"evals": np.max(np.abs(got["evals"] - ref["evals"])) / ref["evals"][0],
           "F": np.max(np.abs(got["F"] - F)) / np.max(np.abs(F)),
           "f": np.max(np.abs(got["f"] - est["f"])) / qf_scale,
           "q": np.max(np.abs((got["q"] + got["f"]) - ref["q"])) / qf_scale,
           "phat": np.max(np.abs(got["phat"] - est["phat"])) / phat_scale,
           "pcov": np.max(np.abs(got["pcov"] - est["pcov"])) / (cond * np.max(np.abs(est["pcov"])))}
    err = {k: float(v) for k, v in err.items()}
    print(f"{name}: " + ", ".join(f"{k} {v:.2e}" for k, v in err.items()))
    for k, v in err.items():
        assert v <= tol, (name, k, v, tol)
    return err


def test_fisher_build_box_1728_cells():
    """The benchmark's CPU-runnable configuration: 12^3 periodic box,
    n = 3e-4 exp(-(r/300)^2), 20 bands on [0, 0.2], 4^3 x 4^3 Gauss rule,
    4096 log-spaced xi points, 500 modes (moved to a spectral gap).  The
    projection + Fisher + epilogue on the oracle's modes meet 1e-6, and so does
    the whole GPU path at a cut in a spectral gap (measured 4.8e-7 in F)."""
    sv, cells = synth.box_survey(12)
    bands = synth.band_edges(20, 0.0, 0.2)
    layout = O.LAYOUT_LOG4096
    tabs = O.xi_tables(*PK, bands, layout)
    Q = O.qtable_keys(sv, O.keys_all(sv), tabs, layout)
    S = O.signal_matrix(sv, cells, Q[:, 0])
    lam = np.sort(np.linalg.eigvalsh(S))[::-1]
    M = O.gap_nmodes(lam, 500, rel_gap=1e-4, span=64)
    counts = synth.grf_counts(sv, cells)
    e = api.Engine(api.make_config(sv, bands=bands, layout=layout))
    e.set_pk(*PK)
    ref = O.fisher_build(sv, cells, counts, *PK, bands, M, layout=layout)
    cov = e.comma(cells, ref["modes"])
    y = e.dot(cells, counts, ref["modes"])
    got = e.estimate(ref["evals"], cov, y)
    got["evals"] = ref["evals"]
    check_estimates(got, ref, "box1728/oracle-modes", tol=1e-6)
    got = e.fisher_build(cells, counts, M)
    rel_F = np.max(np.abs(got["F"] - ref["est"]["F"])) / np.max(np.abs(ref["est"]["F"]))
    gap = (lam[M - 1] - lam[M]) / lam[0]
    print(f"box1728: M={M} relative gap {gap:.2e}, end-to-end Fisher rel err {rel_F:.3e}")
    check_estimates(got, ref, "box1728/end-to-end", tol=1e-6)
    e.close()


@pytest.mark.parametrize("dims", [(8, 8, 16), (16, 16, 32), (6, 10, 12)])
def test_block_eigensolver_matches_library(dims):
    """The hand-written block eigensolver (azimuthal.eig = own: Householder tridiagonalisation,
    bisection, twisted-factorisation eigenvectors, back-transformation) against cuSOLVER's
    batched syevd on the same blocks: eigenvalues to 1e-12 of lambda_0, the kept modes' span
    to 1e-8 at a cut with a gap of 1e-5 lambda_0, and the Fisher matrix to 1e-9."""
    sv, cells = synth.shell_survey(*dims)
    bands = synth.band_edges(6, 0.0, 0.3)
    counts = synth.grf_counts(sv, cells)
    e = api.Engine(api.make_config(sv, bands=bands, extra=["azimuthal.eig = batched"]))
    e.set_pk(*PK)
    lam, _ = e.klt(cells, cells.size // 4 + 64)
    e.close()
    M = O.gap_nmodes(lam, cells.size // 4, rel_gap=1e-5, span=63)
    out = {}
    for eig in ("own", "batched"):
        e = api.Engine(api.make_config(sv, bands=bands, extra=[f"azimuthal.eig = {eig}"]))
        e.set_pk(*PK)
        ev, modes = e.klt(cells, M)
        st = e.eig_stats()
        F = e.fisher_build(cells, counts, M)["F"]
        out[eig] = (ev, modes, F, st)
        e.close()
    (ev, B, F, st), (ev0, B0, F0, _) = out["own"], out["batched"]
    assert st["solver"] == "azimuthal" and st["iterations"] == 1, st
    d_ev = np.max(np.abs(ev - ev0)) / ev0[0]
    # each own mode's distance from the library's kept span (no 1 - cos^2 cancellation)
    sin = float(np.max(np.linalg.norm(B - (B @ B0.T) @ B0, axis=1)))
    d_F = np.max(np.abs(F - F0)) / np.max(np.abs(F0))
    print(f"{dims}: {st['block']} eigenvectors computed for {M} modes; eigenvalues {d_ev:.2e}, "
          f"span sin {sin:.2e}, F {d_F:.2e}")
    assert d_ev <= 1e-12 and sin <= 1e-8 and d_F <= 1e-9, (d_ev, sin, d_F)


@pytest.mark.parametrize("dims", [(4, 4, 16), (3, 4, 32), (2, 2, 64)])
def test_projection_arc_tables(dims):
    """The tensor-core projection's arc-run gather (cells in arc order, 16, 32 or 64 phi cells
    per arc: each K-slice's tile expanded from the runs of the square key table it spans)
    against the general per-element gather: bit for bit, and both against the oracle."""
    sv, cells = synth.shell_survey(*dims)
    bands = synth.band_edges(3, 0.0, 0.3)
    tabs = O.xi_tables(*PK, bands)
    Q = O.qtable_keys(sv, O.keys_all(sv), tabs)
    _, modes = O.klt(O.signal_matrix(sv, cells, Q[:, 0]), 40)
    out = {}
    for arcs in ("1", "0"):
        e = api.Engine(api.make_config(sv, bands=bands, extra=["projection = tc", f"projection.arc_tables = {arcs}"]))
        e.set_pk(*PK)
        out[arcs] = e.comma(cells, modes)
        e.close()
    np.testing.assert_array_equal(out["1"], out["0"])
    for p in range(len(bands)):
        ref = O.project(modes, O.signal_matrix(sv, cells, Q[:, 1 + p]))
        assert np.max(np.abs(out["1"][p] - ref)) <= 1e-5 * np.max(np.abs(ref)), p
