"""The 65,536-cell configuration (64 x 32 x 32 full-sky shell on r in [200, 1000], 64 bands on
[0, 0.4], 16,384 modes) at full size:

1. S at 256 cell pairs (random ones plus self and neighbouring pairs) against the oracle's
   Gauss rule on the same pairs (sig.cpp:125-213).
2. C_p at 256 random cells (seed 3, all 32,896 pairs among them) through `opsec_gpu_comma`,
   i.e. the fused tensor-core projection that gathers S_p tiles from the key tables and never
   stores an N x N band matrix (comma-scalapack.cpp:228-265), with modes that pick one cell
   each: against the oracle's FP64 Gauss rule on those pairs, and against the finite
   difference [S(p + e_n eps) - S(p - e_n eps)] / 2 eps of the signal matrix with respect to
   the band power p_n, S(p) built from the xi table sum_n p_n xi_n.
3. The whole build against the oracle's FP64 restatement in the azimuthal basis
   (oracle.fisher_azimuthal), fed with the GPU's S rows: eigenvalues, F, f, q, estimates.
4. The same configuration downsampled to 8 x 8 x 16 = 1,024 cells (64 bands on [0, 0.4],
   modes = cells / 4 as at full size), end to end against the dense FP64 oracle.
"""
import numpy as np
import pytest

from opsec_gpu import api, synth
import oracle as O
from fullsize import LAYOUT, check_full_build, check_pairs, pair_sample

PK = synth.pk_table()
pytestmark = pytest.mark.gpu


def engine(sv, nbands, nmodes):
    bands = synth.band_edges(nbands, 0.0, 0.4)
    e = api.Engine(api.make_config(sv, bands=bands, nmodes=nmodes, layout=LAYOUT, gauss=4))
    e.set_pk(*PK)
    return e, bands


def test_c3_signal_pairs_projection_and_full_build():
    sv, cells = synth.shell_survey(64, 32, 32)
    nbands, nmodes = 64, 16384
    e, bands = engine(sv, nbands, nmodes)
    tabs = O.xi_tables(*PK, bands, LAYOUT)
    rows, cols = pair_sample(cells, 32, 32)
    check_pairs(e, cells, rows, cols, tabs, [0, 32, 64])

    # C_p at 256 random cells through the fused projection
    sel = np.sort(np.random.default_rng(3).choice(cells.size, 256, replace=False)).astype(np.int32)
    B = np.zeros((sel.size, cells.size))
    B[np.arange(sel.size), sel] = 1.0
    cov = e.comma(cells, B)                       # [64][256 * 257 / 2], packed upper triangle
    i, j = O.packed_ij(sel.size)
    a, b = sel[i], sel[j]
    ch = [0, 21, 42, 63]
    Qp = O.q_pairs(2, 0.0, O.cell_bounds(cells[a]), O.cell_bounds(cells[b]), tabs[[1 + n for n in ch]], LAYOUT)
    nb = np.sqrt(cells["Nbar"][a] * cells["Nbar"][b])
    err_oracle = {n: float(np.max(np.abs(cov[n] - nb * Qp[:, k])) / np.max(np.abs(nb * Qp[:, k])))
                  for k, n in enumerate(ch)}
    p = e.get_params()
    r, xi = e.xi_tables()
    base = np.tensordot(p, xi[1:], axes=(0, 0))
    err_fd = {}
    for n in ch:
        eps = np.max(p)  # S is linear in the band powers: any step; a small one loses digits
        e.set_xi_table(0, base + eps * xi[1 + n])
        sp = e.signal_block(cells, sel, sel, table=0)
        e.set_xi_table(0, base - eps * xi[1 + n])
        sm = e.signal_block(cells, sel, sel, table=0)
        fd = ((sp - sm) / (2 * eps))[i, j]
        err_fd[n] = float(np.max(np.abs(cov[n] - fd)) / np.max(np.abs(fd)))
    e.set_pk(*PK)                                 # back to the model's own tables
    print("C_p at 256 random cells: vs oracle", err_oracle, "vs finite differences", err_fd)
    assert max(err_oracle.values()) <= 1e-6, err_oracle
    assert max(err_fd.values()) <= 1e-5, err_fd

    counts = synth.grf_counts(sv, cells)
    err = check_full_build(e, sv, cells, nbands, nmodes, counts, check_modes=False)
    e.close()
    assert err["evals"] <= 1e-12, err
    for k in ("F", "f", "q", "phat", "pcov/cond"):
        assert err[k] <= 1e-6, (k, err)


def test_c3_downsampled_against_dense_oracle():
    sv, cells = synth.shell_survey(8, 8, 16)
    nbands = 64
    bands = synth.band_edges(nbands, 0.0, 0.4)
    tabs = O.xi_tables(*PK, bands, LAYOUT)
    Q = O.qtable_keys(sv, O.keys_all(sv), tabs[:1], LAYOUT)
    lam = np.sort(np.linalg.eigvalsh(O.signal_matrix(sv, cells, Q[:, 0])))[::-1]
    M = O.gap_nmodes(lam, cells.size // 4, rel_gap=1e-4, span=64)
    counts = synth.grf_counts(sv, cells)
    ref = O.fisher_build(sv, cells, counts, *PK, bands, M, layout=LAYOUT)
    e, _ = engine(sv, nbands, M)
    got = e.fisher_build(cells, counts, M)
    e.close()
    F = ref["est"]["F"]
    rel = {"evals": float(np.max(np.abs(got["evals"] - ref["evals"])) / ref["evals"][0]),
           "F": float(np.max(np.abs(got["F"] - F)) / np.max(np.abs(F)))}
    print(f"1,024 cells, 64 bands, {M} modes, end to end:", rel)
    assert rel["evals"] <= 1e-6 and rel["F"] <= 1e-6, rel
