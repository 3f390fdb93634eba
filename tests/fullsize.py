"""Checks shared by the full-size tests of full-sky shells: S at sampled cell pairs against
the oracle's Gauss rule, and a whole Fisher build against the oracle's FP64 restatement in the
azimuthal basis (oracle.fisher_azimuthal)."""
import numpy as np

import oracle as O

LAYOUT = (256, 4096, 10.0, 20000.0)  # 256 linear xi points on [0, 10), 4096 log-spaced to 20,000


def pair_sample(cells, nphi, nmu, n=16, seed=3):
    rng = np.random.default_rng(seed)
    rows = rng.choice(cells.size, n, replace=False).astype(np.int32)
    a = int(rows[0])
    near = [a, a + 1, a - 1, a + nphi, a - nphi, a + nphi * nmu, a - nphi * nmu]
    cols = np.array(near + list(rng.choice(cells.size, n - len(near), replace=False)), dtype=np.int32)
    return rows, np.clip(cols, 0, cells.size - 1).astype(np.int32)


def check_pairs(e, cells, rows, cols, tabs, sel, tol=3e-7):
    c1 = O.cell_bounds(cells[np.repeat(rows, cols.size)])
    c2 = O.cell_bounds(cells[np.tile(cols, rows.size)])
    Q = O.q_pairs(2, 0.0, c1, c2, tabs[sel], LAYOUT)
    nb = np.sqrt(cells["Nbar"][np.repeat(rows, cols.size)] * cells["Nbar"][np.tile(cols, rows.size)])
    errs = {}
    for j, t in enumerate(sel):
        got = e.signal_block(cells, rows, cols, table=t).ravel()
        ref = nb * Q[:, j]
        errs[t] = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
    print("S at sampled pairs, error / max|S| per table:", errs)
    assert max(errs.values()) <= tol, errs


def check_full_build(e, sv, cells, nbands, nmodes, counts, check_modes=True):
    """Returns the measured relative errors of the whole build against the FP64 restatement."""
    nr, nmu, nphi = sv.n
    H = nr * nmu
    out = e.fisher_build(cells, counts, nmodes)
    arc_rows = (np.arange(H) * nphi).astype(np.int32)
    x = (counts - cells["Nbar"]) / np.sqrt(cells["Nbar"])
    prior = e.get_params()
    ref = O.fisher_azimuthal(lambda t: e.signal_block(cells, arc_rows, None, table=t), nphi, nbands, nmodes, x,
                             prior)
    lam = ref["evals"]
    err = {"evals": float(np.max(np.abs(out["evals"] - lam)) / lam[0])}
    q_gpu = out["q"] + out["f"]  # the estfile's q record is q - f (estimate-mpi.cpp:603)
    err["F"] = float(np.max(np.abs(out["F"] - ref["F"])) / np.max(np.abs(ref["F"])))
    qf = max(np.max(np.abs(ref["q"])), np.max(np.abs(ref["f"])))
    err["f"] = float(np.max(np.abs(out["f"] - ref["f"])) / qf)
    err["q"] = float(np.max(np.abs(q_gpu - ref["q"])) / qf)
    est = O.estimate_epilogue(ref["F"], ref["q"], ref["f"])
    phat_scale = np.max(np.abs(est["M"]) @ (np.abs(ref["q"]) + np.abs(ref["f"])))
    err["phat"] = float(np.max(np.abs(out["phat"] - est["phat"])) / phat_scale)
    err["pcov/cond"] = float(np.max(np.abs(out["pcov"] - est["pcov"])) / np.max(np.abs(est["pcov"]))
                             / np.linalg.cond(ref["F"]))
    if check_modes:
        ev, modes = e.klt(cells, nmodes)
        pick = np.unique(np.concatenate([np.arange(64), np.arange(nmodes - 64, nmodes),
                                         np.random.default_rng(3).choice(nmodes, 128, replace=False)]))
        nrm = O.mode_projection_norms(modes[pick], ref["groups"], H, nphi)
        err["mode sin"] = float(np.sqrt(max(0.0, np.max(1.0 - nrm))))
        err["klt evals"] = float(np.max(np.abs(ev - lam)) / lam[0])
        del modes
    gap = None if ref["next_eval"] is None else (lam[nmodes - 1] - ref["next_eval"]) / lam[0]
    print(f"{cells.size} cells, {nbands} bands, {nmodes} modes: relative gap at the cut {gap}; errors {err}")
    return err
