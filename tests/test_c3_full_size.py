"""The 65,536-cell configuration at full size: S at 256 cell pairs (random ones
plus self and neighbouring pairs) against the oracle's Gauss rule on the same
pairs, and a whole Fisher build (no packed triangle: it would be 34 GB)."""
import numpy as np
import pytest

from opsec_gpu import api, synth
import oracle as O

PK = synth.pk_table()
pytestmark = pytest.mark.gpu


def test_c3_signal_pairs_and_fisher_build():
    sv, cells = synth.shell_survey(64, 32, 32)
    bands = synth.band_edges(64, 0.0, 0.4)
    layout = (256, 4096, 10.0, 20000.0)
    e = api.Engine(api.make_config(sv, bands=bands, layout=layout))
    e.set_pk(*PK)
    rng = np.random.default_rng(3)
    # 16 x 16 pairs: random cells, one of them repeated in the columns with its neighbours
    rows = rng.choice(cells.size, 16, replace=False).astype(np.int32)
    a = int(rows[0])
    near = [a, a + 1, a - 1, a + 32, a - 32, a + 1024, a - 1024]
    cols = np.array(near + list(rng.choice(cells.size, 16 - len(near), replace=False)), dtype=np.int32)
    cols = np.clip(cols, 0, cells.size - 1).astype(np.int32)
    tabs = O.xi_tables(*PK, bands, layout)
    sel = [0, 32, 64]
    c1 = O.cell_bounds(cells[np.repeat(rows, cols.size)])
    c2 = O.cell_bounds(cells[np.tile(cols, rows.size)])
    Q = O.q_pairs(2, 0.0, c1, c2, tabs[sel], layout)
    nb = np.sqrt(cells["Nbar"][np.repeat(rows, cols.size)] * cells["Nbar"][np.tile(cols, rows.size)])
    for j, t in enumerate(sel):
        got = e.signal_block(cells, rows, cols, table=t).ravel()
        ref = nb * Q[:, j]
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err <= 3e-7, (t, err)
    counts = rng.poisson(cells["Nbar"]).astype(float)
    out = e.fisher_build(cells, counts, 16384)
    e.close()
    F = out["F"]
    assert np.all(np.isfinite(F)) and np.all(np.diag(F) > 0)
    assert np.max(np.abs(F - F.T)) <= 1e-12 * np.max(np.abs(F))
    assert np.all(np.linalg.eigvalsh(F) > 0)
    assert out["evals"][0] >= out["evals"][-1] > 0
