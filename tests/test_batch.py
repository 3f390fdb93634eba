"""Batched mocks (opsec_gpu_batch_fisher): every mock's Fisher matrix, p-hat and
covariance against the same mock built alone through opsec_gpu_fisher_build.
Tolerance 1e-6 of max|F| (the window cubature's FP32 shared-memory atomics may
add in a different order from one build to the next)."""
import numpy as np
import pytest

from opsec_gpu import api, synth

pytestmark = pytest.mark.gpu

PK = synth.pk_table()


@pytest.mark.parametrize("workers", [1, 3, 0])
def test_batch_matches_single_builds(workers):
    mocks = synth.mock_batch(5, seed=11, ncells_range=(2000, 4000))
    bands = synth.band_edges(20, 0.0, 0.2)
    e = api.Engine(api.make_config(mocks[0]["survey"], bands=bands))
    e.set_pk(*PK)
    out = e.batch_fisher(mocks, workers=workers)
    e.close()
    if workers > 0:
        assert out["workers"] == workers
    else:
        assert out["workers"] in (1, 2, 4, 8, 12, 16)
    for i, m in enumerate(mocks):
        s = api.Engine(api.make_config(m["survey"], bands=bands))
        s.set_pk(*PK)
        ref = s.fisher_build(m["cells"], m["counts"], m["nmodes"])
        s.close()
        sc = np.max(np.abs(ref["F"]))
        assert np.max(np.abs(out["F"][i] - ref["F"])) <= 1e-6 * sc, i
        sig = np.sqrt(np.diag(ref["pcov"]))
        assert np.max(np.abs(out["phat"][i] - ref["phat"]) / sig) <= 1e-4, i


def test_batch_rejects_bad_mock():
    mocks = synth.mock_batch(2, seed=3, ncells_range=(2000, 2500))
    mocks[1]["nr"] += 1  # grid no longer matches the cells
    e = api.Engine(api.make_config(mocks[0]["survey"], bands=synth.band_edges(4, 0.0, 0.2)))
    e.set_pk(*PK)
    with pytest.raises(api.OpsecError):
        e.batch_fisher(mocks, workers=2)
    e.close()


def test_batch_mocks_against_the_oracle():
    """Three batched mocks (8 x 16 x 16 shells with their own radial selections) end to end
    against the dense FP64 oracle: eigensolve, projection, Fisher matrix and estimates of each
    mock (mode counts moved to a spectral gap near Ncells / 4)."""
    import oracle as O

    mocks = synth.mock_batch(3, seed=21, ncells_range=(1000, 1500))
    bands = synth.band_edges(20, 0.0, 0.2)
    refs = []
    for m in mocks:
        sv, cells = m["survey"], m["cells"]
        tabs = O.xi_tables(*PK, bands)
        Q = O.qtable_keys(sv, O.keys_all(sv, fold=True), tabs[:1])
        lam = np.sort(np.linalg.eigvalsh(O.signal_matrix(sv, cells, Q[:, 0], fold=True)))[::-1]
        m["nmodes"] = O.gap_nmodes(lam, cells.size // 4, rel_gap=1e-4, span=64)
        refs.append(O.fisher_build(sv, cells, m["counts"], *PK, bands, m["nmodes"], fold=True))
    e = api.Engine(api.make_config(mocks[0]["survey"], bands=bands))
    e.set_pk(*PK)
    out = e.batch_fisher(mocks, workers=2)
    e.close()
    for i, ref in enumerate(refs):
        F = ref["est"]["F"]
        err = np.max(np.abs(out["F"][i] - F)) / np.max(np.abs(F))
        sig = np.sqrt(np.diag(ref["est"]["pcov"]))
        dp = np.max(np.abs(out["phat"][i] - ref["est"]["phat"]) / sig)
        print(f"mock {i}: {mocks[i]['cells'].size} cells, {mocks[i]['nmodes']} modes: F {err:.2e}, p-hat {dp:.2e} sigma")
        assert err <= 1e-6 and dp <= 1e-4, (i, err, dp)
