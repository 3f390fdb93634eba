"""Repeated builds in one context: the batched block eigensolve is captured into
a CUDA graph on the second build with the same shapes and buffers and replayed
from the third on.  Each build must equal a fresh context's build of the same
survey, so a replay that kept anything from the capture's data would show."""
import numpy as np
import pytest

from opsec_gpu import api, synth

PK = synth.pk_table()


@pytest.mark.gpu
def test_repeated_builds_match_fresh_contexts():
    bands = synth.band_edges(12, 0.0, 0.2)
    # same 8 x 8 x 16 full-sky grid, different radial selections and counts
    surveys = [synth.shell_survey(8, 8, 16, rc=rc, width=wd, nquad=8)
               for rc, wd in ((600.0, 250.0), (450.0, 150.0), (800.0, 300.0), (600.0, 250.0))]
    rng = np.random.default_rng(7)
    counts = [rng.poisson(cells["Nbar"]).astype(float) for _, cells in surveys]
    nmodes = 256
    e = api.Engine(api.make_config(surveys[0][0], bands=bands))
    e.set_pk(*PK)
    got = [e.fisher_build(cells, cnt, nmodes) for (_, cells), cnt in zip(surveys, counts)]
    e.close()
    for k, ((sv, cells), cnt) in enumerate(zip(surveys, counts)):
        s = api.Engine(api.make_config(sv, bands=bands))
        s.set_pk(*PK)
        ref = s.fisher_build(cells, cnt, nmodes)
        s.close()
        # shared-memory atomics may sum in another order between runs: 1e-6, far below what a
        # replay of another survey's data would change
        assert np.max(np.abs(got[k]["evals"] - ref["evals"])) <= 1e-6 * ref["evals"][0], k
        sc = np.max(np.abs(ref["F"]))
        assert np.max(np.abs(got[k]["F"] - ref["F"])) <= 1e-6 * sc, k
        sig = np.sqrt(np.diag(ref["pcov"]))
        assert np.max(np.abs(got[k]["phat"] - ref["phat"]) / sig) <= 1e-4, k
    # the four surveys differ by far more than the tolerance
    assert np.max(np.abs(got[0]["F"] - got[1]["F"])) > 1e-3 * np.max(np.abs(got[0]["F"]))
