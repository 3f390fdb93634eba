"""The benchmark's headline configuration at full size against the FP64 oracle: the
32 x 32 x 32 full-sky shell on r in [200, 1000] (32,768 cells), 40 bands on [0, 0.4],
8,192 modes, 4096 log-spaced xi points beyond r = 10, 4^3 x 4^3 Gauss rule -- the
workload `python bench.py` times.

1. S at 256 cell pairs (random ones plus self and neighbouring pairs, seed 3), tables 0,
   20 and 40, against the oracle's Gauss rule on the same pairs (sig.cpp:125-213).
2. The whole build (klt.cpp:173-248, comma-scalapack.cpp:228-252, estimate-mpi.cpp:480-641)
   against the oracle's FP64 restatement in the grid's azimuthal basis
   (oracle.fisher_azimuthal, itself equal to the dense oracle on small shells), fed with the
   GPU's S rows: eigenvalues, F, f, q, the estimates, and the kept mode subspace.
"""
import numpy as np
import pytest

from opsec_gpu import api, synth
import oracle as O
from fullsize import LAYOUT, check_full_build, check_pairs, pair_sample

PK = synth.pk_table()
pytestmark = pytest.mark.gpu


def test_c2_signal_pairs_and_full_build():
    sv, cells = synth.shell_survey(32, 32, 32)
    nbands, nmodes = 40, 8192
    bands = synth.band_edges(nbands, 0.0, 0.4)
    e = api.Engine(api.make_config(sv, bands=bands, nmodes=nmodes, layout=LAYOUT, gauss=4))
    e.set_pk(*PK)
    tabs = O.xi_tables(*PK, bands, LAYOUT)
    rows, cols = pair_sample(cells, 32, 32)
    check_pairs(e, cells, rows, cols, tabs, [0, 20, 40])
    counts = synth.grf_counts(sv, cells)
    err = check_full_build(e, sv, cells, nbands, nmodes, counts)
    e.close()
    assert err["evals"] <= 1e-12 and err["klt evals"] <= 1e-12, err
    assert err["mode sin"] <= 1e-6, err
    for k in ("F", "f", "q", "phat", "pcov/cond"):
        assert err[k] <= 1e-6, (k, err)
