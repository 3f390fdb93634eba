"""Failure handling without a GPU fault.  The reference stops the whole job on any error
(opsec_abort / MPI_Abort, opsec.c:88-116); the engine returns a status from every call and keeps
the context usable.  Two host-side and device-side forms are exercised here:

- a failed device allocation, injected on the host (opsec_gpu_fail_alloc): the call that meets
  it returns OPSEC_ERR_NOMEM, and the context's next call rebuilds what it needs and gives the
  same result as a fresh context;
- the bounded mbarrier wait of the tensor-core projection kernels, on a barrier that nothing
  completes (opsec_gpu_wait_probe): the kernel gives up after the limit, the host reads the
  timeout, and the context goes on (a projection right after matches the oracle).
"""
import numpy as np
import pytest

import oracle as O
from opsec_gpu import api, synth

PK = synth.pk_table()


def test_injection_and_probe_arguments_are_checked_without_a_device():
    L = api.load()
    assert L.opsec_gpu_fail_alloc(None, 0) == api.ERR_ARG
    assert L.opsec_gpu_wait_probe(None, 1000, 0, 0, None) == api.ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("warm", [False, True])
@pytest.mark.parametrize("after", [0, 2, 5])
def test_failed_allocation_leaves_the_context_usable(after, warm):
    sv, cells = synth.shell_survey(3, 4, 8)
    bands = synth.band_edges(4, 0.0, 0.2)
    counts = synth.grf_counts(sv, cells)
    cfg = api.make_config(sv, bands=bands)
    with api.Engine(cfg) as fresh:
        fresh.set_pk(*PK)
        ref = fresh.fisher_build(cells, counts, 40)
    e = api.Engine(cfg)
    e.set_pk(*PK)
    if warm:  # some buffers exist already; the build allocates the rest
        e.klt(cells, 20)
    e.fail_alloc(after)
    with pytest.raises(api.OpsecError) as ex:
        e.fisher_build(cells, counts, 40)
    assert ex.value.code == api.ERR_NOMEM and "injected" in str(ex.value)
    e.fail_alloc(-1)
    got = e.fisher_build(cells, counts, 40)
    e.close()
    assert np.max(np.abs(got["F"] - ref["F"])) <= 1e-12 * np.max(np.abs(ref["F"]))


@pytest.mark.gpu
def test_bounded_wait_gives_up_and_the_context_goes_on():
    sv, cells = synth.box_survey(4, side=200.0, scale=100.0)
    bands = synth.band_edges(3, 0.0, 0.15)
    e = api.Engine(api.make_config(sv, bands=bands, extra=["projection = tc"]))
    e.set_pk(*PK)
    assert e.wait_probe(2000, arrive=False) is True          # nothing arrives: gives up
    assert e.wait_probe(200_000_000, arrive=True, delay_cycles=20_000) is False  # arrives in time
    assert e.wait_probe(5000, arrive=False) is True
    tabs = O.xi_tables(*PK, bands)
    Q = O.qtable_keys(sv, O.keys_all(sv), tabs)
    S = O.signal_matrix(sv, cells, Q[:, 0])
    _, modes = O.klt(S, 16)
    cov = e.comma(cells, modes)
    e.close()
    for p in range(len(bands)):
        ref = O.project(modes, O.signal_matrix(sv, cells, Q[:, 1 + p]))
        assert np.max(np.abs(cov[p] - ref)) <= 1e-5 * np.max(np.abs(ref))
