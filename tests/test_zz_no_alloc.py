"""opsec_gpu_fisher_noalloc against the allocating estimate entry point.

The no-allocation entry point exists for callers that cannot call cudaMalloc
-- code whose device memory is all owned by its own pool allocator, or a
latency-critical loop where an allocation could synchronize the device.  The
test owns every device buffer (allocated here with torch); the entry point
only launches kernels into them and its file-scope scratch array.  Two calls
in a row must both match the allocating path (opsec_gpu_estimate), within the
1e-6 relative tolerance of the other Fisher tests.

This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from opsec_gpu import api, synth

pytestmark = pytest.mark.gpu


def _dev_ptr(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("nb", [1, 6, 64])
def test_fisher_noalloc_matches_allocating_path(nb):
    """nb = 64 is the limit: the largest shared-memory request and partial stride."""
    import torch

    torch.cuda.init()
    L = api.load()
    L.opsec_gpu_fisher_noalloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(3)
    M = 96
    K = M * (M + 1) // 2
    evals = np.ascontiguousarray(np.sort(rng.uniform(0.05, 4.0, M))[::-1])
    cov32 = np.stack([O.pack_upper((lambda A: A @ A.T / M)(rng.standard_normal((M, M)))) for _ in range(nb)]).astype(
        np.float32)
    y = rng.standard_normal(M)

    sv, _ = synth.shell_survey(3, 4, 8)
    eng = api.Engine(api.make_config(sv, bands=synth.band_edges(nb, 0.0, 0.3)))
    eng.set_pk(*synth.pk_table())
    prior = eng.get_params()
    ref = eng.estimate(evals, cov32.astype(np.float64), y)
    eng.close()
    F_ref, f_ref = ref["F"], ref["f"]
    q_ref = ref["q"] + ref["f"]  # the estimate record holds q - f

    dev = torch.device("cuda:0")
    d_cov = torch.from_numpy(cov32.ravel()).to(dev)
    d_ev = torch.from_numpy(evals).to(dev)
    d_y = torch.from_numpy(y).to(dev)
    d_pr = torch.from_numpy(prior).to(dev)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        d_out = torch.full((nb * nb + 2 * nb,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = L.opsec_gpu_fisher_noalloc(M, nb, _dev_ptr(d_cov), _dev_ptr(d_ev), _dev_ptr(d_y), _dev_ptr(d_pr),
                                        _dev_ptr(d_out), C.c_void_p(stream.cuda_stream))
        assert rc == 0, rc
        torch.cuda.synchronize()
        out = d_out.cpu().numpy()
        F, f, q = out[: nb * nb].reshape(nb, nb), out[nb * nb: nb * nb + nb], out[nb * nb + nb:]
        assert np.max(np.abs(F - F_ref)) <= 1e-6 * np.max(np.abs(F_ref)), call
        scale = max(np.max(np.abs(q_ref)), np.max(np.abs(f_ref)))
        assert np.max(np.abs(f - f_ref)) <= 1e-6 * scale, call
        assert np.max(np.abs(q - q_ref)) <= 1e-6 * scale, call


def test_fisher_noalloc_rejects_too_many_bands():
    L = api.load()
    L.opsec_gpu_fisher_noalloc.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    one = C.c_void_p(1)
    assert L.opsec_gpu_fisher_noalloc(8, 65, one, one, one, one, one, None) == -2
