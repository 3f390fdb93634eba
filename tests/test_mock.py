"""Mock counts: the GPU's Gaussian random field and Poisson draws against the
numpy restatement with the same Philox streams (oracle/mock_grf.py), which is
itself pinned to numpy's Philox4x64-10."""
import math

import numpy as np
import pytest

from opsec_gpu import api, synth
import mock_grf as M
import oracle as O

PK = synth.pk_table()


def test_philox_matches_numpy():
    for key in [(0, 0), (12345, 678), (2 ** 63 + 5, 3)]:
        for ctr in [(0, 0, 0, 0), (7, 0, 0, 0), (2 ** 64 - 2, 5, 9, 1)]:
            ref = np.random.Philox(counter=np.array(ctr, dtype=np.uint64), key=np.array(key, dtype=np.uint64))
            ref = ref.random_raw(4)
            c = list(ctr)  # numpy advances the counter before its first block
            c[0] = (c[0] + 1) % 2 ** 64
            if c[0] == 0:
                c[1] += 1
            got = M.philox4x64(*[np.array([x], dtype=np.uint64) for x in c], *key)
            assert [int(g[0]) for g in got] == [int(r) for r in ref], (key, ctr)


def test_poisson_sampler_statistics():
    """Both branches (inversion below 10, PTRS above) have the Poisson mean and variance."""
    for lam in (0.7, 4.0, 9.5, 10.5, 37.0, 400.0):
        x = np.array([M.poisson(lam, a, 99) for a in range(4000)], dtype=float)
        assert abs(x.mean() - lam) < 5 * math.sqrt(lam / x.size), lam
        assert abs(x.var() / lam - 1.0) < 0.12, lam


def test_white_noise_is_standard_normal():
    g = M.white_noise(32, 5).ravel()
    assert abs(g.mean()) < 5 / math.sqrt(g.size)
    assert abs(g.std() - 1.0) < 0.01


@pytest.mark.gpu
@pytest.mark.parametrize("geom", ["box", "shell"])
def test_mock_counts_match_oracle(geom):
    if geom == "box":
        sv, cells = synth.box_survey(12)
        coordsys, n = 1, 32
    else:
        sv, cells = synth.shell_survey(8, 8, 16, nquad=8)
        coordsys, n = 2, 48
    bands = synth.band_edges(4, 0.0, 0.2)
    e = api.Engine(api.make_config(sv, bands=bands))
    e.set_pk(*PK)
    counts, delta = e.mock_counts(cells, ngrid=n, seed=17, bias=1.3, want_delta=True)
    again = e.mock_counts(cells, ngrid=n, seed=17, bias=1.3)
    other = e.mock_counts(cells, ngrid=n, seed=18, bias=1.3)
    e.close()
    spl = O.CubicSpline(*PK)
    ref_counts, ref_delta = M.mock_counts(coordsys, cells, n, 17, 1.3, spl)
    assert np.max(np.abs(delta - ref_delta)) <= 1e-10 * np.max(np.abs(ref_delta))
    assert np.array_equal(counts, ref_counts)
    assert np.array_equal(again, counts)          # deterministic in the seed
    assert not np.array_equal(other, counts)      # and a different seed differs
    # the field's variance follows the spectrum: sum over the mesh modes of P(k) / V
    idx, box = M.mesh_index(coordsys, cells, n)
    kf = 2 * math.pi / box
    f = np.fft.fftfreq(n, d=1.0 / n)
    kk = kf * np.sqrt(f[:, None, None] ** 2 + f[None, :, None] ** 2 + f[None, None, :] ** 2).ravel()
    var = np.sum(np.asarray(spl(kk[1:]))) / box ** 3
    fld = M.field(n, box, 17, spl)
    assert abs(fld.var() / var - 1.0) < 0.1
    lam = np.fmax(cells["Nbar"] * (1 + 1.3 * delta), 0)
    assert abs(counts.sum() - lam.sum()) < 6 * math.sqrt(lam.sum())
