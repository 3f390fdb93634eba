"""The cell builder: HEALPix pixels and cell Nbar against the reference's own
chealpix.c / FinalizeCell (tests/golden/basis_ref.npz, made by
tests/golden/make_basis_golden.py) and against the numpy restatement
(oracle/basis.py)."""
import os

import numpy as np
import pytest

from opsec_gpu import api, synth
import basis as B

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "basis_ref.npz"))
NSIDES = (1, 2, 4, 16, 256, 8192)


def test_ang2pix_restatement_matches_reference():
    for ns in NSIDES:
        for nest, name in ((0, "ring"), (1, "nest")):
            got = B.ang2pix(ns, nest, G["hp_theta"], G["hp_phi"])
            assert np.array_equal(got, G[f"hp_{name}_{ns}"]), (ns, name)


def test_basis_restatement_matches_reference():
    rad = (G["rad_r"], G["rad_n"])
    box = B.basis(1, G["box_grid"], G["box_n"], nbar=float(G["box_nbar"][0]))
    assert np.allclose(box, G["box_out"][:, :2], rtol=1e-14, atol=0)
    # no map: the reference's adaptive cubature (epsrel 1e-5) against the closed-form radial integral,
    # and its Nbar is 3x the expected count (quirk 3)
    sph = B.basis(2, G["sph_grid"], G["sph_n"], rad=rad, quirk3=True)
    assert np.max(np.abs(sph[:, 0] - G["sph_out"][:, 0]) / G["sph_out"][:, 0]) <= 1e-14
    assert np.max(np.abs(sph[:, 1] - G["sph_out"][:, 1])) <= 1e-6 * np.max(G["sph_out"][:, 1])
    plain = B.basis(2, G["sph_grid"], G["sph_n"], rad=rad)
    assert np.allclose(3 * plain[:, 1], sph[:, 1], rtol=1e-14)
    # with a map the sampled mean converges (64^2 against 256^2 points per cell) ...
    for nest in (0, 1):
        a = B.basis(2, G["map_grid"], G["map_n"], rad=rad, nside=2, nest=nest, mask=G["map"], samples=64, quirk3=True)
        b = B.basis(2, G["map_grid"], G["map_n"], rad=rad, nside=2, nest=nest, mask=G["map"], samples=256, quirk3=True)
        assert np.max(np.abs(a[:, 1] - b[:, 1])) <= 1e-4 * np.max(b[:, 1])
        ref = G["map_nest_out" if nest else "map_ring_out"][:, 1]
        diff = np.abs(b[:, 1] - ref) / np.max(ref)
        # ... while the reference's adaptive cubature, whose error estimate a piecewise-constant map can
        # fool, agrees to 2e-3 on the RING map and on 18 of 24 cells of the NESTED one (its six
        # equatorial cells are off by up to 7 %: nested pixels there are not resolved by its rule)
        if nest:
            assert np.sum(diff > 2e-3) <= 6
        else:
            assert np.max(diff) <= 2e-3


def _engine(sv, extra=()):
    cfg = api.make_config(sv, bands=synth.band_edges(2, 0.0, 0.2), extra=extra)
    e = api.Engine(cfg)
    e.set_pk(*synth.pk_table())
    return e


@pytest.mark.gpu
def test_gpu_ang2pix_matches_reference():
    sv, _ = synth.box_survey(2)
    e = _engine(sv)
    for ns in NSIDES:
        for nest, name in ((0, "ring"), (1, "nest")):
            got = e.ang2pix(ns, nest, G["hp_theta"], G["hp_phi"])
            assert np.array_equal(got, G[f"hp_{name}_{ns}"]), (ns, name)
    e.close()


@pytest.mark.gpu
def test_gpu_basis_matches_reference_and_oracle():
    rad = (G["rad_r"], G["rad_n"])
    # Cartesian constant selection
    g, n = G["box_grid"], G["box_n"]
    sv = synth.Survey(1, g, n, L=0.0)
    e = _engine(sv, extra=(f"survey.nbar = {float(G['box_nbar'][0])!r}",))
    cells = e.basis()
    e.close()
    assert cells.size == np.prod(n)
    assert np.array_equal(cells["a"], np.arange(cells.size))
    assert np.allclose(cells["Veff"], G["box_out"][:, 0], rtol=1e-14)
    assert np.allclose(cells["Nbar"], G["box_out"][:, 1], rtol=1e-14)
    # spherical, radial spline only: reference (quirk 3 on) and 1/3 of it by default
    for quirk in (1, 0):
        sv = synth.Survey(2, G["sph_grid"], G["sph_n"])
        e = _engine(sv, extra=(f"basis.quirk3 = {quirk}",))
        e.set_radial(*rad)
        cells = e.basis()
        e.close()
        ref = G["sph_out"][:, 1] / (1 if quirk else 3)
        assert np.max(np.abs(cells["Nbar"] - ref)) <= 1e-6 * np.max(ref)
        assert np.allclose(cells["Veff"], G["sph_out"][:, 0], rtol=1e-14)
        mine = B.basis(2, G["sph_grid"], G["sph_n"], rad=rad, quirk3=bool(quirk))
        assert np.allclose(cells["Nbar"], mine[:, 1], rtol=1e-12)
    # spherical with maps: the numpy restatement's sampling, cell for cell; empty cells dropped
    mask = np.array(G["map"], dtype=np.float32)
    for nest in (0, 1):
        sv = synth.Survey(2, G["map_grid"], G["map_n"])
        e = _engine(sv, extra=("basis.samples = 32",))
        e.set_radial(*rad)
        e.set_mask(2, nest, mask)
        cells = e.basis()
        e.close()
        mine = B.basis(2, G["map_grid"], G["map_n"], rad=rad, nside=2, nest=nest, mask=mask, samples=32)
        keep = mine[:, 1] > 0
        assert cells.size == int(np.sum(keep))
        assert np.allclose(cells["Nbar"], mine[keep, 1], rtol=1e-12)


@pytest.mark.gpu
def test_new_entry_points_reject_bad_arguments():
    """Invalid sizes and states return errors (no fault, no partial output)."""
    sv = synth.Survey(2, G["sph_grid"], G["sph_n"])
    e = _engine(sv)
    with pytest.raises(api.OpsecError):
        e.basis()                      # no radial selection yet
    with pytest.raises(api.OpsecError):
        e.set_radial([1.0], [2.0])     # one point
    with pytest.raises(api.OpsecError):
        e.set_radial([2.0, 1.0], [1.0, 1.0])  # decreasing abscissae
    with pytest.raises(api.OpsecError):
        e.set_mask(3, True, np.ones(12 * 9, dtype=np.float32))  # NESTED needs a power of two
    with pytest.raises(api.OpsecError):
        e.ang2pix(0, 0, [0.1], [0.2])
    e.set_radial(*(G["rad_r"], G["rad_n"]))
    cells = e.basis()
    assert cells.size == int(np.prod(G["sph_n"]))
    with pytest.raises(api.OpsecError):
        e.mock_counts(cells, ngrid=33)  # odd mesh
    with pytest.raises(api.OpsecError):
        e.mock_counts(cells, ngrid=2)
    # a negative bias beyond -1/delta clips lambda at zero: counts stay non-negative integers
    c = e.mock_counts(cells, ngrid=16, seed=3, bias=-50.0)
    assert np.all(c >= 0) and np.all(c == np.floor(c))
    e.close()
