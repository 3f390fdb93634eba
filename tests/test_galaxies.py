"""Galaxy counts per cell (the dot program's binning, code/opsec/src/dot.cpp:105-129):
the numpy restatement (oracle/basis.py) against the reference's own GetGridIndex and
counting loop (tests/golden/galaxy_ref.npz, made by tests/golden/make_galaxy_golden.py),
and the GPU binning against the restatement."""
import os
import subprocess

import numpy as np
import pytest

from opsec_gpu import api, formats, synth
import basis as B

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "galaxy_ref.npz"))
CASES = (("box", synth.COORD_CARTESIAN), ("sph", synth.COORD_SPHERICAL))


def _cells(n, cellidx):
    cells = np.zeros(len(cellidx), dtype=synth.CELL_DTYPE)
    cells["a"] = np.arange(len(cellidx))
    cells["d1"] = cellidx // (n[1] * n[2])
    cells["d2"] = (cellidx // n[2]) % n[1]
    cells["d3"] = cellidx % n[2]
    return cells


def test_grid_index_and_counts_restatement_match_reference():
    for p, _ in CASES:
        e = B.grid_index(G[p + "_grid"], G[p + "_n"], G[p + "_gals"])
        assert np.array_equal(e, G[p + "_index"]), p
        # the reference's counting, galaxies of grid index 0 sent to no cell, to the last bit
        c = B.count_galaxies(G[p + "_grid"], G[p + "_n"], G[p + "_cellidx"], G[p + "_gals"], ref_zero=True)
        assert np.array_equal(c, G[p + "_counts"]), p
        # the golden set has galaxies on the cell edges, outside, and in grid cell 0
        assert np.sum(e == 0) > 0 and np.sum(e < 0) > 0


def test_restatement_counts_grid_index_zero():
    for p, _ in CASES:
        e = B.grid_index(G[p + "_grid"], G[p + "_n"], G[p + "_gals"])
        w0 = float(np.sum(G[p + "_gals"][e == 0, 3].astype(np.float64)))
        fixed = B.count_galaxies(G[p + "_grid"], G[p + "_n"], G[p + "_cellidx"], G[p + "_gals"])
        ref = G[p + "_counts"]
        assert G[p + "_cellidx"][0] == 0
        assert np.isclose(fixed[0] - ref[0], w0, rtol=1e-12) and np.isclose(ref[-1] - fixed[-1], w0, rtol=1e-12)
        assert np.isclose(fixed.sum(), ref.sum(), rtol=1e-12)


def _engine(coordsys, grid, n):
    sv = synth.Survey(coordsys, grid, n)
    return sv, api.Engine(api.make_config(sv, bands=synth.band_edges(2, 0.0, 0.2)))


@pytest.mark.gpu
def test_gpu_counts_match_restatement():
    for p, cs in CASES:
        grid, n, gals, cellidx = G[p + "_grid"], G[p + "_n"], G[p + "_gals"], G[p + "_cellidx"]
        _, e = _engine(cs, grid, n)
        want = B.count_galaxies(grid, n, cellidx, gals)
        got, outside = e.count_galaxies(_cells(n, cellidx), gals)
        # weights 1, 0.5, 2, 0.37f: FP64 sums in another order
        np.testing.assert_allclose(got, want[:-1], rtol=1e-13, atol=1e-12)
        assert abs(outside - want[-1]) <= 1e-12 * want[-1]
        # dyadic weights sum exactly in any order
        g2 = gals.copy()
        g2[:, 3] = np.where(g2[:, 3] == np.float32(0.37), np.float32(0.25), g2[:, 3])
        got2, out2 = e.count_galaxies(_cells(n, cellidx), g2)
        want2 = B.count_galaxies(grid, n, cellidx, g2)
        assert np.array_equal(got2, want2[:-1]) and out2 == want2[-1]
        e.close()


@pytest.mark.gpu
def test_gpu_counts_large_and_edge_cases():
    rng = np.random.default_rng(11)
    grid, n = (200.0, 1000.0, -1.0, 1.0, 0.0, 2 * np.pi), (16, 32, 32)
    _, e = _engine(synth.COORD_SPHERICAL, grid, n)
    ncell = int(np.prod(n))
    cellidx = np.flatnonzero(rng.random(ncell) < 0.8).astype(np.int32)
    m = 2_000_000
    lo, hi = np.array(grid[0::2]), np.array(grid[1::2])
    x = lo - 0.05 * (hi - lo) + 1.1 * (hi - lo) * rng.random((m, 3))
    gals = np.concatenate([x, rng.integers(1, 4, (m, 1))], axis=1).astype(np.float32)
    # NaN and huge coordinates go to no cell
    gals[:3, 0] = [np.nan, 3e38, -3e38]
    got, outside = e.count_galaxies(_cells(n, cellidx), gals)
    want = B.count_galaxies(grid, n, cellidx, gals)
    assert np.array_equal(got, want[:-1]) and outside == want[-1]
    assert outside >= float(gals[:3, 3].sum())
    # no galaxies: zero counts
    got, outside = e.count_galaxies(_cells(n, cellidx), np.zeros((0, 4), np.float32))
    assert not got.any() and outside == 0.0
    # a cell outside the grid is refused
    bad = _cells(n, cellidx[:4])
    bad["d2"][1] = n[1]
    with pytest.raises(api.OpsecError):
        e.count_galaxies(bad, gals[:10])
    e.close()


@pytest.mark.gpu
def test_dot_program_bins_galfile(tmp_path):
    """dot with survey.galfile equals count_galaxies followed by the library's dot."""
    from opsec_gpu import build

    build.build()
    grid, n, gals, cellidx = G["sph_grid"], G["sph_n"], G["sph_gals"], G["sph_cellidx"]
    sv = synth.Survey(synth.COORD_SPHERICAL, grid, n)
    full = synth.shell_survey(int(n[0]), int(n[1]), int(n[2]), rmin=grid[0], rmax=grid[1])[1]
    cells = full[cellidx].copy()
    cells["a"] = np.arange(cells.size)
    nmodes = 12
    rng = np.random.default_rng(3)
    modes = rng.standard_normal((nmodes, cells.size))
    files = {k: tmp_path / f"{k}.abn" for k in ("cells", "modes", "gals", "pix")}
    formats.write_cells(str(files["cells"]), cells, sv.config_lines())
    with open(files["modes"], "wb") as f:
        formats.write(f, modes.ravel(), "d", {"Nmodes": nmodes, "Ncells": cells.size})
    with open(files["gals"], "wb") as f:
        formats.write(f, np.ascontiguousarray(gals).view("V16").ravel(), "4f")  # one 16-byte record per galaxy
    cfg = api.make_config(sv, bands=synth.band_edges(2, 0.0, 0.2), extra=(
        f"survey.galfile = {files['gals']}", f"cellfile = {files['cells']}", f"modefile = {files['modes']}",
        f"pixfile = {files['pix']}", f"Nmodes = {nmodes}"))
    cfgfile = tmp_path / "dot.cfg"
    cfgfile.write_text(cfg)
    res = subprocess.run([os.path.join(os.path.dirname(HERE), "opsec_gpu", "bin", "dot"), "-c", str(cfgfile)],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    _, y = formats.read(str(files["pix"]))
    e = api.Engine(api.make_config(sv, bands=synth.band_edges(2, 0.0, 0.2)))
    counts, _ = e.count_galaxies(cells, gals)
    want = B.count_galaxies(grid, n, cellidx, gals)
    np.testing.assert_allclose(counts, want[:-1], rtol=1e-13, atol=1e-12)
    np.testing.assert_allclose(y, e.dot(cells, counts, modes), rtol=1e-12, atol=1e-12)
    e.close()
