"""The drop-in programs klt -> comma -> dot -> estimate, run as the reference
pipeline is (code/opsec/python/opsec-submit.in:196-201), on files, against the
library called directly on the same inputs."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from opsec_gpu import api, formats, synth

pytestmark = pytest.mark.gpu
BIN = os.path.join(ROOT, "opsec_gpu", "bin")


def run(prog, cfgfile, *args):
    res = subprocess.run([os.path.join(BIN, prog), "-c", str(cfgfile), *args], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return res


def test_pipeline_programs(tmp_path):
    from opsec_gpu import build

    build.build()
    sv, cells = synth.shell_survey(3, 4, 8)
    k, P = synth.pk_table()
    pk = tmp_path / "pk.dat"
    synth.write_pkfile(str(pk), k, P)
    bands = synth.band_edges(3, 0.0, 0.15)
    nmodes = 40
    cfg = api.make_config(sv, bands=bands, nmodes=nmodes, pkfile=str(pk), extra=("solver = parpack",))
    files = {n: tmp_path / f"{n}.abn" for n in ("cells", "modes", "evals", "cov", "counts", "pix", "est")}
    cfg += "".join(f"{n}file = {p}\n" for n, p in [("cell", files["cells"]), ("mode", files["modes"]),
                                                    ("eval", files["evals"]), ("cov", files["cov"]),
                                                    ("count", files["counts"]), ("pix", files["pix"]),
                                                    ("est", files["est"])])
    cfgfile = tmp_path / "opsec.cfg"
    cfgfile.write_text(cfg)
    formats.write_cells(str(files["cells"]), cells, sv.config_lines())
    counts = synth.grf_counts(sv, cells)
    with open(files["counts"], "wb") as f:
        formats.write(f, counts, "d")
    run("klt", cfgfile)
    run("comma", cfgfile)
    run("dot", cfgfile)
    out = run("estimate", cfgfile)
    assert "p_n" in out.stdout

    mopts, modes = formats.read(str(files["modes"]))
    assert int(mopts["Nmodes"]) == nmodes and int(mopts["Ncells"]) == cells.size and int(mopts["nconv"]) == nmodes
    modes = modes.reshape(nmodes, cells.size)
    _, evals = formats.read(str(files["evals"]))
    copts, cov = formats.read(str(files["cov"]))
    assert copts["packed"] == "1" and int(copts["Nparams"]) == len(bands)
    _, y = formats.read(str(files["pix"]))
    est = formats.read_estfile(str(files["est"]))

    e = api.Engine(api.make_config(sv, bands=bands, nmodes=nmodes))
    e.set_pk(k, P)
    ev2, modes2 = e.klt(cells, nmodes)
    np.testing.assert_array_equal(evals, ev2)
    np.testing.assert_array_equal(modes, modes2)
    cov2 = e.comma(cells, modes)
    np.testing.assert_array_equal(cov.reshape(cov2.shape), cov2)
    np.testing.assert_array_equal(y, e.dot(cells, counts, modes))
    r = e.estimate(evals, cov2, y)
    for name in ("phat", "pcov", "F", "W", "M", "q", "f"):
        np.testing.assert_array_equal(est[name], r[name])
    e.close()


def test_programs_reject_missing_options(tmp_path):
    from opsec_gpu import build

    build.build()
    cfgfile = tmp_path / "empty.cfg"
    cfgfile.write_text("# nothing\n")
    res = subprocess.run([os.path.join(BIN, "klt"), "-c", str(cfgfile)], capture_output=True, text=True)
    assert res.returncode == 1 and "missing configuration options" in res.stderr
    res = subprocess.run([os.path.join(BIN, "klt"), "-h"], capture_output=True, text=True)
    assert res.returncode == 0 and "Usage: klt" in res.stdout
    # the reference's solver key: parpack and anasazi are accepted, anything else refused (klt.cpp:167-193)
    bad = tmp_path / "badsolver.cfg"
    bad.write_text("cellfile = none.abn\nNmodes = 2\nmodefile = m.abn\nevalfile = e.abn\nsolver = lanczos\n")
    res = subprocess.run([os.path.join(BIN, "klt"), "-c", str(bad)], capture_output=True, text=True)
    assert res.returncode == 1 and "unrecognized solver: lanczos" in res.stderr


def test_basis_and_mockcounts_programs(tmp_path):
    """basis writes the cell list (radial selection, quirk off and on), mockcounts the counts per
    cell; both equal the library's own calls."""
    from opsec_gpu import build

    build.build()
    sv = synth.Survey(2, (200.0, 1000.0, -1.0, 1.0, 0.0, 2 * np.pi), (4, 4, 8))
    rr = np.linspace(150.0, 1100.0, 12)
    rn = 3e-4 * np.exp(-((rr - 600.0) / 250.0) ** 2)
    rad = tmp_path / "radial.dat"
    rad.write_text("".join(f"{float(a)!r} {float(b)!r}\n" for a, b in zip(rr, rn)))
    k, P = synth.pk_table()
    pk = tmp_path / "pk.dat"
    synth.write_pkfile(str(pk), k, P)
    bands = synth.band_edges(2, 0.0, 0.1)
    for quirk in (0, 1):
        cells_f, counts_f = tmp_path / f"cells{quirk}.abn", tmp_path / f"counts{quirk}.abn"
        cfg = api.make_config(sv, bands=bands, pkfile=str(pk), extra=(
            f"survey.radial = {rad}", f"basis.quirk3 = {quirk}", f"cellfile = {cells_f}", f"countfile = {counts_f}",
            "mock.seed = 7", "mock.ngrid = 32"))
        cfgfile = tmp_path / f"opsec{quirk}.cfg"
        cfgfile.write_text(cfg)
        run("basis", cfgfile)
        run("mockcounts", cfgfile)
        opts, data = formats.read(str(cells_f))
        cells = np.frombuffer(data.tobytes(), dtype=synth.CELL_DTYPE)
        assert int(opts["Ncells"]) == cells.size == 128
        _, counts = formats.read(str(counts_f))
        e = api.Engine(api.make_config(sv, bands=bands, extra=(f"basis.quirk3 = {quirk}",)))
        e.set_pk(k, P)
        e.set_radial(rr, rn)
        ref = e.basis()
        ref_counts = e.mock_counts(ref, ngrid=32, seed=7)
        e.close()
        assert np.array_equal(cells.view(np.uint8), ref.view(np.uint8))
        assert np.array_equal(counts, ref_counts)
