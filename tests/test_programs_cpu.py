"""The drop-in programs' option handling, which runs before any device call (no GPU needed):
usage text, missing options, the reference's solver key, and the dot program's count source."""
import os
import subprocess

import pytest

from conftest import ROOT

BIN = os.path.join(ROOT, "opsec_gpu", "bin")


@pytest.fixture(scope="module")
def run():
    from opsec_gpu import build

    build.build()

    def go(prog, text=None, *args, tmp=None):
        cmd = [os.path.join(BIN, prog)]
        if text is not None:
            p = os.path.join(tmp, f"{prog}.cfg")
            with open(p, "w") as f:
                f.write(text)
            cmd += ["-c", p]
        return subprocess.run(cmd + list(args), capture_output=True, text=True, timeout=60)

    return go


@pytest.mark.parametrize("prog", ["basis", "klt", "comma", "dot", "estimate", "mockcounts"])
def test_usage_and_missing_options(run, tmp_path, prog):
    res = run(prog, None, "-h")
    assert res.returncode == 0 and f"Usage: {prog}" in res.stdout
    res = run(prog, "# nothing\n", tmp=str(tmp_path))
    assert res.returncode == 1 and "missing configuration options" in res.stderr


def test_klt_solver_key(run, tmp_path):
    base = "cellfile = none.abn\nNmodes = 2\nmodefile = m.abn\nevalfile = e.abn\n"
    res = run("klt", base + "solver = lanczos\n", tmp=str(tmp_path))
    assert res.returncode == 1 and "unrecognized solver: lanczos" in res.stderr
    for ok in ("parpack", "anasazi"):
        res = run("klt", base + f"solver = {ok}\n", tmp=str(tmp_path))
        # accepted: the program goes on to the cell file, which does not exist
        assert res.returncode == 1 and "could not open 'none.abn'" in res.stderr


def test_dot_needs_a_galaxy_or_count_file(run, tmp_path):
    base = "cellfile = c.abn\nmodefile = m.abn\npixfile = p.abn\nNmodes = 2\n"
    res = run("dot", base, tmp=str(tmp_path))
    assert res.returncode == 1 and "survey.galfile or countfile" in res.stderr
    res = run("dot", base + "survey.galfile = none\n", tmp=str(tmp_path))
    assert res.returncode == 1 and "survey.galfile or countfile" in res.stderr


def test_configuration_file_stops_at_an_invalid_line(run, tmp_path):
    """cfg_read (cfg.c:200-214): options after the first invalid line of a -c file are not read,
    so Nmodes below is missing; on the command line each option line stands alone."""
    text = "cellfile = c.abn\nmodefile = m.abn\nevalfile = e.abn\nnot an option\nNmodes = 2\n"
    res = run("klt", text, tmp=str(tmp_path))
    assert res.returncode == 1 and "not a valid configuration line" in res.stderr
    assert "missing configuration options Nmodes" in res.stderr
    res = run("klt", text, "Nmodes=2", tmp=str(tmp_path))
    assert res.returncode == 1 and "could not open 'c.abn'" in res.stderr
