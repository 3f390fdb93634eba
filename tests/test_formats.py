"""ABN files and configuration text: the Python reader/writer against a cell
file written by the reference's own abn_write (tests/golden/cells_ref.abn,
made by make_golden.py), and round trips."""
import os

import numpy as np

from conftest import ROOT
from opsec_gpu import formats, synth


def test_reads_reference_written_cellfile(golden):
    opts, cells = formats.read(os.path.join(ROOT, "tests", "golden", "cells_ref.abn"))
    ref = golden["cells_ref"]
    assert cells.dtype == synth.CELL_DTYPE
    assert int(opts["Ncells"]) == ref.size == cells.size
    assert opts["coordsys"] == "spherical"
    assert int(opts["Nr"]) == 3 and int(opts["Nmu"]) == 4 and int(opts["Nphi"]) == 6
    for name in synth.CELL_DTYPE.names:
        np.testing.assert_array_equal(cells[name], ref[name])


def test_abn_round_trip(tmp_path):
    path = tmp_path / "x.abn"
    a = np.arange(10, dtype=np.float64) * 0.5
    b = np.arange(4, dtype=np.float64)
    with open(path, "wb") as f:
        formats.write(f, a, "d", {"Nparams": 10, "packed": 1}, comment="# a comment")
        formats.write(f, b, "d")
    blocks = formats.read_blocks(str(path))
    assert len(blocks) == 2
    assert blocks[0][0] == {"Nparams": "10", "packed": "1"}
    np.testing.assert_array_equal(blocks[0][1], a)
    np.testing.assert_array_equal(blocks[1][1], b)


def test_cellfile_round_trip(tmp_path):
    sv, cells = synth.shell_survey(2, 3, 4)
    p = tmp_path / "cells.abn"
    formats.write_cells(str(p), cells, sv.config_lines())
    opts, back = formats.read(str(p))
    # the header basis writes: the survey's options unprefixed (Survey.cpp:103-129) and Ncells
    assert int(opts["Ncells"]) == cells.size and opts["coordsys"] == "spherical"
    assert (opts["Nr"], opts["Nmu"], opts["Nphi"]) == ("2", "3", "4") and opts["RMin"] == "200"
    assert back.tobytes() == cells.tobytes()


def test_config_parsing_rules():
    text = "# comment\n  key = value  \nq = \"  spaced  \"\nbad line\nk2=v2\nkey = override\n"
    # a configuration file stops at its first invalid line (cfg.c:200-214) ...
    assert formats.parse_config(text) == {"key": "value", "q": "  spaced  "}
    # ... an ABN header reads on past it (abn.c:221-247)
    assert formats.parse_config(text, stop_at_invalid=False) == {"key": "override", "q": "  spaced  ", "k2": "v2"}
