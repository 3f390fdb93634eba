"""The C-ABI library builds, loads and exports every entry point that
include/opsec_gpu.h declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "opsec_gpu.h")).read()
    return sorted(set(re.findall(r"\b(opsec_gpu_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from opsec_gpu import build

    lib, _ = build.build()
    L = ctypes.CDLL(lib)
    names = declared_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_cell_layout_matches_reference():
    from opsec_gpu import synth

    assert synth.CELL_DTYPE.itemsize == 80
    assert [synth.CELL_DTYPE.fields[n][1] for n in ("a", "d1", "d2", "d3", "min1", "Nbar")] == [0, 4, 8, 12, 16, 72]
