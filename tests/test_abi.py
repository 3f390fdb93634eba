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


def test_python_bindings_match_the_header():
    """Every entry point the ctypes mirror binds takes as many arguments as include/opsec_gpu.h
    declares (a missing or extra argtype would pass garbage without a GPU error)."""
    import re
    from opsec_gpu import api, build

    build.build()
    text = open(os.path.join(ROOT, "include", "opsec_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//.*", "", text)
    decls = dict(re.findall(r"\b(?:int|void|long long|const char\s*\*|double)\s+(opsec_gpu_\w+)\s*\(([^;]*?)\)\s*;",
                            text, flags=re.S))
    assert len(decls) == len(declared_symbols())
    L = api.load()
    bound = 0
    for name, params in decls.items():
        fn = getattr(L, name)
        if fn.argtypes is None:
            continue
        nparam = len([p for p in params.split(",") if p.strip() and p.strip() != "void"])
        assert len(fn.argtypes) == nparam, (name, len(fn.argtypes), nparam)
        bound += 1
    assert bound >= 25, bound
