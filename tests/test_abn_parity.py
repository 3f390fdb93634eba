"""ABN files and configuration files as the reference writes and reads them: the
programs' code (opsec_gpu/programs/progs.cpp, compiled here with g++) and the Python
one (opsec_gpu/formats.py) against the reference's own cfg.c / abn.c:
- blocks it wrote (tests/golden/abn_ref.npz, tests/golden/make_abn_golden.py): comment,
  the options sorted as its Config keeps them, quoting, the data-block line, the data;
- configuration texts it read (tests/golden/cfg_ref.npz, tests/golden/make_cfg_golden.py):
  comments, whitespace, quotes, repeated keys, and the end of reading at the first line
  that is not key = value;
- blocks of several struct formats in both byte orders as its abn_read returns them
  (byte-swapped field by field when the order is not the host's);
- a block cut into pieces name.00, name.01, ... as its SplitFile reads it (estimate's
  covfile and evalfile, comma's modefile)."""
import ctypes as C
import io
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from opsec_gpu import formats

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "abn_ref.npz"))
CASES = ("klt_eval", "comma_cov", "cells_quoted")
GC = np.load(os.path.join(HERE, "golden", "cfg_ref.npz"))
CFG_CASES = sorted({k[:-3] for k in GC.files if k.endswith("_in")})
READ_CASES = sorted({k[:-5] for k in G.files if k.startswith("read_") and k.endswith("_file")})


def _case(name):
    meta = json.loads(G[name + "_meta"].tobytes())
    return meta, G[name + "_data"].tobytes(), G[name + "_file"].tobytes()


@pytest.fixture(scope="module")
def writer(tmp_path_factory):
    from opsec_gpu import build

    build.build()
    libdir = os.path.join(ROOT, "opsec_gpu")
    so = str(tmp_path_factory.mktemp("abn") / "libabn_check.so")
    subprocess.check_call(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-o", so,
                           os.path.join(HERE, "abn_check.cpp"), os.path.join(ROOT, "opsec_gpu", "programs", "progs.cpp"),
                           f"-L{libdir}", "-lopsec_gpu", f"-Wl,-rpath,{libdir}"])
    L = C.CDLL(so)
    L.chk_abn_write.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p),
                                C.c_void_p, C.c_size_t, C.c_char_p]
    L.chk_cfg_dump.argtypes = [C.c_char_p, C.c_char_p]
    L.chk_abn_read.argtypes = [C.c_char_p, C.c_void_p, C.c_size_t]
    L.chk_abn_read.restype = C.c_longlong
    L.chk_abn_read_split.argtypes = [C.c_char_p, C.c_void_p, C.c_size_t]
    L.chk_abn_read_split.restype = C.c_longlong
    L.chk_get_int.argtypes = [C.c_char_p]
    L.chk_read_cells.argtypes = [C.c_char_p]
    L.chk_read_cells.restype = C.c_longlong
    L.chk_survey_header.argtypes = [C.c_char_p, C.c_int, C.c_char_p]
    return L


@pytest.mark.parametrize("name", CASES)
def test_program_writer_matches_reference_bytes(writer, tmp_path, name):
    meta, data, ref = _case(name)
    keys = (C.c_char_p * len(meta["opts"]))(*[k.encode() for k, _ in meta["opts"]])
    vals = (C.c_char_p * len(meta["opts"]))(*[v.encode() for _, v in meta["opts"]])
    buf = C.create_string_buffer(data, len(data))
    path = tmp_path / "out.abn"
    assert writer.chk_abn_write(str(path).encode(), meta["comment"].encode(), len(meta["opts"]), keys, vals,
                                C.cast(buf, C.c_void_p), meta["n"], meta["fmt"].encode()) == 0
    assert path.read_bytes() == ref


@pytest.mark.parametrize("name", CASES)
def test_python_writer_matches_reference_bytes(name):
    meta, data, ref = _case(name)
    rec = {"d": np.float64, "4i8d": np.dtype((np.void, 80))}[meta["fmt"]]
    arr = np.frombuffer(data, dtype=rec)
    f = io.BytesIO()
    formats.write(f, arr, meta["fmt"], dict(meta["opts"]), comment=meta["comment"])  # the comment keeps its newline
    assert f.getvalue() == ref


def test_reader_round_trip_of_reference_bytes(tmp_path):
    for name in CASES:
        meta, data, ref = _case(name)
        p = tmp_path / f"{name}.abn"
        p.write_bytes(ref)
        opts, arr = formats.read(str(p))
        for k, v in meta["opts"]:
            assert opts[k] == v, (name, k)
        assert arr.tobytes() == data


def test_cfg_cases_cover_the_rules():
    assert {"plain", "whitespace", "quotes", "values", "stop", "stop_eq"} <= set(CFG_CASES)


@pytest.mark.parametrize("name", CFG_CASES)
def test_program_config_reader_matches_reference(writer, tmp_path, name):
    src, dst = tmp_path / "in.cfg", tmp_path / "out.abn"
    src.write_bytes(GC[name + "_in"].tobytes())
    assert writer.chk_cfg_dump(str(src).encode(), str(dst).encode()) == 0
    assert dst.read_bytes() == GC[name + "_out"].tobytes()


@pytest.mark.parametrize("name", CFG_CASES)
def test_python_config_reader_matches_reference(name):
    opts = formats.parse_config(GC[name + "_in"].tobytes().decode("latin-1"))
    f = io.BytesIO()
    formats.write(f, np.zeros(0), "d", opts)
    assert f.getvalue() == GC[name + "_out"].tobytes()


def test_read_cases_cover_both_byte_orders():
    assert len(READ_CASES) >= 10 and {c[-1] for c in READ_CASES} == {"L", "B"}


@pytest.mark.parametrize("name", READ_CASES)
def test_program_reader_matches_reference(writer, tmp_path, name):
    p = tmp_path / "in.abn"
    p.write_bytes(G[name + "_file"].tobytes())
    want = G[name + "_data"].tobytes()
    buf = C.create_string_buffer(len(want) + 16)
    assert writer.chk_abn_read(str(p).encode(), buf, len(buf)) == len(want)
    assert buf.raw[:len(want)] == want


@pytest.mark.parametrize("name", READ_CASES)
def test_python_reader_matches_reference(tmp_path, name):
    p = tmp_path / "in.abn"
    p.write_bytes(G[name + "_file"].tobytes())
    opts, arr = formats.read(str(p))
    assert opts["Ncells"] == "3"
    assert arr.astype(arr.dtype.newbyteorder("=")).tobytes() == G[name + "_data"].tobytes()


@pytest.mark.parametrize("name", ["three", "header_only", "whole", "missing"])
def test_split_file_reading_matches_reference(writer, tmp_path, name):
    npieces = int(G[f"split_{name}_npieces"][0])
    for i in range(npieces):
        (tmp_path / f"cov.abn.{i:02d}").write_bytes(G[f"split_{name}_piece{i}"].tobytes())
    want = G[f"split_{name}_data"].tobytes()
    buf = C.create_string_buffer(4096)
    got = writer.chk_abn_read_split(str(tmp_path / "cov.abn.00").encode(), buf, len(buf))
    if name == "missing":
        # the reference returns the 2,000 bytes it found; the programs refuse the short block
        assert len(want) == 2000 and got == -1
    else:
        assert got == len(want) == 4000 and buf.raw[:got] == want
        # the Python reader follows the pieces too
        _, arr = formats.read(str(tmp_path / "cov.abn.00"))
        assert arr.tobytes() == want


def test_integer_options_read_as_scanf_i(writer):
    """cfg_get_int (cfg.c:430-440) reads "%i": octal and hex prefixes, trailing text ignored."""
    for text, want in (("500", 500), ("010", 8), ("0x1F", 31), ("12abc", 12), ("500 # modes", 500), ("  -7", -7)):
        assert writer.chk_get_int(text.encode()) == want, text


def test_cell_file_checks_follow_read_cells(writer, tmp_path):
    """ReadCells (Cell.cpp:16-56): the header's Ncells must equal the record count and the
    record size must be 80 bytes; the format string itself is not checked."""
    from opsec_gpu import synth

    cells = np.zeros(3, dtype=synth.CELL_DTYPE)
    cells["a"] = np.arange(3)

    def put(name, opts, fmt="4i8d", arr=cells):
        p = tmp_path / name
        with open(p, "wb") as f:
            formats.write(f, arr, fmt, opts)
        return str(p).encode()

    assert writer.chk_read_cells(put("ok.abn", {"Ncells": 3})) == 3
    assert writer.chk_read_cells(put("other_fmt.abn", {"Ncells": 3}, fmt="10d")) == 3
    assert writer.chk_read_cells(put("no_ncells.abn", {"survey.type": "BoxSurvey"})) == -1
    assert writer.chk_read_cells(put("wrong_ncells.abn", {"Ncells": 4})) == -1
    assert writer.chk_read_cells(put("small.abn", {"Ncells": 3}, fmt="9d", arr=np.zeros((3, 9)))) == -1


@pytest.mark.parametrize("name", ["box", "sph"])
def test_basis_cell_file_header_matches_reference(writer, tmp_path, name):
    """The basis program's cell-file header: the survey's GetConfigurationOptions (unprefixed
    keys, doubles as "%g", MuMin from MuMuin) and Ncells, as the reference's basis writes it."""
    cfg, out = tmp_path / "opsec.cfg", tmp_path / "head.abn"
    cfg.write_bytes(G[f"survey_{name}_cfg"].tobytes())
    assert writer.chk_survey_header(str(cfg).encode(), 1728, str(out).encode()) == 0
    assert out.read_bytes() == G[f"survey_{name}_head"].tobytes()


@pytest.mark.parametrize("name", ["box", "sph"])
def test_python_cell_file_header_matches_reference(name):
    opts = formats.survey_header(formats.parse_config(G[f"survey_{name}_cfg"].tobytes().decode()), 1728)
    f = io.BytesIO()
    formats.write(f, np.zeros(1728, dtype=np.dtype((np.void, 80))), "4i8d", opts)
    assert f.getvalue()[:len(G[f"survey_{name}_head"])] == G[f"survey_{name}_head"].tobytes()


def test_c_number_readers():
    for text, want in (("12", 12), ("0x0c", 12), ("010", 8), ("0", 0), ("-7 # x", -7), ("abc", 0), ("  +5", 5)):
        assert formats.c_int(text) == want, text
    for text, want in (("3e-4", 3e-4), ("600.0", 600.0), (".5x", 0.5), ("-1", -1.0), ("", 0.0)):
        assert formats.c_double(text) == want, text


def test_split_command_pieces_read_back(writer, tmp_path):
    """After testSplitFile.cpp: a file cut by `split -d -b 999` (pieces name00, name01, ...)
    reads back whole -- here an ABN block of 4,096 random bytes, by the programs' reader and
    the Python reader."""
    rng = np.random.default_rng(32)
    data = rng.integers(0, 256, 4096, dtype=np.uint8)
    full = tmp_path / "fullrandom"
    with open(full, "wb") as f:
        formats.write(f, data, "B", {"Nbytes": 4096})
    subprocess.check_call(["split", "-d", "-b", "999", str(full), str(tmp_path / "splitrandom")])
    first = tmp_path / "splitrandom00"
    assert (tmp_path / "splitrandom04").exists()
    buf = C.create_string_buffer(4096)
    assert writer.chk_abn_read_split(str(first).encode(), buf, 4096) == 4096
    assert buf.raw == data.tobytes()
    opts, arr = formats.read(str(first))
    assert opts["Nbytes"] == "4096" and arr.tobytes() == data.tobytes()


def test_program_round_trip_after_testabn(writer, tmp_path):
    """After testabn.c: 100 values cos(i) written with no options and read back -- count, record
    size and values -- through the programs' writer and reader."""
    data = np.cos(np.arange(100.0))
    p = tmp_path / "cos.abn"
    keys = (C.c_char_p * 0)()
    assert writer.chk_abn_write(str(p).encode(), b"", 0, keys, keys, data.ctypes.data, 100, b"d") == 0
    buf = C.create_string_buffer(800)
    assert writer.chk_abn_read(str(p).encode(), buf, 800) == 800
    assert np.array_equal(np.frombuffer(buf.raw, dtype=np.float64), data)
    opts, arr = formats.read(str(p))
    assert opts == {} and arr.dtype == np.float64 and np.array_equal(arr, data)
