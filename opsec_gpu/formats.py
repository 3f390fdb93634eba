"""Annotated binary (ABN) files and key = value configuration, in Python.

The layout is the reference's (code/opsec/src/abn.h:13-60, abn.c:150-330):
free text and ``key = value`` lines, then the line
``#!Begin data block: n = N, size = S, endian = E, format = F`` followed by
N*S raw bytes; several blocks may follow each other (the estfile holds seven).
Used by the tests and by callers that want to read or write the programs'
files from Python.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

from .synth import CELL_DTYPE

_BEGIN = re.compile(rb"#!Begin data block: n = (\d+), size = (\d+), endian = (\S), format = (\S+)")
_DTYPES = {"d": "f8", "f": "f4", "i": "i4", "q": "i8", "4i8d": None}


_CSPACE = " \t\n\v\f\r"  # C isspace


def parse_line(line: str):
    """cfg_read_line (cfg.c:238-295): (key, value), None for a blank or '#' line, False for a
    line that is not key = value.  Whitespace is C isspace; one pair of quotes is stripped."""
    s = line.lstrip(_CSPACE)
    if not s or s[0] == "#":
        return None
    eq = s.find("=")
    if eq <= 0:
        return False
    k = s[:eq].rstrip(_CSPACE)
    v = s[eq + 1:].strip(_CSPACE)
    if len(v) >= 2 and v[0] == v[-1] and v[0] in "\"'":
        v = v[1:-1]
    return k, v


def parse_config(text: str, stop_at_invalid: bool = True) -> dict:
    """A configuration file as cfg_read reads it (cfg.c:200-214): key = value lines, the last
    value of a key kept, reading stopped by the first invalid line (stop_at_invalid; ABN
    headers, read line by line by abn_read_header, abn.c:221-247, skip it instead)."""
    out = {}
    for line in text.split("\n"):
        r = parse_line(line)
        if r is False:
            if stop_at_invalid:
                break
            continue
        if r is not None:
            out[r[0]] = r[1]
    return out


_CODES = {"x": "V1", "c": "S1", "b": "i1", "B": "u1", "h": "i2", "H": "u2", "i": "i4", "I": "u4", "l": "i8",
          "L": "u8", "q": "i8", "Q": "u8", "f": "f4", "d": "f8"}


def _fields(fmt: str):
    """Field codes of an ABN struct format, repeat counts expanded (abn.c:96-176)."""
    out, num = [], ""
    for ch in fmt:
        if ch.isspace():
            continue
        if ch.isdigit():
            num += ch
            continue
        out += [ch] * (int(num) if num else 1)
        num = ""
    return out


def _dtype(fmt: str, size: int, endian: str):
    """numpy dtype of one record in the file's byte order; values read through it come out
    as abn_read returns them after abn_byte_swap."""
    e = "<" if endian == "L" else ">"
    if fmt == "4i8d":
        dt = CELL_DTYPE if e == "<" else CELL_DTYPE.newbyteorder(">")
        return dt
    code = _DTYPES.get(fmt)
    if code is not None:
        return np.dtype(e + code)
    fl = _fields(fmt)
    if not fl or any(c not in _CODES for c in fl):
        return np.dtype(f"V{size}")
    dt = np.dtype([(f"f{k}", (e if _CODES[c][0] not in "VS" else "") + _CODES[c]) for k, c in enumerate(fl)])
    return dt if dt.itemsize == size else np.dtype(f"V{size}")


def _next_piece(name: str, index: int) -> str:
    """SplitFile's next piece (SplitFile.cpp:150-175): the last two characters replaced by the
    two-digit index."""
    return name[:-2] + f"{index % 100:02d}"


def read_blocks(path: str):
    """All data blocks of an ABN file: list of (opts, array).  A block whose data runs past the
    end of the file goes on in the next pieces of a `split -d` series (name.00, name.01, ...),
    as the reference's SplitFile reads it."""
    data = open(path, "rb").read()
    name, index = path, 0
    pos = 0
    blocks = []
    while True:
        m = _BEGIN.search(data, pos)
        if not m:
            break
        header = data[pos:m.start()].decode("ascii", "replace")
        n, size, endian, fmt = int(m.group(1)), int(m.group(2)), m.group(3).decode(), m.group(4).decode()
        start = data.index(b"\n", m.end()) + 1
        while len(data) < start + n * size and len(name) >= 2:
            index += 1
            name = _next_piece(name, index)
            if not os.path.exists(name):
                break
            data += open(name, "rb").read()
        dt = _dtype(fmt, size, endian)
        arr = np.frombuffer(data[start:start + n * size], dtype=dt, count=n).copy()
        blocks.append((parse_config(header, stop_at_invalid=False), arr))
        pos = start + n * size
    return blocks


def read(path: str):
    """The first data block: (opts, array)."""
    b = read_blocks(path)
    if not b:
        raise ValueError(f"{path}: no ABN data block")
    return b[0]


def write(f, array, fmt: str, opts: dict | None = None, comment: str = ""):
    """Append one block to an open binary file (abn_write, abn.c:186-220): `comment`, the text
    the programs print before the block (its lines ending in a newline), then the block's
    header -- an empty line, the options, the data-block line -- and the data."""
    a = np.ascontiguousarray(array)
    size = a.dtype.itemsize
    endian = "L" if sys.byteorder == "little" else "B"
    head = comment + "\n"
    # keys in strcmp order with the quoting rule of cfg_write (cfg.c:292-312): the reference's
    # Config keeps its entries sorted
    for k in sorted((opts or {}), key=lambda x: str(x).encode()):
        v = str(opts[k])
        head += f'{k} = "{v}"\n' if v and (v[0].isspace() or v[-1].isspace()) else f"{k} = {v}\n"
    head += f"#!Begin data block: n = {a.size}, size = {size}, endian = {endian}, format = {fmt}\n"
    f.write(head.encode())
    f.write(a.tobytes())


_C_INT = re.compile(r"\s*([+-]?)(0[xX][0-9a-fA-F]+|0[0-7]*|[1-9][0-9]*)")
_C_DBL = re.compile(r"\s*[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?")


def c_int(text: str) -> int:
    """The leading integer of text as strtol(text, 0, 0) / "%i" reads it (0 when there is none)."""
    m = _C_INT.match(text)
    if not m:
        return 0
    sign, digits = m.groups()
    v = int(digits, 16) if digits[:2] in ("0x", "0X") else int(digits, 8) if digits.startswith("0") else int(digits)
    return -v if sign == "-" else v


def c_double(text: str) -> float:
    """The leading number of text as strtod reads it (0 when there is none)."""
    m = _C_DBL.match(text)
    return float(m.group(0)) if m else 0.0


def survey_header(opts: dict, ncells: int) -> dict:
    """The options basis writes on its cell file (basis.cpp:195-199): the survey's
    GetConfigurationOptions (Survey.cpp:103-129, BoxSurvey.cpp:135-141,
    SphericalSurvey.cpp:172-178) from `survey.*` options -- keys unprefixed, doubles "%g",
    MuMin from MuMuin (Survey.cpp:39) -- and Ncells."""
    g = lambda k: f"{c_double(opts.get('survey.' + k, '')):g}"
    i = lambda k: str(c_int(opts.get("survey." + k, "")))
    if opts.get("survey.type") == "BoxSurvey":
        out = {"coordsys": "cartesian"}
        out.update({k: g(k) for k in ("XMin", "XMax", "YMin", "YMax", "ZMin", "ZMax")})
        out.update({k: i(k) for k in ("Nx", "Ny", "Nz")})
        out.update(galfile=opts.get("survey.galfile", ""), nbar=g("nbar"), L=g("L"))
    else:
        out = {"coordsys": "spherical", "RMin": g("RMin"), "RMax": g("RMax"),
               "MuMin": g("MuMuin" if "survey.MuMuin" in opts else "MuMin"), "MuMax": g("MuMax"),
               "PhiMin": g("PhiMin"), "PhiMax": g("PhiMax")}
        out.update({k: i(k) for k in ("Nr", "Nmu", "Nphi")})
        out.update(galfile=opts.get("survey.galfile", ""), maskfile=opts.get("survey.maskfile", ""),
                   radial=opts.get("survey.radial", ""))
    out["Ncells"] = str(ncells)
    return out


def write_cells(path: str, cells, survey_lines=()):
    """A cellfile as basis writes it (basis.cpp:195-201): the header of survey_header from the
    `survey.*` configuration lines, then the 4i8d records."""
    opts = survey_header(parse_config("\n".join(survey_lines)), len(cells))
    with open(path, "wb") as f:
        write(f, np.asarray(cells, dtype=CELL_DTYPE), "4i8d", opts)


def read_estfile(path: str):
    """The seven records of an estfile (estimate-mpi.cpp:635-641)."""
    b = read_blocks(path)
    nb = int(b[0][0]["Nparams"])
    names = ["phat", "pcov", "F", "W", "M", "q", "f"]
    out = {}
    for name, (_, arr) in zip(names, b):
        out[name] = arr.reshape(nb, nb) if arr.size == nb * nb and name in ("pcov", "F", "W", "M") else arr
    return out
