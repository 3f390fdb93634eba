"""Generate tests/golden/abn_ref.npz: ABN blocks written by the reference's own cfg.c and abn.c.

Run where the reference checkout is present (it is absent on GPU hosts):

    make -C oracle ref REF=<checkout>/code/opsec/src   # builds oracle/_ref/libopsecref.so
    python tests/golden/make_abn_golden.py

Each case is a comment written first (as the programs do with fprintf), then one
abn_write of data under a Config filled with cfg_set in the given order
(abn.c:186-220, cfg.c:297-312): the header of klt's evalfile (klt.cpp:209-218),
comma's covfile (comma-scalapack.cpp:216-223), and a cell block whose options
need quotes and mix upper- and lower-case keys.  Stored: the bytes of the file,
the options in insertion order, the format, the comment and the data bytes.

Split cases: one block cut into pieces name.00, name.01, ... (as `split -d -a 2` cuts a file)
at byte offsets inside the data, read by the reference's SplitFile the way estimate reads its
covfile (ref_split_read in oracle/ref_shim.cpp; SplitFile.cpp:120-175).  Stored: the pieces
and the data as read; a case with its last piece missing stores the short read.

Survey cases: the header the reference's basis writes on its cell file for a box and a
shell (ref_survey_header in oracle/ref_shim.cpp: GetConfigurationOptions plus Ncells), from
the survey's options; stored with the program configuration they come from.

Read cases: blocks of several formats in both byte orders (header written here, data
laid out field by field in that order), read back by the reference's abn_read
(abn.c:249-283, byte-swapped by abn_byte_swap, abn.c:96-183, when the order is not the
host's).  Stored: the file bytes and the data as abn_read returns it.
"""
import ctypes as C
import ctypes.util
import json
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libopsecref.so"))
libc = C.CDLL(ctypes.util.find_library("c"))
libc.fopen.restype = C.c_void_p
libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
libc.fputs.argtypes = [C.c_char_p, C.c_void_p]
libc.fclose.argtypes = [C.c_void_p]
L.cfg_new.restype = C.c_void_p
L.cfg_set.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p]
L.cfg_destroy.argtypes = [C.c_void_p]
L.abn_write.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_char_p, C.c_void_p]
L.abn_write.restype = C.c_size_t


def ref_write(comment, opts, data, n, fmt):
    fd, path = tempfile.mkstemp()
    os.close(fd)
    f = libc.fopen(path.encode(), b"wb")
    libc.fputs(comment.encode(), f)
    cfg = L.cfg_new()
    for k, v in opts:
        L.cfg_set(cfg, k.encode(), v.encode())
    L.abn_write(f, data.ctypes.data, n, fmt.encode(), cfg)
    L.cfg_destroy(cfg)
    libc.fclose(f)
    raw = open(path, "rb").read()
    os.remove(path)
    return raw


L.abn_read.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t),
                       C.c_char_p, C.c_char_p, C.c_void_p]
libc.free.argtypes = [C.c_void_p]
CODES = {"c": "S1", "b": "i1", "B": "u1", "h": "i2", "H": "u2", "i": "i4", "I": "u4", "q": "i8", "Q": "u8",
         "l": "i8", "f": "f4", "d": "f8"}


def fields(fmt):
    out, num = [], ""
    for ch in fmt:
        if ch.isdigit():
            num += ch
            continue
        out += [ch] * (int(num) if num else 1)
        num = ""
    return out


def ref_read(raw):
    fd, path = tempfile.mkstemp()
    os.write(fd, raw)
    os.close(fd)
    f = libc.fopen(path.encode(), b"rb")
    ptr, n, size = C.c_void_p(), C.c_size_t(), C.c_size_t()
    endian, fmt = C.create_string_buffer(4), C.create_string_buffer(64)
    assert L.abn_read(f, C.byref(ptr), C.byref(n), C.byref(size), endian, fmt, None) == 0
    data = C.string_at(ptr, n.value * size.value)
    libc.free(ptr)
    libc.fclose(f)
    os.remove(path)
    return data


def read_cases(out):
    rng = np.random.default_rng(7)
    for fmt in ("d", "4f", "4i8d", "2h3q", "c2hfI"):
        fl = fields(fmt)
        n = 3
        for endian, e in (("L", "<"), ("B", ">")):
            dt = np.dtype([(f"f{k}", e + CODES[c]) for k, c in enumerate(fl)])
            rec = np.zeros(n, dtype=dt)
            for k, c in enumerate(fl):
                if c in "fd":
                    rec[f"f{k}"] = rng.standard_normal(n)
                elif c == "c":
                    rec[f"f{k}"] = [b"a", b"Z", b"!"]
                else:
                    info = np.iinfo(np.dtype(CODES[c]))
                    rec[f"f{k}"] = rng.integers(info.min // 2, info.max // 2, n)
            head = (f"\n# a {fmt} block\nNcells = {n}\n#!Begin data block: n = {n}, size = {dt.itemsize}, "
                    f"endian = {endian}, format = {fmt}\n").encode()
            raw = head + rec.tobytes()
            name = f"read_{fmt}_{endian}"
            out[name + "_file"] = np.frombuffer(raw, dtype=np.uint8)
            out[name + "_data"] = np.frombuffer(ref_read(raw), dtype=np.uint8)


L.ref_split_read.argtypes = [C.c_char_p, C.c_void_p, C.c_long]
L.ref_split_read.restype = C.c_long


def split_cases(out):
    rng = np.random.default_rng(11)
    data = rng.standard_normal(500)
    head = b"\n# Derivatives of the covariance matrix\nNmodes = 4\n" \
           b"#!Begin data block: n = 500, size = 8, endian = L, format = d\n"
    raw = head + data.tobytes()
    for name, cuts, drop_last in (("three", (len(head) + 100, len(head) + 2501), False),
                                  ("header_only", (len(head),), False),
                                  ("whole", (), False),
                                  ("missing", (len(head) + 800, len(head) + 2000), True)):
        pieces, prev = [], 0
        for c in list(cuts) + [len(raw)]:
            pieces.append(raw[prev:c])
            prev = c
        d = tempfile.mkdtemp()
        paths = [os.path.join(d, f"cov.abn.{i:02d}") for i in range(len(pieces))]
        for i, (p, b) in enumerate(zip(paths, pieces)):
            if drop_last and i == len(pieces) - 1:
                continue
            open(p, "wb").write(b)
        buf = C.create_string_buffer(len(data) * 8 + 64)
        got = L.ref_split_read(paths[0].encode(), buf, len(data) * 8)
        for p in paths:
            if os.path.exists(p):
                os.remove(p)
        os.rmdir(d)
        out[f"split_{name}_npieces"] = np.array([len(pieces) - (1 if drop_last else 0)])
        for i, b in enumerate(pieces[:len(pieces) - (1 if drop_last else 0)]):
            out[f"split_{name}_piece{i}"] = np.frombuffer(b, dtype=np.uint8)
        out[f"split_{name}_data"] = np.frombuffer(buf.raw[:got], dtype=np.uint8)


L.ref_survey_header.argtypes = [C.c_int, C.c_char_p, C.c_int, C.c_char_p]

SURVEYS = {
    "box": (1, "survey.type = BoxSurvey\nsurvey.XMin = 0\nsurvey.XMax = 600.0\nsurvey.YMin = -12.5\n"
               "survey.YMax = 587.5\nsurvey.ZMin = 0.001\nsurvey.ZMax = 1234567.891\nsurvey.Nx = 12\n"
               "survey.Ny = 0x0c\nsurvey.Nz = 12\nsurvey.galfile = gals.abn\nsurvey.nbar = 3e-4\nsurvey.L = 600\n"),
    "sph": (2, "survey.type = SphericalSurvey\nsurvey.RMin = 200\nsurvey.RMax = 1000.0\nsurvey.MuMin = -1\n"
               "survey.MuMuin = -1.0\nsurvey.MuMax = 1\nsurvey.PhiMin = 0\nsurvey.PhiMax = 6.283185307179586\n"
               "survey.Nr = 32\nsurvey.Nmu = 32\nsurvey.Nphi = 32\nsurvey.galfile = none\n"
               "survey.maskfile = none\nsurvey.radial = none\n"),
}


def survey_cases(out):
    for name, (coordsys, text) in SURVEYS.items():
        sub = "".join(line[len("survey."):] + "\n" for line in text.splitlines() if line.startswith("survey."))
        d = tempfile.mkdtemp()
        src, dst = os.path.join(d, "survey.cfg"), os.path.join(d, "head.abn")
        open(src, "w").write(sub)
        assert L.ref_survey_header(coordsys, src.encode(), 1728, dst.encode()) == 0
        out[f"survey_{name}_cfg"] = np.frombuffer(text.encode(), dtype=np.uint8)
        out[f"survey_{name}_head"] = np.frombuffer(open(dst, "rb").read(), dtype=np.uint8)
        os.remove(src)
        os.remove(dst)
        os.rmdir(d)


def main():
    rng = np.random.default_rng(20261203)
    cases = {
        "klt_eval": ("# Signal matrix eigenvalues\n",
                     [("cellfile", "cells.abn"), ("Ncells", "1728"), ("Nmodes", "5"), ("nconv", "5")],
                     rng.standard_normal(5), 5, "d"),
        "comma_cov": ("# Derivatives of the covariance matrix in KL basis, C_{ij,m}.\n",
                      [("Nmodes", "3"), ("Nparams", "2"), ("packed", "1")], rng.standard_normal(12), 12, "d"),
        "cells_quoted": ("",
                         [("survey.type", "BoxSurvey"), ("zeta", " padded "), ("Ncells", "2"), ("alpha", "x y"),
                          ("Beta", "tab\t")],
                         rng.integers(0, 255, 160, dtype=np.uint8), 2, "4i8d"),
    }
    out = {}
    for name, (comment, opts, data, n, fmt) in cases.items():
        data = np.ascontiguousarray(data)
        out[name + "_file"] = np.frombuffer(ref_write(comment, opts, data, n, fmt), dtype=np.uint8)
        out[name + "_meta"] = np.frombuffer(json.dumps({"comment": comment, "opts": opts, "n": n, "fmt": fmt}).encode(),
                                            dtype=np.uint8)
        out[name + "_data"] = np.frombuffer(data.tobytes(), dtype=np.uint8)
    read_cases(out)
    split_cases(out)
    survey_cases(out)
    np.savez_compressed(os.path.join(HERE, "abn_ref.npz"), **out)
    for name in cases:
        print(name, out[name + "_file"].tobytes()[:400])


if __name__ == "__main__":
    main()
