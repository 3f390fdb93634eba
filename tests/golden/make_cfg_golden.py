"""Generate tests/golden/cfg_ref.npz: configuration files as the reference's cfg.c reads them.

Run where the reference checkout is present (it is absent on GPU hosts):

    make -C oracle ref REF=<checkout>/code/opsec/src   # builds oracle/_ref/libopsecref.so
    python tests/golden/make_cfg_golden.py

Each case is a configuration text, read with cfg_read_file (cfg.c:200-232; opsec_init
reads `-c FILE` with it, opsec.c:33-35) and written back with abn_write_header (abn.c:186-211:
an empty line, cfg_write's sorted `key = value` lines with its quoting, the data-block line
for n = 0 doubles).  Stored: the input bytes and the reference's output bytes.
"""
import ctypes as C
import ctypes.util
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libopsecref.so"))
libc = C.CDLL(ctypes.util.find_library("c"))
libc.fopen.restype = C.c_void_p
libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
libc.fclose.argtypes = [C.c_void_p]
L.cfg_new.restype = C.c_void_p
L.cfg_read_file.argtypes = [C.c_void_p, C.c_char_p]
L.cfg_destroy.argtypes = [C.c_void_p]
L.abn_write_header.argtypes = [C.c_void_p, C.c_size_t, C.c_char_p, C.c_void_p]

CASES = {
    "plain": b"# a comment\nNmodes = 500\ncellfile = cells.abn\n\nmodel = RealModel\n",
    "whitespace": b"   # indented comment\n\t key\t=\tvalue with  spaces \t\n"
                  b"crlf = dos\r\nvt\x0b= \x0cformfeed\x0c\nkey with space = x\n",
    "quotes": b"q1 = \"  padded  \"\nq2 = 'single'\nq3 = \"unbalanced\nq4 = \"\"\nq5 = ''\nq6 = \"a\"b\"\n"
              b"q7 = \"x'\n",
    "values": b"empty =\nblank =    \nab = b=c\nnum = 1e-5\ndup = 1\ndup = 2\nZeta = upper\nalpha = lower\n",
    "stop": b"first = 1\nsecond = 2\nthis line is not key value\nthird = 3\n",
    "stop_eq": b"a = 1\n = no key\nb = 2\n",
}


def ref_read(text):
    fd, src = tempfile.mkstemp()
    os.write(fd, text)
    os.close(fd)
    fd, dst = tempfile.mkstemp()
    os.close(fd)
    cfg = L.cfg_new()
    L.cfg_read_file(cfg, src.encode())
    f = libc.fopen(dst.encode(), b"wb")
    L.abn_write_header(f, 0, b"d", cfg)
    libc.fclose(f)
    L.cfg_destroy(cfg)
    out = open(dst, "rb").read()
    os.remove(src)
    os.remove(dst)
    return out


def main():
    out = {}
    for name, text in CASES.items():
        out[name + "_in"] = np.frombuffer(text, dtype=np.uint8)
        out[name + "_out"] = np.frombuffer(ref_read(text), dtype=np.uint8)
        print(name, out[name + "_out"].tobytes())
    np.savez_compressed(os.path.join(HERE, "cfg_ref.npz"), **out)


if __name__ == "__main__":
    main()
