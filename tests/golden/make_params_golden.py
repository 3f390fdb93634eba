"""Generate tests/golden/params_ref.npz: the band powers of the reference's RealModel::GetParam.

Run where the reference checkout is present (it is absent on GPU hosts):

    make -C oracle ref REF=<checkout>/code/opsec/src   # builds oracle/_ref/libopsecref.so
    python tests/golden/make_params_golden.py

P(k) is the benchmark spectrum tabulated as a pkfile (opsec_gpu.synth.write_pkfile, 17
significant digits), read by the reference's own CubicSpline; the bands are the regular
Nbands / kmin / kmax ones of RealModel.cpp:60-70 and GetParam averages P over 256 midpoints
of each (RealModel.cpp:85-96).  Stored: the pk table and the priors per case.
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from opsec_gpu import synth  # noqa: E402

L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libopsecref.so"))
L.ref_band_params.argtypes = [C.c_char_p, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double)]


def main():
    k, P = synth.pk_table()
    fd, pkfile = tempfile.mkstemp(suffix=".dat")
    os.close(fd)
    synth.write_pkfile(pkfile, k, P)
    out = {"pk_k": k, "pk_P": P}
    for name, nb, kmin, kmax in (("c1", 20, 0.0, 0.2), ("c2", 40, 0.0, 0.4), ("narrow", 7, 0.013, 0.05)):
        v = np.zeros(nb)
        assert L.ref_band_params(pkfile.encode(), nb, kmin, kmax, v.ctypes.data_as(C.POINTER(C.c_double))) == 0
        out[f"{name}_bands"] = np.array([nb, kmin, kmax])
        out[f"{name}_params"] = v
        print(name, v[:3])
    os.remove(pkfile)
    np.savez_compressed(os.path.join(HERE, "params_ref.npz"), **out)


if __name__ == "__main__":
    main()
