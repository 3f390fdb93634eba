"""Configuration checks of opsec_gpu_create.  The configuration is parsed before the device
is touched, so these run without a GPU: every out-of-range or unknown value is refused with
OPSEC_ERR_CONFIG and a message naming the key; a valid configuration gets past the parser
(OPSEC_OK on a GPU host, a CUDA error without one)."""
import ctypes as C
import os

import pytest

from opsec_gpu import api, build, synth


@pytest.fixture(scope="module")
def create():
    build.build()
    L = api.load()

    def run(text):
        h = C.c_void_p()
        rc = L.opsec_gpu_create(C.byref(h), text.encode())
        msg = L.opsec_gpu_last_error(h).decode() if h else ""
        L.opsec_gpu_destroy(h)
        return rc, msg

    return run


def _base(coordsys=1):
    if coordsys == 1:
        sv, _ = synth.box_survey(4)
    else:
        sv = synth.Survey(2, (200.0, 1000.0, -1.0, 1.0, 0.0, 6.283185307179586), (4, 4, 8))
    return api.make_config(sv, bands=synth.band_edges(2, 0.0, 0.2))


CONFIG = -1
BAD = [
    ("klt.solver = lanczos", "klt.solver"),
    ("klt.degree = 0", "klt.degree"),
    ("klt.tol = -1", "klt.tol"),
    ("klt.gemm = tf32", "klt.gemm"),
    ("klt.tile = 64", "klt.tile"),
    ("klt.fp64 = f64", "klt.fp64"),
    ("klt.qr = lq", "klt.qr"),
    ("klt.refine = -1", "klt.refine"),
    ("sig.gauss = 7", "sig.gauss"),
    ("azimuthal.split = 17", "azimuthal.split"),
    ("azimuthal.gemm = f16", "azimuthal.gemm"),
    ("azimuthal.gemm = tf32", "azimuthal.gemm"),
    ("cubature.window_bins = 8", "cubature.window_bins"),
    ("cubature.symmetry = half", "cubature.symmetry"),
    ("basis.samples = 0", "basis.samples"),
    ("xi.n1 = 0", "xi table layout"),
    ("projection.chunk = 0", "projection.chunk"),
    ("projection.wait_cycles = 1000", "projection.wait_cycles"),
    ("projection.wait_cycles = soon", "projection.wait_cycles"),
    ("azimuthal.eig = lapack", "azimuthal.eig"),
    ("projection.arc_tables = 2", "projection.arc_tables"),
    ("cubature.log_keys = yes", "cubature.log_keys"),
    ("cubature.order = random", "cubature.order"),
    ("azimuthal.transform = cols", "azimuthal.transform"),
    ("azimuthal.overlap = yes", "azimuthal.overlap"),
]


@pytest.mark.parametrize("line,key", BAD)
def test_bad_values_are_refused(create, line, key):
    rc, msg = create(_base() + line + "\n")
    assert rc == CONFIG and key in msg, (rc, msg)


def test_survey_type_is_required(create):
    rc, msg = create("")
    assert rc == CONFIG and "survey.type" in msg


@pytest.mark.parametrize("coordsys", [1, 2])
def test_valid_configurations_pass_the_parser(create, coordsys):
    text = _base(coordsys)
    for extra in ("", "klt.solver = chfsi\nklt.gemm = f32\nklt.degree = 6\n", "klt.gemm = tc\nklt.tile = 256\n",
                  "klt.gemm = bf16x9\nklt.tile = auto\nklt.fp64 = native\nklt.qr = householder\n", "mixing = inverse-sqrt\n",
                  "solver = parpack\n", "azimuthal.eig = own\nprojection.wait_cycles = 20000000\n",
                  "azimuthal.eig = batched\n"):
        rc, msg = create(text + extra)
        assert rc in (api.OK, -3), (rc, msg)  # -3: OPSEC_ERR_CUDA, no device on this host


def test_parser_rules_of_the_library(create):
    """The library reads key = value lines as cfg_read_line does (C isspace trimmed, quotes
    stripped, the last value kept) and refuses a text with a line that is not key = value."""
    base = _base()
    # trimmed \t, \v, \f, \r and quotes: these values reach the option checks as '7' and 'tf32'
    for line in ("sig.gauss =\t7\x0c", "\x0b sig.gauss = '7' \r", 'klt.gemm = "tf32"'):
        rc, msg = create(base + line + "\n")
        assert rc == CONFIG and ("sig.gauss" in msg or "klt.gemm" in msg), (line, rc, msg)
    # ... and these are valid after trimming and unquoting
    for line in ("mixing = 'inverse'", "sig.gauss\t=\t3\r", "sig.gauss = 9\nsig.gauss = 4"):
        rc, msg = create(base + line + "\n")
        assert rc in (api.OK, -3), (line, rc, msg)
    rc, msg = create(base + "this is not key value\n")
    assert rc == CONFIG and "not a key = value line" in msg


def test_integer_options_read_as_scanf_i(create):
    """Integer options are read as cfg_get_int reads them ("%i", cfg.c:430-440)."""
    base = _base()
    rc, msg = create(base + "sig.gauss = 010\n")  # octal 8: out of range
    assert rc == CONFIG and "sig.gauss" in msg
    for line in ("sig.gauss = 0x3", "sig.gauss = 3 # three points", "sig.gauss = 05"):
        rc, msg = create(base + line + "\n")
        assert rc in (api.OK, -3), (line, rc, msg)
    rc, msg = create(base + "sig.gauss = three\n")
    assert rc == CONFIG and "not an integer" in msg


def test_mixing_is_read_as_cfg_get_enum(create):
    """mixing is cfg_get_enum's (cfg.c:486-501): any prefix of inverse, inverse-sqrt or identity,
    and a value matching none means inverse -- never an error, as in the reference."""
    for v in ("inverse", "inverse-sqrt", "identity", "inv", "inverse-s", "id", "", "bogus"):
        rc, msg = create(_base() + f"mixing = {v}\n")
        assert rc in (api.OK, -3), (v, rc, msg)


def test_band_lists_read_as_cfg_get_array(create):
    """RealModel.bands is read as cfg_get_array_double reads it (space or comma separated,
    empty fields skipped: testcfg.c:55-87); an odd trailing value is dropped (RealModel.cpp:49-52)."""
    L = api.load()
    L.opsec_gpu_num_params.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    sv, _ = synth.box_survey(4)
    for text, nb in (("0 0.1 0.1 0.2", 2), ("0, 0.1, 0.1, 0.2", 2), ("0, 0.1, 0.1, 0.2,", 2),
                     ("0, 0.1, 0.1, 0.2,,", 2), ("0 0.1 0.1", 1)):
        h = C.c_void_p()
        text_cfg = "\n".join(sv.config_lines()) + f"\nmodel = RealModel\nRealModel.bands = {text}\n"
        L.opsec_gpu_create(C.byref(h), text_cfg.encode())
        n = C.c_int(-1)
        rc = L.opsec_gpu_num_params(h, C.byref(n))  # host state: no device needed
        L.opsec_gpu_destroy(h)
        assert rc == api.OK and n.value == nb, (text, rc, n.value)


def test_band_priors_match_reference(tmp_path):
    """Model::GetParam (RealModel.cpp:85-96), the prior estimate reads: the band powers of the
    reference's own RealModel (tests/golden/params_ref.npz, tests/golden/make_params_golden.py)
    against the oracle and against the library, which reads the same pkfile on the host."""
    import numpy as np

    import oracle as O

    G = np.load(os.path.join(os.path.dirname(__file__), "golden", "params_ref.npz"))
    pk = tmp_path / "pk.dat"
    synth.write_pkfile(str(pk), G["pk_k"], G["pk_P"])
    L = api.load()
    L.opsec_gpu_get_params.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    sv, _ = synth.box_survey(4)
    for name in ("c1", "c2", "narrow"):
        nb, kmin, kmax = (float(x) for x in G[f"{name}_bands"])
        nb = int(nb)
        want = G[f"{name}_params"]
        bands = [(kmin + n * (kmax - kmin) / nb, kmin + (n + 1) * (kmax - kmin) / nb) for n in range(nb)]
        np.testing.assert_allclose(O.band_priors(G["pk_k"], G["pk_P"], bands), want, rtol=1e-13)
        text = "\n".join(sv.config_lines()) + (f"\nmodel = RealModel\nRealModel.pkfile = {pk}\n"
                                               f"RealModel.Nbands = {nb}\nRealModel.kmin = {kmin!r}\n"
                                               f"RealModel.kmax = {kmax!r}\n")
        h = C.c_void_p()
        rc = L.opsec_gpu_create(C.byref(h), text.encode())
        assert rc in (api.OK, -3), L.opsec_gpu_last_error(h)  # configuration parsed; -3: no device here
        got = np.zeros(nb)
        rc = L.opsec_gpu_get_params(h, got.ctypes.data_as(C.POINTER(C.c_double)))  # host only
        L.opsec_gpu_destroy(h)
        assert rc == api.OK
        np.testing.assert_allclose(got, want, rtol=1e-13)
