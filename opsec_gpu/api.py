"""Python binding of the C ABI (include/opsec_gpu.h) over ctypes.

The names follow the reference programs and routines they replace:
``klt`` (code/opsec/src/klt.cpp), ``comma`` (comma-scalapack.cpp), ``dot``
(dot.cpp), ``estimate`` (estimate-mpi.cpp) and ``signal_block``
(ComputeSignalMatrixBlock, sig.cpp:50-70).  Errors raise OpsecError with the
library's status code; there is no CPU fallback -- a missing library raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .synth import CELL_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libopsec_gpu.so")

OK = 0
ERR_ARG, ERR_CUDA, ERR_NOMEM = -2, -3, -4
ERR = {-1: "CONFIG", -2: "ARG", -3: "CUDA", -4: "NOMEM", -5: "FILE", -6: "NUMERIC", -7: "STATE"}
MIXING = {"inverse": 0, "inverse-sqrt": 1, "identity": 2}
STAGES = ("xi_tables", "cubature", "eigensolve", "projection", "fisher")

_lib = None


class OpsecError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"OPSEC_ERR_{ERR.get(code, code)}: {msg}")
        self.code = code


def load():
    """Load libopsec_gpu.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m opsec_gpu.build`")
    L = C.CDLL(LIB_PATH)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.opsec_gpu_create.argtypes = [C.POINTER(vp), C.c_char_p]
    L.opsec_gpu_set_pk.argtypes = [vp, C.c_int, dp, dp]
    L.opsec_gpu_set_xi_table.argtypes = [vp, C.c_int, C.c_int, dp]
    L.opsec_gpu_num_params.argtypes = [vp, ip]
    L.opsec_gpu_get_params.argtypes = [vp, dp]
    L.opsec_gpu_xi_tables.argtypes = [vp, ip, dp, dp]
    L.opsec_gpu_signal_block.argtypes = [vp, C.c_int, vp, C.c_int, ip, C.c_int, ip, dp, C.c_int, C.c_int]
    L.opsec_gpu_klt.argtypes = [vp, C.c_int, vp, C.c_int, dp, dp, ip]
    L.opsec_gpu_comma.argtypes = [vp, C.c_int, vp, C.c_int, dp, dp]
    L.opsec_gpu_dot.argtypes = [vp, C.c_int, vp, dp, C.c_int, dp, dp]
    L.opsec_gpu_estimate.argtypes = [vp, C.c_int, dp, dp, dp, C.c_int] + [dp] * 7
    L.opsec_gpu_fisher_build.argtypes = [vp, C.c_int, vp, dp, C.c_int, C.c_int] + [dp] * 8
    L.opsec_gpu_stage_times.argtypes = [vp, dp]
    L.opsec_gpu_kernel_stats.argtypes = [vp, C.c_char_p, C.POINTER(C.c_longlong), dp, dp, dp]
    L.opsec_gpu_eig_stats.argtypes = [vp, dp]
    L.opsec_gpu_launch_count.argtypes = [vp]
    L.opsec_gpu_launch_count.restype = C.c_longlong
    L.opsec_gpu_last_error.argtypes = [vp]
    L.opsec_gpu_last_error.restype = C.c_char_p
    L.opsec_gpu_destroy.argtypes = [vp]
    fp = C.POINTER(C.c_float)
    L.opsec_gpu_surrogate_train.argtypes = [vp, C.c_longlong, C.c_int, C.c_uint, dp]
    L.opsec_gpu_surrogate_size.argtypes = []
    L.opsec_gpu_surrogate_weights.argtypes = [vp, fp, C.c_int]
    L.opsec_gpu_surrogate_stats.argtypes = [vp, C.POINTER(C.c_longlong)]
    L.opsec_gpu_surrogate_eval.argtypes = [vp, fp, C.c_int, fp, fp, fp, fp, dp, fp]
    L.opsec_gpu_batch_fisher.argtypes = [vp, C.c_int, vp, C.c_int, dp, dp, dp, dp]
    L.opsec_gpu_mock_counts.argtypes = [vp, C.c_int, vp, C.c_int, C.c_ulonglong, C.c_double, dp, dp]
    L.opsec_gpu_set_radial.argtypes = [vp, C.c_int, dp, dp]
    L.opsec_gpu_count_galaxies.argtypes = [vp, C.c_int, vp, C.c_longlong, C.POINTER(C.c_float), dp, dp]
    L.opsec_gpu_set_mask.argtypes = [vp, C.c_longlong, C.c_int, C.POINTER(C.c_float)]
    L.opsec_gpu_basis.argtypes = [vp, C.c_int, vp, ip]
    L.opsec_gpu_ang2pix.argtypes = [vp, C.c_longlong, C.c_int, C.c_int, dp, dp, C.POINTER(C.c_longlong)]
    L.opsec_gpu_fail_alloc.argtypes = [vp, C.c_longlong]
    L.opsec_gpu_wait_probe.argtypes = [vp, C.c_longlong, C.c_int, C.c_longlong, ip]
    L.opsec_gpu_block_product.argtypes = [vp, C.c_int, C.c_int, dp, fp, C.c_float, C.c_float, fp, C.c_float, fp]
    _lib = L
    return L


def _d(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int))


class Mock(C.Structure):
    """opsec_mock: one full-sky spherical survey of a batch."""
    _fields_ = [("rmin", C.c_double), ("rmax", C.c_double), ("nr", C.c_int), ("nmu", C.c_int), ("nphi", C.c_int),
                ("ncells", C.c_int), ("cells", C.c_void_p), ("counts", C.c_void_p), ("nmodes", C.c_int)]


def _fp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _cells(cells):
    c = np.ascontiguousarray(cells)
    if c.dtype != CELL_DTYPE:
        raise TypeError("cells must use opsec_gpu.synth.CELL_DTYPE (the reference Cell layout)")
    return c


def make_config(survey, bands=None, nbands=None, kmin=None, kmax=None, nmodes=None, pkfile=None, layout=None,
                gauss=None, mixing=None, extra=()):
    """key = value text in the reference's configuration vocabulary."""
    lines = list(survey.config_lines())
    lines.append("model = RealModel")
    if pkfile:
        lines.append(f"RealModel.pkfile = {pkfile}")
    if bands is not None:
        lines.append("RealModel.bands = " + " ".join(f"{float(lo)!r} {float(hi)!r}" for lo, hi in bands))
    else:
        lines += [f"RealModel.Nbands = {int(nbands)}", f"RealModel.kmin = {float(kmin)!r}",
                  f"RealModel.kmax = {float(kmax)!r}"]
    if nmodes is not None:
        lines.append(f"Nmodes = {nmodes}")
    if layout is not None:
        n1, n2, r1, r2 = layout
        lines += [f"xi.n1 = {int(n1)}", f"xi.n2 = {int(n2)}", f"xi.r1 = {float(r1)!r}", f"xi.r2 = {float(r2)!r}"]
    if gauss is not None:
        lines.append(f"sig.gauss = {gauss}")
    if mixing is not None:
        lines.append(f"mixing = {mixing}")
    lines += list(extra)
    return "\n".join(lines) + "\n"


class Engine:
    """One GPU context (the current CUDA device)."""

    def __init__(self, cfg_text: str):
        self._L = load()
        self._h = C.c_void_p()
        rc = self._L.opsec_gpu_create(C.byref(self._h), cfg_text.encode())
        if rc != OK:
            msg = self._L.opsec_gpu_last_error(self._h).decode() if self._h else ""
            self._L.opsec_gpu_destroy(self._h)
            self._h = None
            raise OpsecError(rc, msg)

    def _check(self, rc):
        if rc != OK:
            raise OpsecError(rc, self._L.opsec_gpu_last_error(self._h).decode())

    def close(self):
        if self._h:
            self._L.opsec_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- model
    def set_pk(self, k, P):
        k, P = _f64(k), _f64(P)
        self._check(self._L.opsec_gpu_set_pk(self._h, k.size, _d(k), _d(P)))

    def num_params(self):
        n = C.c_int()
        self._check(self._L.opsec_gpu_num_params(self._h, C.byref(n)))
        return n.value

    def get_params(self):
        p = np.zeros(self.num_params())
        self._check(self._L.opsec_gpu_get_params(self._h, _d(p)))
        return p

    def xi_tables(self):
        n = C.c_int()
        self._check(self._L.opsec_gpu_xi_tables(self._h, C.byref(n), None, None))
        r = np.zeros(n.value)
        xi = np.zeros((1 + self.num_params(), n.value))
        self._check(self._L.opsec_gpu_xi_tables(self._h, C.byref(n), _d(r), _d(xi)))
        return r, xi

    def set_xi_table(self, table, values):
        v = _f64(values)
        self._check(self._L.opsec_gpu_set_xi_table(self._h, table, v.size, _d(v)))

    # -- the path
    def signal_block(self, cells, rows=None, cols=None, table=0, lld=0):
        cells = _cells(cells)
        rows = np.arange(cells.size, dtype=np.int32) if rows is None else np.ascontiguousarray(rows, dtype=np.int32)
        cols = np.arange(cells.size, dtype=np.int32) if cols is None else np.ascontiguousarray(cols, dtype=np.int32)
        ld = lld if lld > 0 else cols.size
        s = np.zeros((rows.size, ld))
        self._check(self._L.opsec_gpu_signal_block(self._h, cells.size, cells.ctypes.data, rows.size, _i(rows),
                                                   cols.size, _i(cols), _d(s), ld, table))
        return s[:, : cols.size]

    def klt(self, cells, nmodes):
        cells = _cells(cells)
        ev = np.zeros(nmodes)
        modes = np.zeros((nmodes, cells.size))
        nconv = C.c_int()
        self._check(self._L.opsec_gpu_klt(self._h, cells.size, cells.ctypes.data, nmodes, _d(ev), _d(modes),
                                          C.byref(nconv)))
        return ev, modes

    def comma(self, cells, modes):
        cells = _cells(cells)
        modes = _f64(modes)
        M = modes.shape[0]
        out = np.zeros((self.num_params(), M * (M + 1) // 2))
        self._check(self._L.opsec_gpu_comma(self._h, cells.size, cells.ctypes.data, M, _d(modes), _d(out)))
        return out

    def dot(self, cells, counts, modes):
        cells = _cells(cells)
        modes, counts = _f64(modes), _f64(counts)
        y = np.zeros(modes.shape[0])
        self._check(self._L.opsec_gpu_dot(self._h, cells.size, cells.ctypes.data, _d(counts), modes.shape[0],
                                          _d(modes), _d(y)))
        return y

    def count_galaxies(self, cells, gals):
        """Weighted counts per cell of galaxies (n x 4 float32: x1, x2, x3, w); returns (counts, outside)."""
        cells = _cells(cells)
        g = np.ascontiguousarray(gals, dtype=np.float32).reshape(-1, 4)
        counts = np.zeros(cells.size)
        out = np.zeros(1)
        self._check(self._L.opsec_gpu_count_galaxies(self._h, cells.size, cells.ctypes.data, g.shape[0], _fp(g),
                                                     _d(counts), _d(out)))
        return counts, float(out[0])

    def set_radial(self, r, nbar):
        r, nbar = _f64(r), _f64(nbar)
        self._check(self._L.opsec_gpu_set_radial(self._h, r.size, _d(r), _d(nbar)))

    def set_mask(self, nside, nest=False, mask=None):
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
        self._check(self._L.opsec_gpu_set_mask(self._h, int(nside), 1 if nest else 0, _fp(m)))

    def basis(self):
        """Every grid cell with positive Nbar (CELL_DTYPE records, grid order)."""
        from .synth import CELL_DTYPE
        n = C.c_int(0)
        self._check(self._L.opsec_gpu_basis(self._h, 0, None, C.byref(n)))
        cells = np.zeros(n.value, dtype=CELL_DTYPE)
        if n.value:
            self._check(self._L.opsec_gpu_basis(self._h, n.value, cells.ctypes.data, C.byref(n)))
        return cells

    def ang2pix(self, nside, nest, theta, phi):
        theta, phi = _f64(theta), _f64(phi)
        pix = np.zeros(theta.size, dtype=np.int64)
        self._check(self._L.opsec_gpu_ang2pix(self._h, int(nside), 1 if nest else 0, theta.size, _d(theta), _d(phi),
                                              pix.ctypes.data_as(C.POINTER(C.c_longlong))))
        return pix

    def mock_counts(self, cells, ngrid=64, seed=1, bias=1.0, want_delta=False):
        """Poisson counts of a Gaussian random field of this context's P(k) at the cell centres."""
        cells = _cells(cells)
        counts = np.zeros(cells.size)
        delta = np.zeros(cells.size) if want_delta else None
        self._check(self._L.opsec_gpu_mock_counts(self._h, cells.size, cells.ctypes.data, int(ngrid),
                                                  C.c_ulonglong(int(seed)), C.c_double(float(bias)), _d(counts),
                                                  _d(delta)))
        return (counts, delta) if want_delta else counts

    def _records(self):
        nb = self.num_params()
        return {"phat": np.zeros(nb), "pcov": np.zeros((nb, nb)), "F": np.zeros((nb, nb)), "W": np.zeros((nb, nb)),
                "M": np.zeros((nb, nb)), "q": np.zeros(nb), "f": np.zeros(nb)}

    def estimate(self, evals, cov, y, mixing="inverse"):
        evals, cov, y = _f64(evals), _f64(cov), _f64(y)
        r = self._records()
        self._check(self._L.opsec_gpu_estimate(self._h, evals.size, _d(evals), _d(cov), _d(y), MIXING[mixing],
                                               _d(r["phat"]), _d(r["pcov"]), _d(r["F"]), _d(r["W"]), _d(r["M"]),
                                               _d(r["q"]), _d(r["f"])))
        return r

    # ---- learned far-field surrogate
    def surrogate_train(self, max_samples=20_000_000, epochs=4, seed=1):
        """Train the 4-network ensemble on this engine's survey; returns
        samples, validation rms of the residual, seconds and the output scale."""
        st = np.zeros(4)
        self._check(self._L.opsec_gpu_surrogate_train(self._h, int(max_samples), int(epochs), int(seed), _d(st)))
        return {"samples": int(st[0]), "val_rms": st[1], "seconds": st[2], "ysc": st[3]}

    def surrogate_weights(self, weights=None):
        """Without an argument: the ensemble's weights (float32, scale last); with one: load them."""
        n = self._L.opsec_gpu_surrogate_size()
        if weights is None:
            buf = np.zeros(n, dtype=np.float32)
            self._check(self._L.opsec_gpu_surrogate_weights(self._h, _fp(buf), 1))
            return buf
        buf = np.ascontiguousarray(weights, dtype=np.float32)
        if buf.size != n:
            raise ValueError(f"surrogate weights need {n} floats")
        self._check(self._L.opsec_gpu_surrogate_weights(self._h, _fp(buf), 0))

    def surrogate_stats(self):
        out = (C.c_longlong * 3)()
        self._check(self._L.opsec_gpu_surrogate_stats(self._h, out))
        return {"predicted": out[0], "fallback": out[1], "far": out[2]}

    def surrogate_eval(self, params, feats, y=None):
        params = np.ascontiguousarray(params, dtype=np.float32)
        feats = np.ascontiguousarray(feats, dtype=np.float32)
        n = feats.shape[0]
        if feats.shape != (n, 16) or params.size != 35336:
            raise ValueError("params: 35336 floats; feats: n x 16")
        out_tc = np.zeros(n, dtype=np.float32)
        out_simt = np.zeros(n, dtype=np.float32)
        loss = np.zeros(1)
        grad = np.zeros(35336, dtype=np.float32)
        yy = None if y is None else np.ascontiguousarray(y, dtype=np.float32)
        self._check(self._L.opsec_gpu_surrogate_eval(self._h, _fp(params), n, _fp(feats), _fp(yy), _fp(out_tc),
                                                     _fp(out_simt), _d(loss), _fp(grad)))
        return {"out_tc": out_tc, "out_simt": out_simt, "loss": loss[0] if y is not None else None,
                "grad": grad if y is not None else None}

    def batch_fisher(self, mocks, workers=0):
        """mocks: list of dicts (rmin, rmax, nr, nmu, nphi, cells, counts, nmodes).  Returns
        F [n][nb][nb], phat [n][nb], pcov [n][nb][nb] and stats (seconds, workers, autotune rates)."""
        keep = []
        arr = (Mock * len(mocks))()
        for i, m in enumerate(mocks):
            cells = _cells(m["cells"])
            counts = _f64(m["counts"])
            keep += [cells, counts]
            arr[i] = Mock(m["rmin"], m["rmax"], m["nr"], m["nmu"], m["nphi"], cells.size, cells.ctypes.data,
                          counts.ctypes.data, m["nmodes"])
        nb = self.num_params()
        F = np.zeros((len(mocks), nb, nb))
        phat = np.zeros((len(mocks), nb))
        pcov = np.zeros((len(mocks), nb, nb))
        st = np.zeros(8)
        self._check(self._L.opsec_gpu_batch_fisher(self._h, len(mocks), C.cast(arr, C.c_void_p), int(workers), _d(F),
                                                   _d(phat), _d(pcov), _d(st)))
        return {"F": F, "phat": phat, "pcov": pcov, "seconds": st[0], "workers": int(st[1]),
                "autotune_mocks_per_s": {k: st[2 + i] for i, k in enumerate((1, 2, 4, 8, 12, 16))}}

    def fisher_build(self, cells, counts, nmodes, mixing="inverse", want_evals=True):
        cells = _cells(cells)
        counts = _f64(counts)
        r = self._records()
        ev = np.zeros(nmodes) if want_evals else None
        self._check(self._L.opsec_gpu_fisher_build(self._h, cells.size, cells.ctypes.data, _d(counts), nmodes,
                                                   MIXING[mixing], _d(ev), _d(r["phat"]), _d(r["pcov"]), _d(r["F"]),
                                                   _d(r["W"]), _d(r["M"]), _d(r["q"]), _d(r["f"])))
        r["evals"] = ev
        return r

    def stage_times(self):
        t = np.zeros(5)
        self._check(self._L.opsec_gpu_stage_times(self._h, _d(t)))
        return dict(zip(STAGES, t))

    def eig_stats(self):
        """How the last eigensolve ran (opsec_gpu_eig_stats)."""
        t = np.zeros(10)
        self._check(self._L.opsec_gpu_eig_stats(self._h, _d(t)))
        return {"solver": ("dense", "azimuthal", "chfsi")[int(t[0])], "iterations": int(t[1]), "degree": int(t[2]),
                "gemms": int(t[3]), "block": int(t[4]), "lo": t[5], "hi": t[6], "resid": t[7],
                "refine_rounds": int(t[8]), "cg_steps": int(t[9])}

    def kernel_stats(self, name):
        n, ms, fl, by = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
        self._check(self._L.opsec_gpu_kernel_stats(self._h, name.encode(), C.byref(n), C.byref(ms), C.byref(fl),
                                                   C.byref(by)))
        return {"count": n.value, "ms": ms.value, "flops": fl.value, "bytes": by.value}

    def fail_alloc(self, after):
        """Host-side fault injection: the device allocation after `after` more fails (-1: off)."""
        self._check(self._L.opsec_gpu_fail_alloc(self._h, C.c_longlong(after)))

    def wait_probe(self, limit_cycles, arrive=False, delay_cycles=0):
        """Run the projection kernels' bounded wait on a barrier; True when it timed out."""
        out = C.c_int()
        self._check(self._L.opsec_gpu_wait_probe(self._h, C.c_longlong(limit_cycles), int(bool(arrive)),
                                                 C.c_longlong(delay_cycles), C.byref(out)))
        return bool(out.value)

    def block_product(self, S, X, alpha=1.0, beta=0.0, Cin=None, gamma=0.0, D=None):
        """alpha S X + beta Cin + gamma D on the tensor-core block-product kernel of the
        iterative eigensolver: S (N x N, symmetric) FP64, X / Cin / D (N x ncols) FP32."""
        S = np.ascontiguousarray(S, dtype=np.float64)
        N = S.shape[0]
        Xf = np.asfortranarray(X, dtype=np.float32)
        ncols = Xf.shape[1]
        out = np.asfortranarray(Cin if Cin is not None else np.zeros((N, ncols)), dtype=np.float32).copy(order="F")
        Df = None if D is None else np.asfortranarray(D, dtype=np.float32)
        self._check(self._L.opsec_gpu_block_product(self._h, N, ncols, _d(S), _fp(Xf), C.c_float(alpha),
                                                    C.c_float(beta), _fp(out), C.c_float(gamma), _fp(Df)))
        return out

    def launch_count(self):
        return int(self._L.opsec_gpu_launch_count(self._h))
