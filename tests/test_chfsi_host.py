"""Host-side numerics of the iterative eigensolver (opsec_gpu/csrc/chfsi_host.h), compiled
from the same header on the CPU: Lanczos-tridiagonal eigenvalues by Sturm bisection against
LAPACK, the block size, and the Chebyshev degree rule against the closed form of T_d."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("chfsi") / "libchfsi_host_check.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                           os.path.join(HERE, "chfsi_host_check.cpp")])
    L = C.CDLL(so)
    dp = C.POINTER(C.c_double)
    L.chk_tridiag_eig.argtypes = [C.c_int, dp, dp, C.c_int]
    L.chk_tridiag_eig.restype = C.c_double
    L.chk_sturm_count.argtypes = [C.c_int, dp, dp, C.c_double]
    L.chk_block_size.argtypes = [C.c_int, C.c_int, C.c_int]
    L.chk_filter_degree.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double]
    L.chk_max_gain.restype = C.c_double
    return L


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


def test_tridiagonal_eigenvalues_match_lapack(lib):
    rng = np.random.default_rng(7)
    for n in (1, 2, 5, 32):
        for _ in range(5):
            a = rng.standard_normal(n) * rng.uniform(0.1, 10)
            b = rng.standard_normal(max(n - 1, 0)) * rng.uniform(0.01, 3)
            T = np.diag(a) + np.diag(b, 1) + np.diag(b, -1)
            ev = np.linalg.eigvalsh(T)
            scale = np.max(np.abs(ev))
            for k in range(n):
                got = lib.chk_tridiag_eig(n, _d(a), _d(b), k)
                assert abs(got - ev[k]) <= 1e-12 * scale, (n, k, got, ev[k])
            for x in np.linspace(ev[0] - 1, ev[-1] + 1, 9):
                if np.min(np.abs(ev - x)) > 1e-9 * scale:
                    assert lib.chk_sturm_count(n, _d(a), _d(b), x) == int(np.sum(ev < x))


def test_lanczos_bounds_enclose_the_spectrum(lib):
    """32 Lanczos steps on a covariance-like matrix: theta_max + |beta_k| lies above lambda_max
    and the extreme Ritz values inside the spectrum (the bounds the filter uses)."""
    rng = np.random.default_rng(3)
    n = 400
    x = np.sort(rng.uniform(0, 100, n))
    S = np.exp(-((x[:, None] - x[None, :]) / 8.0) ** 2) * np.outer(rng.uniform(0.5, 2, n), np.ones(n))
    S = 0.5 * (S + S.T)
    lam = np.linalg.eigvalsh(S)
    v = rng.uniform(-1, 1, n)
    v /= np.linalg.norm(v)
    v0 = np.zeros(n)
    al, be, beta = [], [], 0.0
    for j in range(32):
        w = S @ v
        a = w @ v
        w -= a * v + beta * v0
        al.append(a)
        beta = np.linalg.norm(w)
        if j == 31:
            break
        be.append(beta)
        v0, v = v, w / beta
    tmin = lib.chk_tridiag_eig(32, _d(al), _d(be), 0)
    tmax = lib.chk_tridiag_eig(32, _d(al), _d(be), 31)
    assert lam[0] - 1e-9 <= tmin and tmax <= lam[-1] + 1e-9
    assert tmax + abs(beta) >= lam[-1]


def test_block_size(lib):
    assert lib.chk_block_size(1728, 200, 50) == 256
    assert lib.chk_block_size(1728, 500, 125) == 640
    assert lib.chk_block_size(100, 90, 32) == 100      # capped at N
    assert lib.chk_block_size(10000, 1, 0) == 32       # at least 8 guard vectors, multiple of 32
    for N, M, g in ((13824, 500, 125), (64000, 1000, 250), (4096, 4000, 32)):
        B = lib.chk_block_size(N, M, g)
        assert M <= B <= N and (B % 32 == 0 or B == N)


def _cheb(d, t):
    t = max(t, 1.0)
    return np.cosh(d * np.arccosh(t))


def test_filter_degree_rule(lib):
    gain = lib.chk_max_gain()
    assert gain == 1e4
    rng = np.random.default_rng(5)
    for _ in range(200):
        lo = -rng.uniform(0, 0.05)
        cut = rng.uniform(0.001, 0.5)
        hi = cut * rng.uniform(1.01, 1e3)
        tm = cut + (hi - cut) * rng.uniform(0, 1) ** 3
        dmax = int(rng.integers(1, 24))
        d = lib.chk_filter_degree(lo, cut, hi, tm, dmax, gain)
        e, c = 0.5 * (cut - lo), 0.5 * (cut + lo)
        ok = [k for k in range(2, dmax + 1) if _cheb(k, (hi - c) / e) / max(_cheb(k, (tm - c) / e), 1.0) <= gain]
        assert d == (max(ok) if ok else 1)
        assert 1 <= d <= dmax
    # a narrow wanted spectrum allows the full degree; a wide one forces degree 1
    assert lib.chk_filter_degree(0.0, 1.0, 1.5, 1.4, 12, gain) == 12
    assert lib.chk_filter_degree(0.0, 1e-3, 10.0, 1.1e-3, 12, gain) == 1
