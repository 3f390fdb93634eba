"""numpy restatement of the GPU mock counts -- TEST INFRASTRUCTURE ONLY.

Only tests/ may import this module.  It restates, step by step and with the
same random streams, what opsec_gpu_mock_counts does on the GPU:

  Philox4x64-10        Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
                       easy as 1, 2, 3" (SC 2011); pinned against numpy's own
                       numpy.random.Philox in tests/test_mock.py
  Box-Muller           two normals per pair of uniforms
  field                white noise -> rfftn -> x sqrt(P(|k|) / V) n^1.5 -> irfftn
                       (the Gaussian random field of the mock generator,
                       code/opsec/utils/gmock.cpp:1-40, drawn from white noise)
  counts               Poisson(Nbar (1 + b delta)^+): CDF inversion below 10,
                       PTRS (Hoermann 1993, "The transformed rejection method for
                       generating Poisson random variables") above
"""
from __future__ import annotations

import math

import numpy as np

M0, M1 = np.uint64(0xD2E7470EE14C6C93), np.uint64(0xCA5A826395121157)
W0, W1 = np.uint64(0x9E3779B97F4A7C15), np.uint64(0xBB67AE8584CAA73B)
NOISE_STREAM = 0x6E6F697365
POISSON_STREAM = 0x706F6973
MAX_ATTEMPTS = 64
_M32 = np.uint64(0xFFFFFFFF)
_S32 = np.uint64(32)


def _mulhilo(a, b):
    al, ah = a & _M32, a >> _S32
    bl, bh = b & _M32, b >> _S32
    ll, lh, hl, hh = al * bl, al * bh, ah * bl, ah * bh
    mid = (ll >> _S32) + (lh & _M32) + (hl & _M32)
    return hh + (lh >> _S32) + (hl >> _S32) + (mid >> _S32), a * b


def philox4x64(c0, c1, c2, c3, k0, k1):
    """Philox4x64-10 of counters (c0..c3) (uint64 arrays) under key (k0, k1)."""
    c0, c1, c2, c3 = (np.asarray(x, np.uint64) for x in (c0, c1, c2, c3))
    k0, k1 = np.uint64(k0), np.uint64(k1)
    with np.errstate(over="ignore"):
        for r in range(10):
            if r:
                k0 = k0 + W0
                k1 = k1 + W1
            hi0, lo0 = _mulhilo(M0, c0)
            hi1, lo1 = _mulhilo(M1, c2)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return c0, c1, c2, c3


def u01(x):
    return (np.asarray(x, np.uint64) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def white_noise(n, seed):
    npts = n ** 3
    t = np.arange((npts + 3) // 4, dtype=np.uint64)
    z = np.zeros_like(t)
    o = philox4x64(t, z, z, z, seed, NOISE_STREAM)
    ra = np.sqrt(-2.0 * np.log(1.0 - u01(o[0])))
    pa = 2.0 * math.pi * u01(o[1])
    rb = np.sqrt(-2.0 * np.log(1.0 - u01(o[2])))
    pb = 2.0 * math.pi * u01(o[3])
    v = np.stack([ra * np.cos(pa), ra * np.sin(pa), rb * np.cos(pb), rb * np.sin(pb)], axis=1).ravel()
    return v[:npts].reshape(n, n, n)


def field(n, box, seed, pk):
    """pk: callable P(k) (the context's cubic spline, zero outside its table)."""
    kf = 2 * math.pi / box
    fx = np.fft.fftfreq(n, d=1.0 / n)
    fz = np.fft.rfftfreq(n, d=1.0 / n)
    FX, FY, FZ = np.meshgrid(fx, fx, fz, indexing="ij")
    kk = kf * np.sqrt(FX ** 2 + FY ** 2 + FZ ** 2)
    P = np.asarray(pk(kk.ravel())).reshape(kk.shape)
    amp = np.sqrt(P / box ** 3) * n ** 1.5
    amp[0, 0, 0] = 0.0
    return np.fft.irfftn(np.fft.rfftn(white_noise(n, seed)) * amp, s=(n, n, n), axes=(0, 1, 2))


def mesh_index(coordsys, cells, n):
    """Mesh point of each cell centre and the mesh side (as the engine computes them)."""
    c1 = 0.5 * (cells["min1"] + cells["max1"])
    c2 = 0.5 * (cells["min2"] + cells["max2"])
    c3 = 0.5 * (cells["min3"] + cells["max3"])
    if coordsys == 2:
        st = np.sqrt(np.fmax(1.0 - c2 * c2, 0.0))
        xyz = np.stack([c1 * st * np.cos(c3), c1 * st * np.sin(c3), c1 * c2], axis=1)
    else:
        xyz = np.stack([c1, c2, c3], axis=1)
    lo = xyz.min(axis=0) - 1.0
    span = float((xyz.max(axis=0) - lo).max())
    box = (span + 1.0) * 1.25
    h = box / n
    m = np.floor((xyz - lo) / h).astype(np.int64) % n
    return (m[:, 0] * n + m[:, 1]) * n + m[:, 2], box


def poisson(lam, cell, seed):
    if not lam > 0.0:
        return 0
    if lam < 10.0:
        o = philox4x64([cell], [0], [0], [0], seed, POISSON_STREAM)
        u = u01(o[0])[0]
        k, p = 0, math.exp(-lam)
        F = p
        while u > F and k < 1000:
            k += 1
            p *= lam / k
            F += p
        return k
    slam, loglam = math.sqrt(lam), math.log(lam)
    b = 0.931 + 2.53 * slam
    a = -0.059 + 0.02483 * b
    invalpha = 1.1239 + 1.1328 / (b - 3.4)
    vr = 0.9277 - 3.6224 / (b - 2.0)
    for j in range(MAX_ATTEMPTS):
        o = philox4x64([cell], [j + 1], [0], [0], seed, POISSON_STREAM)
        U = u01(o[0])[0] - 0.5
        V = u01(o[1])[0]
        us = 0.5 - abs(U)
        k = math.floor((2.0 * a / us + b) * U + lam + 0.43)
        if us >= 0.07 and V <= vr:
            return k
        if k < 0 or (us < 0.013 and V > us):
            continue
        if math.log(V) + math.log(invalpha) - math.log(a / (us * us) + b) <= -lam + k * loglam - math.lgamma(k + 1.0):
            return k
    return math.floor(lam)


def mock_counts(coordsys, cells, n, seed, bias, pk):
    idx, box = mesh_index(coordsys, cells, n)
    f = field(n, box, seed, pk).ravel()
    delta = f[idx]
    lam = np.fmax(cells["Nbar"] * (1.0 + bias * delta), 0.0)
    counts = np.array([poisson(float(l), a, seed) for a, l in enumerate(lam)], dtype=np.float64)
    return counts, delta
