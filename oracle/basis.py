"""numpy restatement of the GPU cell builder -- TEST INFRASTRUCTURE ONLY.

Only tests/ may import this module.  It restates what opsec_gpu_basis does,
and the HEALPix pixelisation it uses (Gorski et al. 2005, ApJ 622:759; the
reference calls chealpix.c ang2pix_ring / ang2pix_nest, whose outputs pin
this restatement in tests/test_basis.py through tests/golden/basis_ref.npz):

  cells        Survey::CreateEmptyCell bounds (code/opsec/src/Survey.cpp:80-97)
  Cartesian    Nbar = nbar V (constant selection, BoxSurvey.cpp:61-75)
  spherical    Nbar = int radial(r) r^2 dr (linear spline, closed form per
               segment) x the mean of the map over S x S points of the cell
               x dmu dphi (SphericalSurvey.cpp:51-80); the reference's 3x
               (basis.cpp:72-84, 103-108) with quirk3
  galaxies     grid index per galaxy (Survey::GetGridIndex, Survey.cpp:93-101)
               and weighted counts per cell (dot.cpp:105-129); pinned against
               the reference through tests/golden/galaxy_ref.npz
"""
from __future__ import annotations

import math

import numpy as np


def _spread(v):
    v = np.asarray(v, dtype=np.int64)
    r = np.zeros_like(v)
    for k in range(31):
        r |= ((v >> k) & 1) << (2 * k)
    return r


def ang2pix(nside, nest, theta, phi):
    theta = np.asarray(theta, dtype=np.float64)
    phi = np.array(phi, dtype=np.float64)
    ns = int(nside)
    z = np.cos(theta)
    phi = np.where(phi >= 2 * math.pi, phi - 2 * math.pi, phi)
    phi = np.where(phi < 0, phi + 2 * math.pi, phi)
    tt = phi / (0.5 * math.pi)
    za = np.abs(z)
    eq = za <= 2.0 / 3.0
    out = np.zeros(theta.shape, dtype=np.int64)
    # equatorial belt
    t1 = ns * (0.5 + tt)
    t2 = ns * z * 0.75
    jp = (t1 - t2).astype(np.int64)
    jm = (t1 + t2).astype(np.int64)
    # polar caps
    with np.errstate(invalid="ignore"):
        tmp = np.sqrt(3.0 * (1.0 - za))
    if not nest:
        ir = ns + 1 + jp - jm
        kshift = 1 - (ir & 1)
        ip = (jp + jm - ns + kshift + 1) // 2
        ip = np.where(ip >= 4 * ns, ip - 4 * ns, ip)
        pe = 2 * ns * (ns - 1) + 4 * ns * (ir - 1) + ip
        tp = tt - np.floor(tt)
        cjp = (ns * tp * tmp).astype(np.int64)
        cjm = (ns * (1.0 - tp) * tmp).astype(np.int64)
        cir = cjp + cjm + 1
        cip = (tt * cir).astype(np.int64)
        cip = np.where(cip >= 4 * cir, cip - 4 * cir, cip)
        pc = np.where(z > 0, 2 * cir * (cir - 1) + cip, 12 * ns * ns - 2 * cir * (cir + 1) + cip)
        out = np.where(eq, pe, pc)
        return out
    fp, fm = jp // ns, jm // ns
    face_e = np.where(fp == fm, fp | 4, np.where(fp < fm, fp, fm + 8))
    ix_e = jm % ns
    iy_e = ns - (jp % ns) - 1
    nt = np.minimum(tt.astype(np.int64), 3)
    tp = tt - nt
    cjp = np.minimum((ns * tp * tmp).astype(np.int64), ns - 1)
    cjm = np.minimum((ns * (1.0 - tp) * tmp).astype(np.int64), ns - 1)
    north = z >= 0
    face_c = np.where(north, nt, nt + 8)
    ix_c = np.where(north, ns - cjm - 1, cjp)
    iy_c = np.where(north, ns - cjp - 1, cjm)
    face = np.where(eq, face_e, face_c)
    ix = np.where(eq, ix_e, ix_c)
    iy = np.where(eq, iy_e, iy_c)
    return face * ns * ns + _spread(ix) + 2 * _spread(iy)


def radial_integral(rr, rn, a, b):
    s = 0.0
    for i in range(len(rr) - 1):
        x0, x1 = max(a, rr[i]), min(b, rr[i + 1])
        if not x1 > x0:
            continue
        slope = (rn[i + 1] - rn[i]) / (rr[i + 1] - rr[i])
        c0 = rn[i] - slope * rr[i]
        s += c0 * (x1 ** 3 - x0 ** 3) / 3.0 + slope * (x1 ** 4 - x0 ** 4) / 4.0
    return s


def basis(coordsys, grid, n, nbar=0.0, rad=None, nside=0, nest=0, mask=None, samples=16, quirk3=False):
    """(Veff, Nbar) of every cell in grid order."""
    out = []
    for d1 in range(n[0]):
        for d2 in range(n[1]):
            for d3 in range(n[2]):
                e = []
                for ax, dd in enumerate((d1, d2, d3)):
                    lo, hi = grid[2 * ax], grid[2 * ax + 1]
                    e += [lo + dd * (hi - lo) / n[ax], lo + (dd + 1) * (hi - lo) / n[ax]]
                if coordsys == 1:
                    V = (e[1] - e[0]) * (e[3] - e[2]) * (e[5] - e[4])
                    out.append((V, nbar * V))
                    continue
                dmu, dphi = e[3] - e[2], e[5] - e[4]
                V = (e[1] ** 3 - e[0] ** 3) / 3.0 * dmu * dphi
                R = radial_integral(rad[0], rad[1], e[0], e[1])
                A = dmu * dphi
                if nside and R != 0.0:
                    s = (np.arange(samples) + 0.5) / samples
                    th = np.arccos(e[2] + s * dmu)
                    ph = e[4] + s * dphi
                    TH, PH = np.meshgrid(th, ph, indexing="ij")
                    A *= float(np.mean(np.asarray(mask, dtype=np.float64)[ang2pix(nside, nest, TH, PH)]))
                out.append((V, R * A * (3.0 if quirk3 else 1.0)))
    return np.array(out)


def grid_index(grid, n, gals):
    """Grid index (d1 N2 + d2) N3 + d3 of each galaxy, -1 outside: floor(N (x - min) / (max - min))
    per axis in FP64 from the float32 coordinate, the reference's order of operations."""
    g = np.asarray(gals, dtype=np.float32)
    d = []
    for ax in range(3):
        lo, hi = float(grid[2 * ax]), float(grid[2 * ax + 1])
        with np.errstate(invalid="ignore"):
            d.append(np.floor(int(n[ax]) * (g[:, ax].astype(np.float64) - lo) / (hi - lo)))
    ok = np.ones(g.shape[0], dtype=bool)
    for ax in range(3):
        ok &= (d[ax] >= 0) & (d[ax] < int(n[ax]))
    di = [np.where(ok, x, 0).astype(np.int64) for x in d]
    return np.where(ok, (di[0] * int(n[1]) + di[1]) * int(n[2]) + di[2], -1)


def count_galaxies(grid, n, cellidx, gals, ref_zero=False):
    """Weighted counts per cell (len(cellidx) + 1 values; the last: galaxies in no cell), summed in
    galaxy order.  ref_zero: as the reference, send the galaxies of grid index 0 to the last entry
    (dot.cpp:127 tests e > 0)."""
    g = np.asarray(gals, dtype=np.float32)
    e = grid_index(grid, n, g)
    cellmap = np.full(int(np.prod(n)), -1, dtype=np.int64)
    cellmap[np.asarray(cellidx)] = np.arange(len(cellidx))
    a = np.where(e >= (1 if ref_zero else 0), cellmap[np.maximum(e, 0)], -1)
    a = np.where(a < 0, len(cellidx), a)
    counts = np.zeros(len(cellidx) + 1)
    np.add.at(counts, a, g[:, 3].astype(np.float64))
    return counts
