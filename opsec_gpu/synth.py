"""Seeded synthetic inputs for the Fisher-build path: cells, P(k), counts.

The reference reads its inputs from files made by other programs: cells from
``basis`` (code/opsec/src/basis.cpp:89-201), the prior power spectrum from a
two-column ``pkfile`` (code/opsec/src/RealModel.cpp:33-40) and galaxy counts
per cell from ``dot`` (code/opsec/src/dot.cpp:120-135).  No survey data ships
with it, so the workloads here are generated from fixed seeds with the
shapes and distributions of the benchmark configurations:

* Cartesian box, side 600 Mpc/h, 12^3 cells, n(r) = 3e-4 exp(-(r/300)^2)
  about the box centre, 20 bands of width 0.01 h/Mpc on [0, 0.2];
* spherical shell r in [200, 1000] Mpc/h on an Nr x Nmu x Nphi grid over
  the full sky, n(r) proportional to exp(-((r-600)/250)^2) normalised so
  that the mean expected count is 3e-4 times the mean cell volume, 40 bands
  on [0, 0.4];
* P(k) = 2e4 k / (1 + (k/0.02)^2)^1.5 tabulated on k in (0, 10].

Expected counts Nbar are the exact integral of n over each cell (the
reference's ``basis`` over-counts spherical cells by 3 because it drops the
1/3 of the r^3 Jacobian, basis.cpp:72-84; that is not reproduced).
"""
from __future__ import annotations

import math

import numpy as np

CELL_DTYPE = np.dtype(
    [
        ("a", "<i4"), ("d1", "<i4"), ("d2", "<i4"), ("d3", "<i4"),
        ("min1", "<f8"), ("max1", "<f8"), ("min2", "<f8"), ("max2", "<f8"),
        ("min3", "<f8"), ("max3", "<f8"), ("Veff", "<f8"), ("Nbar", "<f8"),
    ]
)
assert CELL_DTYPE.itemsize == 80  # the reference's Cell, "4i8d" (Cell.h:74-99)

COORD_CARTESIAN = 1
COORD_SPHERICAL = 2


def pk_model(k):
    """P(k) = 2e4 k / (1 + (k/0.02)^2)^1.5 (h^-3 Mpc^3)."""
    k = np.asarray(k, dtype=np.float64)
    return 2e4 * k / (1.0 + (k / 0.02) ** 2) ** 1.5


def pk_table(n: int = 2001, kmin: float = 1e-4, kmax: float = 10.0):
    """Tabulated P(k) on log-spaced k in [kmin, kmax], as a pkfile holds it."""
    k = np.exp(np.linspace(math.log(kmin), math.log(kmax), n))
    k[-1] = kmax
    return k, pk_model(k)


def write_pkfile(path, k, P):
    with open(path, "w") as f:
        f.write("# k P(k)\n")
        for a, b in zip(k, P):
            f.write(f"{a:.17g} {b:.17g}\n")


class Survey:
    """Grid geometry of a survey, mirroring the reference Survey fields
    (code/opsec/src/Survey.h:56-72)."""

    def __init__(self, coordsys, bounds, n, L=0.0):
        self.coordsys = coordsys
        self.bounds = tuple(float(x) for x in bounds)  # Min1,Max1,Min2,Max2,Min3,Max3
        self.n = tuple(int(x) for x in n)  # N1,N2,N3
        self.L = float(L)  # periodic box size (Cartesian); 0 = open box

    @property
    def ncells_grid(self):
        return self.n[0] * self.n[1] * self.n[2]

    def full_sky(self):
        return self.coordsys == COORD_SPHERICAL and abs(self.bounds[5] - self.bounds[4] - 2 * math.pi) < 1e-12

    def config_lines(self):
        """key=value lines in the reference's configuration vocabulary."""
        b, n = self.bounds, self.n
        if self.coordsys == COORD_CARTESIAN:
            lines = ["coordsys = cartesian", "survey.type = BoxSurvey", f"survey.L = {self.L!r}",
                     "survey.nbar = 1", "survey.galfile = none"]
            names = ["XMin", "XMax", "YMin", "YMax", "ZMin", "ZMax"]
            ns = ["Nx", "Ny", "Nz"]
        else:
            lines = ["coordsys = spherical", "survey.type = SphericalSurvey",
                     "survey.galfile = none", "survey.maskfile = none", "survey.radial = none"]
            names = ["RMin", "RMax", "MuMin", "MuMax", "PhiMin", "PhiMax"]
            ns = ["Nr", "Nmu", "Nphi"]
        for k, v in zip(names, b):
            lines.append(f"survey.{k} = {v!r}")
        # the reference reads MuMin from "MuMuin" (Survey.cpp:39); write both
        if self.coordsys == COORD_SPHERICAL:
            lines.append(f"survey.MuMuin = {b[2]!r}")
        for k, v in zip(ns, n):
            lines.append(f"survey.{k} = {v}")
        return lines


def _gauss01(n):
    x, w = np.polynomial.legendre.leggauss(n)
    return 0.5 * (x + 1.0), 0.5 * w


def _grid_edges(lo, hi, n):
    d = np.arange(n + 1, dtype=np.float64)
    # same arithmetic as Survey::CreateEmptyCell (Survey.cpp:80-97)
    return lo + d * (hi - lo) / n


def make_cells(survey: Survey, nbar_fn, nquad: int = 48):
    """All grid cells with Nbar = integral of n over the cell.

    nbar_fn(x1, x2, x3) evaluates the selection function in the survey's
    coordinates (vectorised)."""
    N1, N2, N3 = survey.n
    b = survey.bounds
    cells = np.zeros(N1 * N2 * N3, dtype=CELL_DTYPE)
    e1 = _grid_edges(b[0], b[1], N1)
    e2 = _grid_edges(b[2], b[3], N2)
    e3 = _grid_edges(b[4], b[5], N3)
    d1, d2, d3 = np.meshgrid(np.arange(N1), np.arange(N2), np.arange(N3), indexing="ij")
    d1, d2, d3 = d1.ravel(), d2.ravel(), d3.ravel()
    cells["a"] = np.arange(cells.size)
    cells["d1"], cells["d2"], cells["d3"] = d1, d2, d3
    cells["min1"], cells["max1"] = e1[d1], e1[d1 + 1]
    cells["min2"], cells["max2"] = e2[d2], e2[d2 + 1]
    cells["min3"], cells["max3"] = e3[d3], e3[d3 + 1]
    if survey.coordsys == COORD_CARTESIAN:
        cells["Veff"] = (cells["max1"] - cells["min1"]) * (cells["max2"] - cells["min2"]) * (cells["max3"] - cells["min3"])
    else:
        cells["Veff"] = (cells["max1"] ** 3 - cells["min1"] ** 3) / 3.0 * (cells["max2"] - cells["min2"]) * (
            cells["max3"] - cells["min3"])
    u, w = _gauss01(nquad)
    nb = np.empty(cells.size)
    for a in range(cells.size):
        c = cells[a]
        x1 = c["min1"] + u * (c["max1"] - c["min1"])
        x2 = c["min2"] + u * (c["max2"] - c["min2"])
        x3 = c["min3"] + u * (c["max3"] - c["min3"])
        X1, X2, X3 = np.meshgrid(x1, x2, x3, indexing="ij")
        W = w[:, None, None] * w[None, :, None] * w[None, None, :]
        f = nbar_fn(X1, X2, X3)
        if survey.coordsys == COORD_SPHERICAL:
            f = f * X1 ** 2
        vol = (c["max1"] - c["min1"]) * (c["max2"] - c["min2"]) * (c["max3"] - c["min3"])
        nb[a] = vol * np.sum(W * f)
    cells["Nbar"] = nb
    return cells


def box_survey(n: int = 12, side: float = 600.0, n0: float = 3e-4, scale: float = 300.0, periodic: bool = True):
    """Cartesian box with a Gaussian selection about its centre."""
    sv = Survey(COORD_CARTESIAN, (0, side, 0, side, 0, side), (n, n, n), L=side if periodic else 0.0)
    c = side / 2

    def nbar(x, y, z):
        r2 = (x - c) ** 2 + (y - c) ** 2 + (z - c) ** 2
        return n0 * np.exp(-r2 / scale ** 2)

    return sv, make_cells(sv, nbar)


def tilted_box_survey(n: int, side: float, periodic: bool = False, n0: float = 3e-4):
    """Cartesian box with an off-centre, anisotropic Gaussian selection: no symmetry of the grid
    survives in S, so its eigenvalues are not degenerate."""
    sv = Survey(COORD_CARTESIAN, (0.0, side, 0.0, side, 0.0, side), (n, n, n), L=side if periodic else 0.0)

    def sel(x, y, z):
        q = (x - 0.42 * side) ** 2 + 1.3 * (y - 0.57 * side) ** 2 + 0.8 * (z - 0.5 * side) ** 2 + 0.2 * x * y
        return n0 * np.exp(-q / (0.5 * side) ** 2)

    return sv, make_cells(sv, sel, nquad=4)


def shell_survey(nr: int = 32, nmu: int = 32, nphi: int = 32, rmin: float = 200.0, rmax: float = 1000.0,
                 rc: float = 600.0, width: float = 250.0, mean_density: float = 3e-4, nquad: int = 24):
    """Full-sky spherical shell with a Gaussian radial selection.

    Nbar depends on (r, mu) cells only through r, so every arc of fixed
    (r, mu) holds Nphi cells with equal Nbar."""
    sv = Survey(COORD_SPHERICAL, (rmin, rmax, -1.0, 1.0, 0.0, 2 * math.pi), (nr, nmu, nphi))
    # radial integral per r-shell, then replicate over (mu, phi)
    u, w = _gauss01(nquad)
    edges = _grid_edges(rmin, rmax, nr)
    shell = np.empty(nr)
    for i in range(nr):
        r = edges[i] + u * (edges[i + 1] - edges[i])
        shell[i] = (edges[i + 1] - edges[i]) * np.sum(w * r * r * np.exp(-((r - rc) / width) ** 2))
    cells = np.zeros(nr * nmu * nphi, dtype=CELL_DTYPE)
    d1, d2, d3 = np.meshgrid(np.arange(nr), np.arange(nmu), np.arange(nphi), indexing="ij")
    d1, d2, d3 = d1.ravel(), d2.ravel(), d3.ravel()
    e2 = _grid_edges(-1.0, 1.0, nmu)
    e3 = _grid_edges(0.0, 2 * math.pi, nphi)
    cells["a"] = np.arange(cells.size)
    cells["d1"], cells["d2"], cells["d3"] = d1, d2, d3
    cells["min1"], cells["max1"] = edges[d1], edges[d1 + 1]
    cells["min2"], cells["max2"] = e2[d2], e2[d2 + 1]
    cells["min3"], cells["max3"] = e3[d3], e3[d3 + 1]
    cells["Veff"] = (cells["max1"] ** 3 - cells["min1"] ** 3) / 3.0 * (cells["max2"] - cells["min2"]) * (
        cells["max3"] - cells["min3"])
    nb = shell[d1] * (cells["max2"] - cells["min2"]) * (cells["max3"] - cells["min3"])
    nb *= mean_density * cells["Veff"].mean() / nb.mean()
    cells["Nbar"] = nb
    return sv, cells


def band_edges(nbands: int, kmin: float, kmax: float):
    """Linearly spaced top-hat bands, RealModel.cpp:60-70."""
    n = np.arange(nbands)
    lo = kmin + n * (kmax - kmin) / nbands
    hi = kmin + (n + 1) * (kmax - kmin) / nbands
    return np.stack([lo, hi], axis=1)


def cell_centres_xyz(survey: Survey, cells):
    c1 = 0.5 * (cells["min1"] + cells["max1"])
    c2 = 0.5 * (cells["min2"] + cells["max2"])
    c3 = 0.5 * (cells["min3"] + cells["max3"])
    if survey.coordsys == COORD_CARTESIAN:
        return np.stack([c1, c2, c3], axis=1)
    s = np.sqrt(np.clip(1 - c2 * c2, 0, None))
    return np.stack([c1 * s * np.cos(c3), c1 * s * np.sin(c3), c1 * c2], axis=1)


def grf_counts(survey: Survey, cells, seed_field: int = 1, seed_poisson: int = 2, ngrid: int = 64):
    """Counts N_a ~ Poisson(Nbar_a (1 + delta_a)) with delta a Gaussian random
    field of the benchmark P(k), sampled at the cell centres.

    The field is drawn on a periodic ngrid^3 mesh enclosing the survey
    (seed_field) and the Poisson draws use seed_poisson."""
    xyz = cell_centres_xyz(survey, cells)
    lo = xyz.min(axis=0) - 1.0
    span = float((xyz.max(axis=0) - lo).max()) + 1.0
    box = span * 1.25
    h = box / ngrid
    rng = np.random.default_rng(seed_field)
    kf = 2 * math.pi / box
    kx = np.fft.fftfreq(ngrid, d=1.0 / ngrid) * kf
    kz = np.fft.rfftfreq(ngrid, d=1.0 / ngrid) * kf
    KX, KY, KZ = np.meshgrid(kx, kx, kz, indexing="ij")
    kk = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    amp = np.sqrt(pk_model(kk) / box ** 3) * ngrid ** 3
    amp[0, 0, 0] = 0.0
    noise = rng.standard_normal((ngrid, ngrid, ngrid))
    field = np.fft.irfftn(np.fft.rfftn(noise) / ngrid ** 1.5 * amp, s=(ngrid, ngrid, ngrid), axes=(0, 1, 2))
    idx = np.floor((xyz - lo) / h).astype(np.int64) % ngrid
    delta = field[idx[:, 0], idx[:, 1], idx[:, 2]]
    lam = np.clip(cells["Nbar"] * (1.0 + delta), 0.0, None)
    return np.random.default_rng(seed_poisson).poisson(lam).astype(np.float64)


def mock_batch(n: int, seed: int = 5, nmu: int = 16, nphi: int = 16, ncells_range=(2000, 20000)):
    """Independent full-sky shells with their own Gaussian radial selections:
    N_s ~ U[ncells_range], centre ~ U[300, 900], width ~ U[100, 300] (Mpc/h);
    grid nr x nmu x nphi with nr = N_s / (nmu nphi) (at least 8), r in
    [max(20, centre - 2 width), centre + 2 width]; counts are Poisson draws of
    Nbar; nmodes = Ncells / 4.  Returns a list of dicts for Engine.batch_fisher."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        ns = rng.uniform(*ncells_range)
        rc = rng.uniform(300.0, 900.0)
        width = rng.uniform(100.0, 300.0)
        nr = max(8, int(round(ns / (nmu * nphi))))
        rmin, rmax = max(20.0, rc - 2 * width), rc + 2 * width
        sv, cells = shell_survey(nr, nmu, nphi, rmin=rmin, rmax=rmax, rc=rc, width=width, nquad=8)
        counts = rng.poisson(cells["Nbar"]).astype(np.float64)
        out.append({"survey": sv, "rmin": rmin, "rmax": rmax, "nr": nr, "nmu": nmu, "nphi": nphi, "cells": cells,
                    "counts": counts, "nmodes": cells.size // 4, "centre": rc, "width": width})
    return out
