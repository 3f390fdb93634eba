"""Generate tests/golden/galaxy_ref.npz from the reference's own code.

Run where the reference checkout is present (it is absent on GPU hosts):

    make -C oracle ref REF=<checkout>/code/opsec/src   # builds oracle/_ref/libopsecref.so
    python tests/golden/make_galaxy_golden.py

The library is the reference's unmodified sources plus oracle/ref_shim.cpp,
whose ref_count_galaxies bins galaxies as the dot program does
(code/opsec/src/dot.cpp:124-129, Survey::GetGridIndex, Survey.cpp:93-101).
The vectors, for a Cartesian box and a spherical shell grid:

* seeded float32 galaxies (x1, x2, x3, w) spread over the grid and 10 % past
  each side, plus galaxies exactly on the float32 images of the cell edges and
  on the grid's corners;
* the list of cells: a seeded subset of the grid cells that always holds grid
  index 0 and leaves out every grid cell some galaxy falls in only once;
* the reference's grid index of every galaxy and its weighted counts per cell
  (counts[ncells]: galaxies it sends to no cell).  Galaxies that land in a grid
  cell without a cell are dropped before the reference runs (dot.cpp:127
  indexes counts[-1] for them).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libopsecref.so"))
dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


def ref_count(coordsys, grid, n, gals, cellidx):
    grid = np.ascontiguousarray(grid, dtype=np.float64)
    n = np.ascontiguousarray(n, dtype=np.int32)
    gals = np.ascontiguousarray(gals, dtype=np.float32)
    cellidx = np.ascontiguousarray(cellidx, dtype=np.int32)
    index = np.zeros(gals.shape[0], dtype=np.int32)
    counts = np.zeros(cellidx.size + 1)
    L.ref_count_galaxies(C.c_int(coordsys), grid.ctypes.data_as(dp), n.ctypes.data_as(ip), C.c_long(gals.shape[0]),
                         gals.ctypes.data_as(C.c_void_p), C.c_int(cellidx.size), cellidx.ctypes.data_as(ip),
                         index.ctypes.data_as(ip), counts.ctypes.data_as(dp))
    return index, counts


def galaxies(rng, grid, n, count):
    lo, hi = np.asarray(grid[0::2]), np.asarray(grid[1::2])
    span = hi - lo
    x = lo - 0.1 * span + 1.2 * span * rng.random((count, 3))
    edges = []
    for ax in range(3):
        e = lo[ax] + np.arange(n[ax] + 1) * span[ax] / n[ax]
        pts = lo + 0.5 * span + 0.3 * span * (rng.random((e.size, 3)) - 0.5)
        pts[:, ax] = e
        edges.append(pts)
    corners = np.array([[grid[i], grid[2 + j], grid[4 + k]] for i in (0, 1) for j in (0, 1) for k in (0, 1)])
    x = np.concatenate([x] + edges + [corners])
    w = rng.choice([1.0, 0.5, 2.0, 0.37], size=x.shape[0])
    return np.concatenate([x, w[:, None]], axis=1).astype(np.float32)


def case(rng, coordsys, grid, n, count):
    g = galaxies(rng, grid, n, count)
    ncell = int(np.prod(n))
    keep = rng.random(ncell) < 0.7
    keep[0] = True
    index, _ = ref_count(coordsys, grid, n, g, np.arange(ncell))
    # drop galaxies in grid cells without a cell (the reference writes counts[-1] for them)
    ok = (index < 0) | keep[np.maximum(index, 0)]
    g = g[ok]
    cellidx = np.flatnonzero(keep).astype(np.int32)
    index, counts = ref_count(coordsys, grid, n, g, cellidx)
    return dict(grid=np.asarray(grid, float), n=np.asarray(n, np.int32), gals=g, cellidx=cellidx,
                index=index, counts=counts)


def main():
    rng = np.random.default_rng(20261204)
    out = {}
    for name, cs, grid, n in (("box", 1, (0.0, 300.0, 0.0, 300.0, 0.0, 300.0), (4, 5, 6)),
                              ("sph", 2, (200.0, 1000.0, -1.0, 1.0, 0.0, 2 * np.pi), (3, 4, 8))):
        for k, v in case(rng, cs, grid, n, 1500).items():
            out[f"{name}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "galaxy_ref.npz"), **out)
    for k, v in out.items():
        print(k, v.shape, v.dtype)


if __name__ == "__main__":
    main()
