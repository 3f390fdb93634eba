"""Generate tests/golden/basis_ref.npz from the reference's own code.

Run where the reference checkout is present (it is absent on GPU hosts):

    make -C oracle ref REF=<checkout>/code/opsec/src   # builds oracle/_ref/libopsecref.so
    python tests/golden/make_basis_golden.py

The library is the reference's unmodified sources plus oracle/ref_shim.cpp;
chealpix.c is compiled against oracle/fitsio_stub/fitsio.h (its map file
readers fail, its pixelisation is the reference's).  The vectors:

* HEALPix pixels of seeded random (theta, phi) by ang2pix_ring / ang2pix_nest
  (chealpix.c:100-246) for several nside, plus points on the poles, the
  equator, the cap boundaries z = +-2/3 and phi = 0;
* the cell builder: Veff and Nbar of every cell by FinalizeCell (basis.cpp:89-128,
  adaptive cubature, epsrel 1e-5) of the constant selection on a 3x3x3 box and of
  the radial-spline x HEALPix-map selection (SphericalSurvey.cpp:51-80) on
  spherical grids, without a map and with seeded maps in both orderings.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libopsecref.so"))
dp = C.POINTER(C.c_double)


def _d(a):
    return a.ctypes.data_as(dp)


def ang2pix(nside, nest, theta, phi):
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    out = np.zeros(theta.size, dtype=np.int64)
    L.ref_ang2pix(C.c_long(nside), C.c_int(nest), C.c_int(theta.size), _d(theta), _d(phi),
                  out.ctypes.data_as(C.POINTER(C.c_long)))
    return out


def basis(coordsys, grid, n, nbar=0.0, rad=None, nside=0, nest=0, mask=None):
    grid = np.ascontiguousarray(grid, dtype=np.float64)
    n = np.ascontiguousarray(n, dtype=np.int32)
    rr, rn = (np.zeros(2), np.zeros(2)) if rad is None else (np.ascontiguousarray(rad[0], float),
                                                               np.ascontiguousarray(rad[1], float))
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
    out = np.zeros(3 * int(np.prod(n)))
    L.ref_basis(C.c_int(coordsys), _d(grid), n.ctypes.data_as(C.POINTER(C.c_int)), C.c_double(nbar),
                C.c_int(rr.size), _d(rr), _d(rn), C.c_long(nside), C.c_int(nest),
                None if m is None else m.ctypes.data_as(C.c_void_p), _d(out))
    return out.reshape(-1, 3)


def main():
    rng = np.random.default_rng(20261203)
    out = {}
    # HEALPix: random directions plus special ones
    z = rng.uniform(-1, 1, 3000)
    theta = np.arccos(z)
    phi = rng.uniform(0, 2 * np.pi, 3000)
    special_t = np.array([0.0, np.pi, np.pi / 2, np.arccos(2 / 3), np.arccos(-2 / 3), 1e-9, np.pi - 1e-9, 0.3])
    special_p = np.array([0.0, 0.0, 0.0, 1.0, 2.0, 3.0, 4.0, 2 * np.pi - 1e-12])
    theta = np.concatenate([theta, special_t])
    phi = np.concatenate([phi, special_p])
    out["hp_theta"], out["hp_phi"] = theta, phi
    for nside in (1, 2, 4, 16, 256, 8192):
        out[f"hp_ring_{nside}"] = ang2pix(nside, 0, theta, phi)
        out[f"hp_nest_{nside}"] = ang2pix(nside, 1, theta, phi)
    # cell builder, Cartesian constant selection
    out["box_grid"] = np.array([0.0, 600.0, 0.0, 600.0, 0.0, 600.0])
    out["box_n"] = np.array([3, 3, 3])
    out["box_nbar"] = np.array([3e-4])
    out["box_out"] = basis(1, out["box_grid"], out["box_n"], nbar=3e-4)
    # spherical: radial spline, no map (one knot beyond each end of the shell, zero at the outer edge)
    rr = np.linspace(150.0, 1100.0, 12)
    rn = 3e-4 * np.exp(-((rr - 600.0) / 250.0) ** 2)
    rn[-1] = 0.0
    out["rad_r"], out["rad_n"] = rr, rn
    out["sph_grid"] = np.array([200.0, 1000.0, -1.0, 1.0, 0.0, 2 * np.pi])
    out["sph_n"] = np.array([4, 4, 8])
    out["sph_out"] = basis(2, out["sph_grid"], out["sph_n"], rad=(rr, rn))
    # spherical with maps (nside 2, seeded completeness in [0, 1], some pixels empty)
    mask = rng.uniform(0.0, 1.0, 48).astype(np.float32)
    mask[rng.choice(48, 10, replace=False)] = 0.0
    out["map"] = mask
    out["map_grid"] = np.array([200.0, 1000.0, -1.0, 1.0, 0.0, 2 * np.pi])
    out["map_n"] = np.array([2, 3, 4])
    out["map_ring_out"] = basis(2, out["map_grid"], out["map_n"], rad=(rr, rn), nside=2, nest=0, mask=mask)
    out["map_nest_out"] = basis(2, out["map_grid"], out["map_n"], rad=(rr, rn), nside=2, nest=1, mask=mask)
    np.savez_compressed(os.path.join(HERE, "basis_ref.npz"), **out)


if __name__ == "__main__":
    main()
