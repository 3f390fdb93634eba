"""Small survey configurations shared by the GPU parity tests."""
import math

import numpy as np

from opsec_gpu import synth


def partial_sky():
    """Spherical grid on part of the sky (phi range < 2 pi): dense eigensolve path."""
    sv = synth.Survey(synth.COORD_SPHERICAL, (200.0, 1000.0, -0.5, 0.8, 0.3, 2.0), (3, 3, 5))

    def nbar(r, mu, phi):
        return 3e-4 * np.exp(-(((r - 600.0) / 250.0) ** 2))

    return sv, synth.make_cells(sv, nbar, nquad=12)


def cases():
    return {
        "box4": synth.box_survey(4, side=200.0, scale=100.0),
        "box4open": synth.box_survey(4, side=200.0, scale=100.0, periodic=False),
        "sph_full": synth.shell_survey(3, 4, 8),
        "sph_part": partial_sky(),
    }
