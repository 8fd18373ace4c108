"""Phase imprints on host FP64 states (one-off, negligible cost).

``imprint_vortex`` is the recipe of examples/example1_vortex.m:26-30 (and
README.md:93-97) of GPE-MATLAB, with the same atan2 argument order.
``imprint_vortex_ring`` is its 3D analogue for a ring in the z = z0 plane.
"""
from __future__ import annotations

import math

import numpy as np


def healing_length(phi, g) -> float:
    """xi = 1/sqrt(2 g max|psi|^2) (example1_vortex.m:26)."""
    return 1.0 / math.sqrt(2 * g * float(np.max(np.abs(phi))) ** 2)


def imprint_vortex(grid, phi, g, x0, y0=0.0, charge=1, xi=None):
    """psi * tanh(r/xi) * exp(i*charge*atan2(X - x0, Y - y0)).

    The atan2 argument order (X first) follows example1_vortex.m:29.
    """
    xi = healing_length(phi, g) if xi is None else xi
    X, Y = grid.mesh["x"], grid.mesh["y"]
    rr = np.sqrt((X - x0) ** 2 + (Y - y0) ** 2)
    angs = np.arctan2(X - x0, Y - y0)
    return phi * np.tanh(rr / xi) * np.exp(1j * charge * angs)


def imprint_vortex_ring(grid, phi, g, radius, z0=0.0, xi=None):
    """Vortex ring of the given radius around the z axis in the plane z = z0.

    Amplitude tanh(d/xi) with d the distance to the ring core, phase
    atan2(Z - z0, rho - radius) winding once around the core.
    """
    xi = healing_length(phi, g) if xi is None else xi
    X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
    rho = np.sqrt(X ** 2 + Y ** 2)
    d = np.sqrt((rho - radius) ** 2 + (Z - z0) ** 2)
    ang = np.arctan2(Z - z0, rho - radius)
    return phi * np.tanh(d / xi) * np.exp(1j * ang)
