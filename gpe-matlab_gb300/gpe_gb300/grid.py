"""grid2d / grid3d: uniform periodic grids of GPE-MATLAB (host side).

Mirrors lib/@grid2d/init.m:1-38 and lib/@grid3d/init.m:1-47 of GPE-MATLAB:
``linspace(-xmax, xmax, n)`` axes (or explicit axes), spacing
``dx = x(2) - x(1)``, FFT-ordered wave numbers with period ``x(end)-x(1)+dx``
and integration weight ``prod(dx)``.

Arrays follow MATLAB's memory order (ny x nx [x nz] column-major meshgrid):
here they are C-order numpy arrays of shape (nx, ny) in 2D and (nz, nx, ny)
in 3D, so ``a.ravel()`` is the MATLAB linear order that libgpe reads.

``precision='single'`` corresponds to a grid built from single-precision
gpuArray axes in MATLAB (README.md:106-116): the split step then runs in
complex FP32 on the device, with FP64 reductions.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib as L


def _axis_k(x: np.ndarray) -> np.ndarray:
    n = x.size
    dx = x[1] - x[0]
    idx = np.concatenate([np.arange(0, n // 2 + 1), -np.arange(n // 2 - 1, 0, -1)])
    return idx * 2.0 * np.pi / (x[-1] - x[0] + dx)


class _GridBase:
    ndims = 0

    def _setup(self, axes, precision):
        if precision not in ("single", "double"):
            raise ValueError("precision must be 'single' or 'double'")
        self.precision = precision
        axes = [np.asarray(a, dtype=np.float64).ravel() for a in axes]
        for a in axes:
            if a.size < 2 or a.size % 2:
                raise ValueError("each axis needs an even number (>= 2) of points (init.m:27)")
        self.x, self.y = axes[0], axes[1]
        self.z = axes[2] if len(axes) == 3 else np.zeros(1)
        self.nx, self.ny = self.x.size, self.y.size
        self.nz = self.z.size if len(axes) == 3 else 1
        self.dx = self.x[1] - self.x[0]
        self.dy = self.y[1] - self.y[0]
        self.dz = (self.z[1] - self.z[0]) if len(axes) == 3 else 1.0
        self.kx, self.ky = _axis_k(self.x), _axis_k(self.y)
        self.kz = _axis_k(self.z) if len(axes) == 3 else np.zeros(1)
        if len(axes) == 2:
            X, Y = np.meshgrid(self.x, self.y, indexing="ij")
            self.mesh = {"x": X, "y": Y, "z": 0.0}
            self.weight = self.dx * self.dy
            self.shape = (self.nx, self.ny)
        else:
            Z, X, Y = np.meshgrid(self.z, self.x, self.y, indexing="ij")
            self.mesh = {"x": X, "y": Y, "z": Z}
            self.weight = self.dx * self.dy * self.dz
            self.shape = (self.nz, self.nx, self.ny)
        self.size = self.shape
        self.npoints = int(np.prod(self.shape))

    @property
    def kk(self):
        """|k|^2/2 on the grid (init.m:31); built on demand (P doubles)."""
        if self.ndims == 2:
            KX, KY = np.meshgrid(self.kx, self.ky, indexing="ij")
            return (KX ** 2 + KY ** 2) / 2
        KZ, KX, KY = np.meshgrid(self.kz, self.kx, self.ky, indexing="ij")
        return (KX ** 2 + KY ** 2 + KZ ** 2) / 2

    def desc(self, device: int = 0) -> L.gpe_grid_desc:
        d = L.gpe_grid_desc()
        d.ndims = self.ndims
        axes = [self.x, self.y] + ([self.z] if self.ndims == 3 else [])
        for i, a in enumerate(axes):
            d.n[i] = a.size
            d.dx[i] = a[1] - a[0]
            d.span[i] = a[-1] - a[0]
        d.precision = L.GPE_FP32 if self.precision == "single" else L.GPE_FP64
        d.device = device
        return d

    # lib/@grid1d/integrate.m:11
    def integrate(self, f):
        return np.sum(f) * self.weight

    # lib/@grid1d/inner.m:12
    def inner(self, lhs, rhs):
        return self.integrate(np.conj(lhs) * rhs)

    # lib/@grid1d/norm.m:11
    def norm(self, psi):
        return math.sqrt(self.integrate(np.abs(psi) ** 2))

    # lib/@grid1d/normalize.m:13-15
    def normalize(self, psi):
        return psi * (1.0 / self.norm(psi))


class grid2d(_GridBase):
    """grid2d(xmax, nx, ymax, ny) or grid2d(x, y) (lib/@grid2d/grid2d.m:16-31)."""

    ndims = 2

    def __init__(self, *args, precision: str = "double"):
        if len(args) == 4:
            axes = [np.linspace(-args[0], args[0], int(args[1])), np.linspace(-args[2], args[2], int(args[3]))]
        elif len(args) == 2:
            axes = list(args)
        else:
            raise TypeError("grid2d(xmax, nx, ymax, ny) or grid2d(x, y)")
        self._setup(axes, precision)


class grid3d(_GridBase):
    """grid3d(xmax, nx, ymax, ny, zmax, nz) or grid3d(x, y, z) (lib/@grid3d/grid3d.m)."""

    ndims = 3

    def __init__(self, *args, precision: str = "double"):
        if len(args) == 6:
            axes = [np.linspace(-args[0], args[0], int(args[1])), np.linspace(-args[2], args[2], int(args[3])),
                    np.linspace(-args[4], args[4], int(args[5]))]
        elif len(args) == 3:
            axes = list(args)
        else:
            raise TypeError("grid3d(xmax, nx, ymax, ny, zmax, nz) or grid3d(x, y, z)")
        self._setup(axes, precision)
