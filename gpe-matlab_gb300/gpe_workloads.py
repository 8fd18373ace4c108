"""Seeded synthetic workloads (the reference publishes no datasets).

Each workload fixes a grid, trap, coupling, particle number, initial state and
time steps.  Where the workload description leaves a value open it is fixed
here and marked ``assumed``:

* "Gaussian width 4" means psi0 = exp(-r^2/(2*4^2)) plus complex noise
  1e-3*(N(0,1) + i N(0,1))/sqrt(2) from numpy's default_rng(seed).
* 3D ITP time steps: the reference's ITP applies the nonlinear factor
  explicitly and oscillates once mu*dt exceeds ~1 (the 256^3 workload at
  dt = 0.02 has mu*dt ~ 1.4 and never meets eps; the FP64 oracle shows the
  same), so 0.01 (256^3, mu ~ 71) and 0.004 (512^3, mu ~ 180) are used,
  with eps = 1e-6.

The parameter tables, potentials and seeded start states here import
nothing of the library: the CPU reference timing builds its grids (the
oracle's), potentials and start states from them without loading libgpe.so.
Only the factories that build library grids and tasks (``make_grid``,
``make_task``, ``make_tasks``) import ``gpe_gb300``, when they are called.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def _grids():
    from gpe_gb300.grid import grid2d, grid3d

    return grid2d, grid3d


@dataclass
class Workload:
    name: str
    ndims: int
    n: tuple
    box: tuple                      # xmax, ymax[, zmax]
    trap: tuple                     # anisotropy (1, 1[, lambda])
    g: float
    Ntotal: float
    itp_dt: float
    itp_eps: float
    dt: float
    niter_inner: int
    niter_outer: int
    gamma: float = 0.0
    vortex_x0: float | None = None
    ring_frac: float | None = None  # vortex ring radius / R_TF
    sigma: float = 4.0
    noise: float = 1e-3
    seed: int = 1
    notes: list = field(default_factory=list)

    @property
    def npoints(self) -> int:
        return int(np.prod(self.n))

    def make_grid(self, precision: str = "double", n=None):
        grid2d, grid3d = _grids()
        n = tuple(n or self.n)
        if self.ndims == 2:
            return grid2d(self.box[0], n[0], self.box[1], n[1], precision=precision)
        return grid3d(self.box[0], n[0], self.box[1], n[1], self.box[2], n[2], precision=precision)

    def potential(self):
        lam = self.trap

        def V(X, Y, Z):
            if self.ndims == 2:
                return 0.5 * ((lam[0] * X) ** 2 + (lam[1] * Y) ** 2)
            return 0.5 * ((lam[0] * X) ** 2 + (lam[1] * Y) ** 2 + (lam[2] * Z) ** 2)

        return V

    def initial_state(self, grid):
        rng = np.random.default_rng(self.seed)
        X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
        r2 = X ** 2 + Y ** 2 + (Z ** 2 if self.ndims == 3 else 0.0)
        phi = np.exp(-r2 / (2 * self.sigma ** 2)).astype(np.complex128)
        noise = (rng.standard_normal(grid.shape) + 1j * rng.standard_normal(grid.shape)) / np.sqrt(2)
        return phi + self.noise * noise

    def make_task(self, precision: str = "double", n=None, device: int = 0):
        from gpe_gb300.task import GPEtask

        grid = self.make_grid(precision, n)
        task = GPEtask(grid, self.potential(), device=device)
        task.Ntotal = self.Ntotal
        task.g = self.g
        task.gamma = self.gamma
        return grid, task


# Plain-method 2D example: 256^2, box [-17, 17]^2, V = 0.5 r^2, N = 1e5, g = 0.06,
# ITP 0.02 / 1e-6 from a Gaussian, vortex at x0 = 5, then 20 x 50 steps of 0.004.
VORTEX2D = Workload(
    name="vortex2d_256", ndims=2, n=(256, 256), box=(17.0, 17.0), trap=(1.0, 1.0), g=0.06, Ntotal=1e5,
    itp_dt=0.02, itp_eps=1e-6, dt=0.004, niter_inner=50, niter_outer=20, vortex_x0=5.0)

# 3D 256^3, box +-12, V = 0.5 (x^2 + y^2 + (4 z)^2), g = 0.5, N = 1e5; ITP
# then 2000 steps of 0.002 with gamma = 0.01 (20 outer x 100 inner).
DAMPED3D = Workload(
    name="damped3d_256", ndims=3, n=(256, 256, 256), box=(12.0, 12.0, 12.0), trap=(1.0, 1.0, 4.0), g=0.5,
    Ntotal=1e5, itp_dt=0.01, itp_eps=1e-6, dt=0.002, niter_inner=100, niter_outer=20, gamma=0.01,
    notes=["ITP dt 0.01 and eps 1e-6 assumed (dt 0.02 oscillates)"])

# 3D 512^3, lambda = (1, 1, 2), g = 1, N = 1e6, vortex ring at 0.5 R_TF,
# 10000 steps of 0.001.  Box +-24 assumed (TF radius ~18.9 in x, y).
RING3D = Workload(
    name="ring3d_512", ndims=3, n=(512, 512, 512), box=(24.0, 24.0, 24.0), trap=(1.0, 1.0, 2.0), g=1.0,
    Ntotal=1e6, itp_dt=0.004, itp_eps=1e-6, dt=0.001, niter_inner=100, niter_outer=100, ring_frac=0.5,
    notes=["box +-24 assumed", "ITP dt 0.004 and eps 1e-6 assumed"])

WORKLOADS = {w.name: w for w in (VORTEX2D, DAMPED3D, RING3D)}


@dataclass
class BatchWorkload:
    """Many independent 2D realisations of uneven sizes, advanced together.

    Sizes uniform in {128^2, 192^2, 256^2, 384^2}, trap V = 0.5 (x^2 + (lam y)^2)
    with lam ~ U(1, 2), g ~ U(0.02, 0.2), and 1-3 vortices at seeded positions
    within 0.6 of the Thomas-Fermi radii; 5000 steps of dt = 0.004.  Assumed:
    box +-16, Ntotal = 2e4, ITP dt = 0.01 (mu*dt <= 0.5), 100 steps per outer step.
    """

    name: str = "batch2d_64"
    count: int = 64
    sizes: tuple = (128, 192, 256, 384)
    box: float = 16.0
    Ntotal: float = 2e4
    itp_dt: float = 0.01
    itp_eps: float = 1e-6
    dt: float = 0.004
    steps: int = 5000
    niter_inner: int = 100
    seed: int = 3

    def realisations(self):
        rng = np.random.default_rng(self.seed)
        out = []
        for _ in range(self.count):
            n = int(rng.choice(self.sizes))
            lam = float(rng.uniform(1.0, 2.0))
            g = float(rng.uniform(0.02, 0.2))
            nv = int(rng.integers(1, 4))
            out.append({"n": n, "lam": lam, "g": g, "nv": nv, "u": rng.random((nv, 2))})
        return out

    @property
    def npoints(self) -> int:
        return int(sum(r["n"] ** 2 for r in self.realisations()))

    def shard(self, rank: int = 0, world: int = 1):
        """Realisation indices of one rank: the independent realisations are
        dealt round-robin over the ranks (no exchange between them)."""
        return list(range(rank, self.count, world))

    def make_tasks(self, precision: str = "single", device: int = 0, rank: int = 0, world: int = 1):
        """Tasks of this rank's realisations, holding their ground state with
        the vortices imprinted."""
        from gpe_gb300.imprint import imprint_vortex
        from gpe_gb300.task import GPEtask

        grid2d, _ = _grids()
        tasks = []
        rs = self.realisations()
        for r in (rs[i] for i in self.shard(rank, world)):
            grid = grid2d(self.box, r["n"], self.box, r["n"], precision=precision)
            lam = r["lam"]
            task = GPEtask(grid, lambda X, Y, Z, lam=lam: 0.5 * (X ** 2 + (lam * Y) ** 2), device=device)
            task.Ntotal, task.g = self.Ntotal, r["g"]
            X, Y = grid.mesh["x"], grid.mesh["y"]
            phi0 = np.exp(-(X ** 2 + (lam * Y) ** 2) / 32.0).astype(np.complex128)
            phi = np.asarray(task.groundstate_itp(self.itp_dt, self.itp_eps, phi0, nargout=2)[0],
                             dtype=np.complex128)
            rx = np.sqrt(2.0 * task.current_mu)
            ry = rx / lam
            for u1, u2 in r["u"]:
                rad, th = 0.6 * np.sqrt(u1), 2.0 * np.pi * u2
                phi = imprint_vortex(grid, phi, r["g"], rad * rx * np.cos(th), rad * ry * np.sin(th))
            task.init_state = phi
            task.current_iter = 0
            tasks.append(task)
        return tasks


BATCH2D = BatchWorkload()


@dataclass
class AdjointWorkload:
    """Gradient of an overlap loss through gamma = 0 split steps.

    256^2, V = 0.5 r^2 + sum_{j=1..16} a_j exp(-|r - c_j|^2 / 2) with
    a_j ~ N(0, 0.1) and c_j uniform in the Thomas-Fermi disc (seed 4), 2000
    steps of 0.002 with checkpoints every 50; loss 1 - |<target|psi(T)>|^2 with
    the target a vortex imprinted at x0 = 3.  Assumed: box +-17, g = 0.06,
    Ntotal = 1e5 (the 2D vortex example's values); psi0 and the target's base
    are the ground state of 0.5 r^2 alone (ITP dt 0.02, eps 1e-6), so the 16
    bumps drive the dynamics whose dloss/da_j is measured.
    """

    name: str = "adjoint2d_256"
    n: int = 256
    box: float = 17.0
    g: float = 0.06
    Ntotal: float = 1e5
    nbumps: int = 16
    a_sigma: float = 0.1
    dt: float = 0.002
    steps: int = 2000
    checkpoint_every: int = 50
    vortex_x0: float = 3.0
    itp_dt: float = 0.02
    itp_eps: float = 1e-6
    seed: int = 4

    def make_grid(self, precision: str = "single", n=None):
        grid2d, _ = _grids()
        n = n or self.n
        return grid2d(self.box, n, self.box, n, precision=precision)

    def bumps(self, grid, mu_tf=None):
        """(a, basis): a_j and the 16 Gaussians exp(-|r - c_j|^2 / 2) on grid."""
        rng = np.random.default_rng(self.seed)
        a = rng.normal(0.0, self.a_sigma, self.nbumps)
        mu = mu_tf if mu_tf is not None else np.sqrt(self.g * self.Ntotal / np.pi)  # 2D TF, V = r^2/2
        R = np.sqrt(2.0 * mu)
        rad = R * np.sqrt(rng.random(self.nbumps))
        th = 2.0 * np.pi * rng.random(self.nbumps)
        X, Y = grid.mesh["x"], grid.mesh["y"]
        basis = [np.exp(-((X - r * np.cos(t)) ** 2 + (Y - r * np.sin(t)) ** 2) / 2.0) for r, t in zip(rad, th)]
        return a, basis

    def trap(self, grid):
        X, Y = grid.mesh["x"], grid.mesh["y"]
        return 0.5 * (X ** 2 + Y ** 2)


ADJOINT2D = AdjointWorkload()


@dataclass
class SpinorWorkload:
    """Coherently coupled two-component dynamics (GPEtaskSpinor.solve_split)
    on the damped 3D grid: 256^3, box +-12, V1 = 0.5 (x^2 + y^2 + (4 z)^2),
    V2 = V1 with the trap centre moved to x = 0.5, g = [[0.5, 0.45],
    [0.45, 0.5]], Rabi coupling 0.5, Ntotal = 1e5, gamma = 0.01, 100 steps of
    0.002 per outer step (n_recalc = 10).  Start: the one-component ITP
    ground state of the damped workload split 70/30 between the components
    (component 2 with a phase 0.3).  All values are assumed: the reference
    names no spinor workload."""

    name: str = "spinor3d_256"
    n: tuple = (256, 256, 256)
    box: float = 12.0
    lam_z: float = 4.0
    shift2: float = 0.5
    g: tuple = ((0.5, 0.45), (0.45, 0.5))
    coupling: complex = 0.5
    Ntotal: float = 1e5
    gamma: float = 0.01
    dt: float = 0.002
    niter_inner: int = 100
    frac1: float = 0.7

    @property
    def npoints(self) -> int:
        return int(np.prod(self.n))

    def potentials(self):
        lz = self.lam_z
        s = self.shift2
        return [lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2 + (lz * Z) ** 2),
                lambda X, Y, Z: 0.5 * ((X - s) ** 2 + Y ** 2 + (lz * Z) ** 2)]

    def initial_pair(self, phi):
        phi = np.asarray(phi, dtype=np.complex128)
        return [np.sqrt(self.frac1) * phi, np.sqrt(1.0 - self.frac1) * np.exp(0.3j) * phi]

    def configure(self, task):
        task.g = np.array(self.g)
        task.coupling = self.coupling
        task.Ntotal = self.Ntotal
        task.gamma = self.gamma
        return task

    def make_task(self, precision: str = "single", device: int = 0):
        from gpe_gb300.task import GPEtaskSpinor

        _, grid3d = _grids()
        b, n = self.box, self.n
        grid = grid3d(b, n[0], b, n[1], b, n[2], precision=precision)
        return grid, self.configure(GPEtaskSpinor(grid, self.potentials(), device=device))


SPINOR3D = SpinorWorkload()
