"""FP64 CPU oracle for the GPE-MATLAB split-step hot path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it.  The product (``libgpe.so`` and its host mirror) never calls it.

It restates, line by line and in FP64 numpy/scipy, the reference's
``GPEtask.groundstate_itp`` / ``GPEtask.solve_split`` on ``grid2d`` /
``grid3d``, with every operation in the reference's order.  Each function
cites the reference file:line it follows (paths relative to the GPE-MATLAB
project root).

PARITY UNPINNED: the reference is MATLAB-only, ships no tests, no golden
vectors and no known-answer fixtures, and neither MATLAB nor Octave exists on
this machine, so the restatement cannot be checked against the reference's own
outputs.  It is instead pinned to analytic known answers (harmonic-oscillator
ground states, exact free propagation of a plane wave, unit-modulus phases at
gamma = 0); see ``tests/test_oracle.py``.

Array layout: MATLAB ``meshgrid`` arrays are ny x nx (x nz), column major, so
the linear index is ``iy + ny*(ix + nx*iz)`` (lib/@grid2d/init.m:30-34,
lib/@grid3d/init.m:75-79).  Here the same memory order is held as C-order numpy
arrays of shape (nx, ny) in 2D and (nz, nx, ny) in 3D: ``a.ravel()`` is the
MATLAB linear order.  FFTs run over every axis, which is what ``fft2`` /
``fftn`` do on the MATLAB array (lib/@grid2d/fft.m:11, lib/@grid3d/fft.m:11).
The third-party FFT arithmetic of the reference is MATLAB's bundled FFTW
(version not pinned by the reference); here it is pocketfft through
``scipy.fft`` with the same conventions (unnormalised forward, 1/N inverse).
"""
from __future__ import annotations

import math
import os
import warnings

import numpy as np
import scipy.fft as sfft

_WORKERS = int(os.environ.get("GPE_ORACLE_WORKERS", os.cpu_count() or 1))


def set_workers(n: int) -> None:
    """Number of threads scipy.fft may use (the CPU baseline uses all cores)."""
    global _WORKERS
    _WORKERS = max(1, int(n))


# ---------------------------------------------------------------------------
# Grids: lib/@grid1d, lib/@grid2d, lib/@grid3d
# ---------------------------------------------------------------------------
def _kvec(x: np.ndarray) -> np.ndarray:
    """FFT-ordered wave numbers, lib/@grid2d/init.m:27 (same rule for y, z)."""
    n = x.size
    dx = x[1] - x[0]
    idx = np.concatenate([np.arange(0, n // 2 + 1), -np.arange(n // 2 - 1, 0, -1)])
    return idx * 2.0 * np.pi / (x[-1] - x[0] + dx)


class Grid:
    """grid2d / grid3d (lib/@grid2d/init.m:1-38, lib/@grid3d/init.m:1-47).

    ``Grid(xmax, nx, ymax, ny)`` or ``Grid(xmax, nx, ymax, ny, zmax, nz)``
    builds ``linspace(-xmax, xmax, n)`` axes (init.m:12-13); explicit axes
    can be given with ``Grid.from_axes(x, y[, z])`` (init.m:5-9).
    """

    def __init__(self, *args):
        if len(args) == 4:
            axes = [np.linspace(-args[0], args[0], int(args[1])),
                    np.linspace(-args[2], args[2], int(args[3]))]
        elif len(args) == 6:
            axes = [np.linspace(-args[0], args[0], int(args[1])),
                    np.linspace(-args[2], args[2], int(args[3])),
                    np.linspace(-args[4], args[4], int(args[5]))]
        else:
            raise ValueError("Grid(xmax,nx,ymax,ny[,zmax,nz])")
        self._init(axes)

    @classmethod
    def from_axes(cls, *axes):
        obj = cls.__new__(cls)
        obj._init([np.asarray(a, dtype=np.float64) for a in axes])
        return obj

    def _init(self, axes):
        self.ndims = len(axes)
        self.x, self.y = axes[0], axes[1]
        self.z = axes[2] if self.ndims == 3 else np.zeros(1)
        self.nx, self.ny = self.x.size, self.y.size
        self.nz = self.z.size if self.ndims == 3 else 1
        # init.m:20-21 / 63-65
        self.dx = self.x[1] - self.x[0]
        self.dy = self.y[1] - self.y[0]
        self.dz = (self.z[1] - self.z[0]) if self.ndims == 3 else 1.0
        kx, ky = _kvec(self.x), _kvec(self.y)
        kz = _kvec(self.z) if self.ndims == 3 else np.zeros(1)
        self.kx1, self.ky1, self.kz1 = kx, ky, kz
        if self.ndims == 2:
            # meshgrid(x, y) -> arrays indexed [ix, iy] here (column-major ny x nx)
            KX, KY = np.meshgrid(kx, ky, indexing="ij")
            self.kk = (KX ** 2 + KY ** 2) / 2                  # init.m:31
            X, Y = np.meshgrid(self.x, self.y, indexing="ij")  # init.m:34
            self.mesh = {"x": X, "y": Y, "z": 0.0}
            self.weight = self.dx * self.dy                    # init.m:36
            self.shape = (self.nx, self.ny)
            self.KX, self.KY, self.KZ = KX, KY, 0.0
            self.axis = {"x": 0, "y": 1}
        else:
            KZ, KX, KY = np.meshgrid(kz, kx, ky, indexing="ij")
            self.kk = (KX ** 2 + KY ** 2 + KZ ** 2) / 2        # grid3d/init.m:76
            Z, X, Y = np.meshgrid(self.z, self.x, self.y, indexing="ij")
            self.mesh = {"x": X, "y": Y, "z": Z}               # grid3d/init.m:79-82
            self.weight = self.dx * self.dy * self.dz          # grid3d/init.m:83
            self.shape = (self.nz, self.nx, self.ny)
            self.KX, self.KY, self.KZ = KX, KY, KZ
            self.axis = {"x": 1, "y": 2, "z": 0}

    # lib/@grid2d/fft.m:11, lib/@grid3d/fft.m:11
    def fft(self, f):
        return sfft.fftn(f, workers=_WORKERS)

    # lib/@grid2d/ifft.m:11, lib/@grid3d/ifft.m:11
    def ifft(self, f):
        return sfft.ifftn(f, workers=_WORKERS)

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

    # lib/@grid2d/fftx.m:11 (dim 2 = x), ffty.m:11 (dim 1 = y),
    # lib/@grid3d/fftz.m:11 (dim 3 = z) and the ifftx/iffty/ifftz files:
    # 1D transforms along one axis, same conventions as fft/ifft.
    def fft1(self, f, ax):
        return sfft.fft(f, axis=self.axis[ax], workers=_WORKERS)

    def ifft1(self, f, ax):
        return sfft.ifft(f, axis=self.axis[ax], workers=_WORKERS)

    # lib/@grid1d/grid1d.m:52-57 (deriv1, stencil1 = [-1, 8, 0, -8, 1]/12):
    # convn(A, stencil/h, 'same') along one axis, zero outside the grid, i.e.
    # (-f(i+2) + 8 f(i+1) - 8 f(i-1) + f(i-2)) / (12 h)
    def deriv1(self, f, ax, h):
        a = self.axis[ax]
        n = f.shape[a]
        pad = [(0, 0)] * f.ndim
        pad[a] = (2, 2)
        g = np.pad(f, pad)

        def sh(k):  # f(i + k) for i = 0..n-1
            return np.take(g, np.arange(2 + k, 2 + k + n), axis=a)

        return (-sh(2) + 8 * sh(1) - 8 * sh(-1) + sh(-2)) / (12 * h)

    # lib/@grid2d/derivx.m:2, derivy.m:2 (both take the spacing obj.dx)
    def derivx(self, f):
        return self.deriv1(f, "x", self.dx)

    def derivy(self, f):
        return self.deriv1(f, "y", self.dx)

    # lib/@grid2d/lz.m:4-8
    def lz(self, phi, r0=(0.0, 0.0)):
        return -1j * ((self.mesh["x"] - r0[0]) * self.derivy(phi) - (self.mesh["y"] - r0[1]) * self.derivx(phi))

    # lib/@grid2d/lap.m:5-10, lib/@grid3d/lap.m:5-11
    def lap(self, phi, omega=0.0):
        if omega == 0:
            return self.ifft(self.kk * self.fft(phi))
        Y, X = self.mesh["y"], self.mesh["x"]
        res = self.ifft1((self.KX ** 2 / 2 - self.KX * Y * omega) * self.fft1(phi, "x"), "x") + \
            self.ifft1((self.KY ** 2 / 2 + self.KY * X * omega) * self.fft1(phi, "y"), "y")
        if self.ndims == 3:
            res = res + self.ifft1((self.KZ ** 2 / 2) * self.fft1(phi, "z"), "z")
        return res


# ---------------------------------------------------------------------------
# Solver: lib/@GPEtask
# ---------------------------------------------------------------------------
class GPEtask:
    """lib/@GPEtask/GPEtask.m:1-167: omega == 0, scalar omega (rotating
    frame) and array omega (the Lz Crank-Nicolson branches)."""

    def __init__(self, grid: Grid, trappot):
        # GPEtask.m:41-60 (rng('shuffle') and the FFTW planner are not numerics)
        self.grid = grid
        self.g = 0.0
        self.omega = 0.0
        self.n_crank = 3
        self.n_recalc = 10
        self.gamma = 0.0
        self.decay_rate = 0.0
        self.Ntotal = 0.0
        self.mu_init = 0.0
        self.Vtd = None
        self.V0 = 0
        self.init_state = np.zeros(grid.shape, dtype=np.complex128)
        self.current_state = None
        self.current_time = 0.0
        self.current_iter = 0
        self.current_mu = 0.0
        self.current_n = 0.0
        self.history = {"mu": [], "n": []}
        self.user_callback = None
        self.itp_max_iter = 5000
        self.itp_min_iter = 50
        self.itp_adjust_stepsize = False
        self.kinop = None
        self.nlinop = None
        if callable(trappot):
            self.Vtrap = trappot(grid.mesh["x"], grid.mesh["y"], grid.mesh["z"])  # :44
        else:
            self.Vtrap = np.asarray(trappot, dtype=np.float64)                  # :46
        self.Vtrap = np.broadcast_to(self.Vtrap, grid.shape).astype(np.float64)

    # GPEtask.m:62-71
    def getVtotal(self, time):
        if time == 0 and np.size(self.V0) > 1:
            return self.V0
        if callable(self.Vtd):
            return self.Vtrap + self.Vtd(self, time)
        return self.Vtrap

    # GPEtask.m:73-78
    def applyham(self, phi, time=None):
        if time is None:
            time = self.current_time
        return self.applyh0(phi, time) + self.g * np.abs(phi) ** 2 * phi

    def _omega_array(self):
        return np.size(self.omega) > 1  # ~isscalar(omega)

    # GPEtask.m:80-95
    def applyh0(self, phi, time=None):
        if time is None:
            time = self.current_time
        res = self.getVtotal(time) * phi
        if not self._omega_array() and self.omega != 0:
            res = res + self.grid.lap(phi, self.omega)
        else:
            res = res + self.grid.lap(phi)
        if self._omega_array():
            res = res - self.omega * self.grid.lz(phi)
        return res

    # GPEtask.m:97-107
    def get_energy(self, phi=None, time=None):
        if phi is None:
            phi = self.current_state
        tmp = self.g
        self.g = 0.5 * self.g
        try:
            res = np.real(self.grid.inner(phi, self.applyham(phi, time)))
        finally:
            self.g = tmp
        return res

    # GPEtask.m:115-142 (plot and console line omitted)
    def ext_callback(self, phi, step, time, mu, n):
        self.current_state = phi
        self.current_time = time
        self.current_iter = step
        self.current_mu = mu
        _set_hist(self.history["mu"], step, mu)
        self.current_n = n
        _set_hist(self.history["n"], step, n)
        res = self.user_callback(self) if callable(self.user_callback) else ""
        return res  # SGPEtask.m:33-43 returns the callback's text; GPEtask's callers ignore it

    # GPEtask.m:144-164
    def process_init_state(self, phi0, rng=None):
        if isinstance(phi0, str):
            if self.Ntotal > 0:
                if phi0 == "tf":
                    res, _ = self.groundstate_tf(np.finfo(float).eps)
                    return res.astype(np.complex128)
                rng = rng or np.random.default_rng()
                r = rng.random(self.grid.shape) + 1j * rng.random(self.grid.shape)
                return math.sqrt(self.Ntotal) * self.grid.normalize(r)
            V = self.getVtotal(0)  # the reference leaves V undefined here (:157)
            return np.real(np.sqrt((self.mu_init - V).astype(np.complex128) / self.g))
        if self.Ntotal > 0:
            return math.sqrt(self.Ntotal) * self.grid.normalize(np.asarray(phi0, np.complex128))
        return np.asarray(phi0, np.complex128)

    # lib/@GPEtask/groundstate_tf.m:1-37
    def groundstate_tf(self, eps, N=None, V=None, mul=None, mur=None):
        if N is None:
            N = self.Ntotal
        if V is None:
            V = self.getVtotal(0)
        if mul is None:
            mul, mur = float(np.min(V)), float(np.max(V))
        NC = N * self.g
        mu = (mul + mur) / 2
        vvv = (mu - V) * (V < mu)
        while (mur - mul) / mu > eps:
            vvv = (mu - V) * (V < mu)
            NN = self.grid.integrate(vvv)
            if NN > NC:
                mur = mu
            else:
                mul = mu
            mu = (mul + mur) / 2
        return np.sqrt(vvv / self.g), mu

    # lib/@GPEtask/set_kinop.m:1-11 (array omega: :3-4, scalar omega: :5-7, omega == 0: :9)
    def set_kinop(self, dt):
        grid = self.grid
        if self._omega_array():
            self.kinop = np.exp(-grid.kk * dt / 2)
        elif self.omega != 0:
            self.kinop = np.exp(-(grid.KX ** 2 / 2 - grid.KX * grid.mesh["y"] * self.omega) * dt / 2)
            self.kinop2 = np.exp(-(grid.KY ** 2 / 2 + grid.KZ ** 2 / 2 + grid.KY * grid.mesh["x"] * self.omega) * dt)
        else:
            self.kinop = np.exp(-grid.kk * dt)

    # lib/@GPEtask/ssft_kin_step.m:1-17
    def ssft_kin_step(self, phi, dt):
        grid = self.grid
        if self._omega_array():                                                      # :3-11
            phi = grid.ifft(self.kinop * grid.fft(phi))
            lphi = phi
            for _ in range(self.n_crank):
                lphi = phi + dt * self.omega * grid.lz(lphi)
                lphi = 0.5 * (phi + lphi)
            phi = phi + dt * self.omega * grid.lz(lphi)
            return grid.ifft(self.kinop * grid.fft(phi))
        if self.omega != 0:
            phi = grid.ifft1(self.kinop * grid.fft1(phi, "x"), "x")                 # :13
            if grid.ndims == 3:                                                      # :14
                phi = grid.ifft1(grid.ifft1(self.kinop2 * grid.fft1(grid.fft1(phi, "y"), "z"), "z"), "y")
            else:
                phi = grid.ifft1(self.kinop2 * grid.fft1(phi, "y"), "y")
            return grid.ifft1(self.kinop * grid.fft1(phi, "x"), "x")                # :15
        return grid.ifft(self.kinop * grid.fft(phi))

    # lib/@GPEtask/groundstate_itp.m:1-112
    def groundstate_itp(self, dt, eps, phi0="rand", nargout=4, rng=None):
        """Returns (phi, MU, MU2, EE) with MU2/EE computed iff nargout >= 3/4."""
        grid = self.grid
        V = self.getVtotal(0)                                           # :20
        nnn = self.Ntotal if self.Ntotal > 0 else 1                     # :21-25
        phi = self.process_init_state(phi0, rng=rng)                    # :27
        self.current_state = phi                                        # :28
        self.set_kinop(dt)                                              # :30
        MU = np.zeros(self.itp_max_iter)
        MU2 = np.zeros(self.itp_max_iter)
        EE = np.zeros(self.itp_max_iter)
        i = 0
        self.itp_deltas = []
        dtmin = math.sqrt(eps)                                          # :35
        self.nlinop = np.exp(-dt * 0.5 * (np.abs(phi) ** 2 * self.g + V))  # :36
        while True:
            i += 1
            phi = self.nlinop * phi                                     # :40
            phi = self.ssft_kin_step(phi, dt)                           # :41
            phi = self.nlinop * phi                                     # :42
            self.nlinop = np.abs(phi) ** 2                              # :44
            if self.Ntotal > 0:
                mu = math.sqrt(self.Ntotal / grid.integrate(self.nlinop))  # :46
                MU[i - 1] = math.log(mu) / dt
            else:
                mu = math.exp(self.mu_init * dt)
                MU[i - 1] = grid.integrate(self.nlinop) * mu ** 2
            phi = phi * mu                                              # :52
            if i > self.itp_min_iter and i % 10 == 0:                   # :54
                if nargout >= 3:
                    MU2[i - 1] = np.real(grid.inner(phi, self.applyham(phi)))
                if nargout >= 4:
                    EE[i - 1] = self.get_energy(phi)
                delta = np.max(np.abs(np.abs(phi.ravel()) - np.abs(self.current_state.ravel()))) / (dt * 10)
                self.itp_deltas.append((i, delta))  # diagnostics only
                self.current_state = phi
                if delta < eps:
                    if nargout >= 3:
                        dtmin = dt * math.sqrt(eps / abs(MU[i - 1] - MU2[i - 1] / nnn))
                    if (not self.itp_adjust_stepsize) or dt < dtmin:
                        break
                    dt = dt / 2
                    self.set_kinop(dt)
            self.nlinop = np.exp(-dt * 0.5 * (self.nlinop * self.g * mu ** 2 + V))  # :76
            if i >= self.itp_max_iter:
                warnings.warn("Convergence not reached")
                break
        MU = MU[:i].copy()
        if self.Ntotal > 0:
            self.current_mu = MU[-1]
            self.current_n = self.Ntotal
            MU2 = MU2[:i] / self.Ntotal
            EE = EE[:i] / self.Ntotal
        else:
            MU2 = MU2[:i] / MU
            self.current_mu = MU2[-1]
            self.current_n = MU[-1]
            EE = EE[:i] / MU
        self.init_state = phi                                           # :111
        return phi, MU, MU2, EE

    # lib/@GPEtask/solve_split.m:1-84
    def solve_split(self, ddt, niter_inner, niter_outer, inner_callback=None):
        """``inner_callback(i)`` (timing hook, not in the reference) runs after
        every inner step; it may raise to stop the run."""
        grid = self.grid
        g = self.g
        NN0 = self.Ntotal if self.Ntotal > 0 else grid.integrate(np.abs(self.init_state) ** 2)  # :17-21
        NNN = NN0
        gam = self.gamma
        n_rec = self.n_recalc
        if niter_inner % n_rec != 0:                                    # :25-27
            n_rec = 1
        tau = self.decay_rate
        start = self.current_iter
        dt = ddt * 1j / (1 + 1j * gam)                                  # :31
        self.set_kinop(dt)
        phi = self.current_state if start > 0 else self.init_state      # :34-38
        self.nlinop = np.real(phi * np.conj(phi))                       # :40
        muc = np.real(grid.inner(phi, self.applyham(phi))) / NN0        # :41
        mu = self.mu_init if self.mu_init > 0 else muc                  # :42-46
        dt_outer = ddt * niter_inner
        ncur = None
        time2 = None
        for j in range(start + 1, niter_outer + 1):                     # :49
            time = (j - 1) * dt_outer
            for jj in range(1, niter_inner // n_rec + 1):               # :51
                time2 = time + (jj - 1) * ddt * n_rec
                VV = self.getVtotal(time2) - mu                         # :54
                self.nlinop = np.exp((-VV - g * self.nlinop) * dt * 0.5)
                phi = self.nlinop * phi
                for _ in range(n_rec):                                  # :58-62
                    phi = self.ssft_kin_step(phi, dt)
                    self.nlinop = np.exp((-VV - g * phi * np.conj(phi)) * dt)
                    phi = self.nlinop * phi
                    if inner_callback is not None:
                        inner_callback(j)
                self.nlinop = np.exp((VV + g * phi * np.conj(phi)) * dt * 0.5)  # :63-64
                phi = self.nlinop * phi
                self.nlinop = np.real(phi * np.conj(phi))               # :65
                ncur = grid.integrate(self.nlinop)                      # :67
                if gam > 0 and self.mu_init == 0:                       # :68-75
                    if tau > 0:
                        NNN = NN0 * math.exp(-time2 / tau)
                    phi = phi * math.sqrt(NNN / ncur)
                    self.nlinop = self.nlinop * (NNN / ncur)
                    muc = np.real(grid.inner(phi, self.applyham(phi, time2))) / NNN
                    mu = muc
                else:                                                   # :76-78
                    muc = np.real(grid.inner(phi, self.applyham(phi, time2))) / ncur
            self.ext_callback(phi, j, time2, muc, ncur)                 # :80
        return phi


# ---------------------------------------------------------------------------
# Discrete adjoint of the gamma = 0 split step.  Not in the reference: the
# forward operator is solve_split.m:55-64 at gamma = 0, where every nonlinear
# factor is a pure phase, so a block of n_recalc steps equals
# (N_h K N_h)^n_recalc with N_h(phi) = exp(-i (V - mu + g|phi|^2) ddt/2) phi and
# K = ifft(exp(-i kk ddt) fft(.)) (set_kinop.m:9 with dt = i ddt).  mu is a
# global phase that the overlap loss does not see and is left out.
# ---------------------------------------------------------------------------
def _nl_half(V, g, h, phi):
    return np.exp(-1j * (V + g * np.real(phi * np.conj(phi))) * h) * phi


def split_forward(grid: Grid, V, g, psi0, ddt, nsteps, keep_states=False):
    """psi(T) after nsteps steps N_h K N_h; with keep_states also every
    step-start state."""
    kin = np.exp(-1j * grid.kk * ddt)
    h = 0.5 * ddt
    phi = np.asarray(psi0, dtype=np.complex128)
    states = []
    for _ in range(nsteps):
        if keep_states:
            states.append(phi)
        phi = _nl_half(V, g, h, phi)
        phi = grid.ifft(kin * grid.fft(phi))
        phi = _nl_half(V, g, h, phi)
    return phi, states


def overlap_loss(grid: Grid, target, psiT, psi0):
    """1 - |<target|psi(T)>|^2 / (<target|target> <psi0|psi0>), and the
    normalised overlap c."""
    denom = math.sqrt(grid.integrate(np.abs(target) ** 2) * grid.integrate(np.abs(psi0) ** 2))
    c = grid.inner(target, psiT) / denom
    return 1.0 - abs(c) ** 2, c


def _adj_nl(V, g, h, lam, x):
    """Adjoint of y = exp(-i th) x, th = (V + g|x|^2) h, for lam = dL/dy*
    (Wirtinger): returns dL/dx* and the contribution to dL/dV."""
    u = np.exp(1j * (V + g * np.real(x * np.conj(x))) * h) * lam
    s = 2.0 * np.imag(np.conj(u) * x)
    return u + g * h * s * x, s * h


def adjoint_grad(grid: Grid, V, g, psi0, target, ddt, nsteps):
    """(loss, dL/dV) of overlap_loss after split_forward, by the reverse sweep
    of the same operator sequence; dL/dV[i] is the derivative with respect to
    the potential's value at grid point i."""
    V = np.asarray(V, dtype=np.float64)
    psiT, states = split_forward(grid, V, g, psi0, ddt, nsteps, keep_states=True)
    loss, c = overlap_loss(grid, target, psiT, psi0)
    denom = math.sqrt(grid.integrate(np.abs(target) ** 2) * grid.integrate(np.abs(psi0) ** 2))
    lam = -c * grid.weight / denom * np.asarray(target, dtype=np.complex128)
    kin = np.exp(-1j * grid.kk * ddt)
    h = 0.5 * ddt
    dLdV = np.zeros(grid.shape)
    for x0 in reversed(states):
        phi2 = grid.ifft(kin * grid.fft(_nl_half(V, g, h, x0)))
        lam, d = _adj_nl(V, g, h, lam, phi2)
        dLdV += d
        lam = grid.ifft(np.conj(kin) * grid.fft(lam))
        lam, d = _adj_nl(V, g, h, lam, x0)
        dLdV += d
    return loss, dLdV


def _set_hist(lst, step, val):
    """MATLAB ``history.mu(step) = mu`` grows the row vector with zeros."""
    while len(lst) < step:
        lst.append(0.0)
    lst[step - 1] = val


# ---------------------------------------------------------------------------
# Stochastic GPE: lib/@SGPEtask/solve_split.m:1-81 (scalar omega = 0)
# ---------------------------------------------------------------------------
class SGPEtask(GPEtask):
    """SGPEtask (lib/@SGPEtask/SGPEtask.m:1-48): GPEtask with temperature T and
    energy cut-off ecut.  ``noise(shape)`` supplies the complex standard
    normal variates randn + 1i*randn of solve_split.m:55 (the reference draws
    them from MATLAB's generator; a seeded numpy generator by default)."""

    def __init__(self, grid, trappot):
        super().__init__(grid, trappot)
        self.T = 0.0
        self.ecut = 0.0
        self.noise = None

    def solve_split(self, ddt, niter_inner, niter_outer, rng=None):
        grid = self.grid
        g = self.g
        NN0 = self.Ntotal if self.Ntotal > 0 else grid.integrate(np.abs(self.init_state) ** 2)  # :19-23
        gam = self.gamma
        n_rec = self.n_recalc
        start = self.current_iter
        dt = ddt * 1j / (1 + 1j * gam)                                   # :31
        phi = self.current_state if start > 0 else self.init_state       # :33-37
        tmp2 = np.real(phi * np.conj(phi))                               # :39
        if self.ecut > 0 and self.T > 0:                                 # :41-46
            mask = grid.kk < self.ecut
            ekk = np.exp(-grid.kk * dt) * mask
        else:
            ekk = np.exp(-grid.kk * dt)
        dt_outer = ddt * niter_inner
        variance = math.sqrt(self.T * gam * ddt / grid.weight)          # :49
        rng = rng or np.random.default_rng(0)
        noise = self.noise or (lambda shape: rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
        ncur = time2 = None
        mu = self.mu_init
        for j in range(start + 1, niter_outer + 1):                     # :51
            mu = self.mu_init                                            # :52
            time = (j - 1) * dt_outer
            for jj in range(1, niter_inner // n_rec + 1):                # :54
                time2 = time + (jj - 1) * ddt * n_rec
                VV = self.getVtotal(time2)
                phi = np.exp((mu - VV - g * tmp2) * dt / 2) * phi        # :57
                for _ in range(n_rec):                                   # :59-70
                    phi = phi + variance * noise(phi.shape)
                    phi = grid.ifft(ekk * grid.fft(phi))
                    if self.omega != 0:                                  # :61-67
                        lphi = phi
                        for _ in range(self.n_crank):
                            lphi = phi + dt * self.omega * grid.lz(lphi)
                            lphi = 0.5 * (phi + lphi)
                        phi = phi + dt * self.omega * grid.lz(lphi)
                    phi = np.exp((mu - VV - g * phi * np.conj(phi)) * dt) * phi
                phi = np.exp((VV - mu + g * phi * np.conj(phi)) * dt / 2) * phi  # :73
                tmp2 = np.real(phi * np.conj(phi))
                ncur = grid.integrate(tmp2)                              # :76
            err = self.ext_callback(phi, j, time2, mu, ncur)             # :77
            if isinstance(err, str) and err == "TERM":                   # :78-80
                break
        return phi


# ---------------------------------------------------------------------------
# Coherently coupled two-component condensate: lib/@GPEtaskSpinor
# ---------------------------------------------------------------------------
class GPEtaskSpinor(GPEtask):
    """GPEtaskSpinor (lib/@GPEtaskSpinor/GPEtaskSpinor.m:1-147): states and
    potentials are lists of two arrays, g a 2x2 matrix, ``coupling`` the
    (complex) Rabi coupling and ``nlincpl`` its density-dependent part.
    omega == 0 only.  (lib/@GPEtask2comp/solve_split.m is the same loop; that
    class declares no coupling/nlincpl properties, so it is this one with
    coupling = nlincpl = 0.)"""

    def __init__(self, grid, trappot):
        super().__init__(grid, lambda X, Y, Z: 0.0 * X)
        self.coupling = 0.0
        self.nlincpl = 0.0
        self.ncomp = len(trappot)                                        # :13-20
        X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
        self.Vtrap = [np.broadcast_to(f(X, Y, Z) if callable(f) else np.asarray(f, np.float64),
                                      grid.shape).astype(np.float64) for f in trappot]
        self.g = np.zeros((self.ncomp, self.ncomp))
        self.init_state = [np.zeros(grid.shape, np.complex128) for _ in range(self.ncomp)]

    # GPEtaskSpinor.m:23-42 (the internal V0 branch is not restated)
    def getVtotal(self, time):
        if callable(self.Vtd):
            return [V + self.Vtd(self, time) for V in self.Vtrap]
        if isinstance(self.Vtd, (list, tuple)):
            return [V + f(self, time) for V, f in zip(self.Vtrap, self.Vtd)]
        return self.Vtrap

    # GPEtaskSpinor.m:55-76 (scalar omega: -omega lz with grid1d's stencil, :72-74)
    def applyham1c(self, phi, j, time=None):
        if time is None:
            time = self.current_time
        res = self.getVtotal(time)[j]
        for k in range(self.ncomp):
            res = res + self.g[j, k] * np.abs(phi[k]) ** 2
        res = res * phi[j] + self.grid.lap(phi[j])
        if j == 0:
            res = res + self.coupling * phi[1]
        else:
            res = res + np.conj(self.coupling) * phi[0]
        if self.omega != 0:
            res = res - self.omega * self.grid.lz(phi[j])
        return res

    # the rotating half step of groundstate_itp.m:61-65 (spinor: x then y on
    # both sides) and of GPEtask2comp/groundstate_itp.m:61-80 (y then x after
    # the nonlinear factor); ekx/eky of :31-32, tau = dt/(2M)
    def _rot_factors(self, dt, M=1.0):
        grid = self.grid
        om = self.omega
        ekx = np.exp(-(grid.KX ** 2 - 2 * grid.KX * grid.mesh["y"] * om) / 4 * dt / M)
        eky = np.exp(-(grid.KY ** 2 + 2 * grid.KY * grid.mesh["x"] * om) / 4 * dt / M)
        return ekx, eky

    def _rot_half(self, p, ek, order):
        grid = self.grid
        for ax in order:
            f = ek[0] if ax == "x" else ek[1]
            p = grid.ifft1(f * grid.fft1(p, ax), ax)
        return p

    # GPEtaskSpinor.m:74-82
    def applyham(self, phi, time=None):
        return [self.applyham1c(phi, j, time) for j in range(self.ncomp)]

    # GPEtaskSpinor.m:84-89
    def inner(self, left, right):
        return sum(self.grid.inner(a, b) for a, b in zip(left, right))

    # GPEtaskSpinor.m:98-110
    def get_energy(self, phi=None, time=None):
        if phi is None:
            phi = self.current_state
        tmp = self.g
        self.g = 0.5 * self.g
        try:
            res = np.real(self.inner(phi, self.applyham(phi, time)))
        finally:
            self.g = tmp
        return res

    # lib/@GPEtaskSpinor/groundstate_itp.m:1-145 (scalar omega: the x and y
    # half steps of :30-33, 61-80 in place of ekk)
    def groundstate_itp(self, dt, eps, phi, nargout=4, max_iter=500000):
        """Returns (phi, MU, MU2, EE); MU2/EE are filled as the reference does
        for the given nargout (MU2 = MU when nargout < 3, EE = MU2 when
        nargout < 4), and the returned arrays drop the last iteration (:132-141)."""
        grid = self.grid
        ncomp = self.g.shape[0]                                          # :20
        VV = self.getVtotal(0)
        coupl = self.coupling
        g = self.g
        phi = [np.asarray(p, dtype=np.complex128) for p in phi]
        ekk = np.exp(-grid.kk * dt * 0.5)                                # :29
        rot = self.omega != 0
        ek = self._rot_factors(dt) if rot else None                      # :30-33
        MU, MU2, EE = [], [], []
        i = 1
        iswitch = 20
        cang = np.angle(coupl)                                           # :45-48
        cosom = np.cosh(dt * abs(coupl))
        sinomm = np.sinh(dt * abs(coupl)) * np.exp(-1j * cang)
        sinomp = np.sinh(dt * abs(coupl)) * np.exp(1j * cang)
        while True:
            tmp2 = [VV[j] + sum(g[j, k] * np.abs(phi[k]) ** 2 for k in range(ncomp)) for j in range(ncomp)]
            if rot:                                                      # :61-65
                phi = [self._rot_half(p, ek, "xy") for p in phi]
            else:
                phi = [grid.ifft(ekk * grid.fft(p)) for p in phi]        # :69-70
            t0 = np.exp(-tmp2[0] * dt) * (cosom * phi[0] - sinomp * phi[1])  # :72-73
            t1 = np.exp(-tmp2[1] * dt) * (cosom * phi[1] - sinomm * phi[0])
            if rot:                                                      # :74-78
                phi = [self._rot_half(t, ek, "xy") for t in (t0, t1)]
            else:
                phi = [grid.ifft(ekk * grid.fft(t)) for t in (t0, t1)]  # :80-81
            ntot = np.real(grid.integrate(phi[0] * np.conj(phi[0]) + phi[1] * np.conj(phi[1])))
            mu = math.sqrt(self.Ntotal / ntot)                           # :84-88
            MU.append(math.log(mu) / dt)
            phi = [p * mu for p in phi]
            self.current_state = phi
            MU2.append(np.real(self.inner(phi, self.applyham(phi))) / self.Ntotal if nargout >= 3 else MU[-1])
            EE.append(self.get_energy(phi) / self.Ntotal if nargout >= 4 else MU2[-1])
            if (i - iswitch) > 10 and i % 10 == 0:                       # :101-122
                delta = (abs(EE[i - 1] - EE[i - 10]) / 9 + abs(EE[i - 1] - EE[i - 2])) / dt
                if delta < eps:
                    if dt < eps or dt < 5e-6:
                        break
                    dt = dt / 1.5
                    ekk = np.exp(-grid.kk * dt * 0.5)
                    ek = self._rot_factors(dt) if rot else None
                    cosom = np.cosh(dt * abs(coupl))
                    sinomm = np.sinh(dt * abs(coupl)) * np.exp(-1j * cang)
                    sinomp = np.sinh(dt * abs(coupl)) * np.exp(1j * cang)
                    iswitch = i
            if i >= max_iter:                                            # :123-126
                warnings.warn("Convergence not reached")
                break
            i += 1
        self.init_state = phi                                            # :143-144
        self.current_state = phi
        self.final_dt = dt
        return phi, np.array(MU[:i - 1]), np.array(MU2[:i - 1]), np.array(EE[:i - 1])

    # lib/@GPEtaskSpinor/solve_split.m:1-119
    def solve_split(self, ddt, niter_inner, niter_outer):
        grid = self.grid
        ncomp = self.g.shape[0]                                          # :14
        g = self.g
        gam = self.gamma
        n_rec = self.n_recalc
        tau = self.decay_rate
        start = self.current_iter
        phi = list(self.current_state) if start > 0 else list(self.init_state)  # :23-27
        if self.Ntotal > 0:                                              # :29-37
            NN0 = self.Ntotal
        else:
            # :33-35; the reference then overwrites NN0 with
            # integrate(abs(init_state).^2) (:36), which errors on a cell array
            NN0 = sum(grid.integrate(np.real(p * np.conj(p))) for p in phi)
        NNN = NN0
        ncur = NN0
        dt = ddt * 1j / (1 + 1j * gam)                                   # :41
        ekk = np.exp(-grid.kk * dt)
        ekkp = np.exp(-grid.kk * dt * 0.5)
        ekkm = np.exp(grid.kk * dt * 0.5)
        tmp2 = [None] * ncomp
        hphi = self.applyham(phi)                                        # :52-57
        mu = sum(np.real(grid.inner(phi[j], hphi[j])) for j in range(ncomp)) / NN0
        dt_outer = ddt * niter_inner
        time2 = None
        for j in range(start + 1, niter_outer + 1):                     # :59
            coupl = self.coupling
            cang = np.angle(coupl)
            cosom = np.cosh(dt * abs(coupl))
            sinomm = np.sinh(dt * abs(coupl)) * np.exp(-1j * cang)
            sinomp = np.sinh(dt * abs(coupl)) * np.exp(1j * cang)
            time = (j - 1) * dt_outer
            for jj in range(1, niter_inner // n_rec + 1):                # :66
                time2 = time + (jj - 1) * ddt * n_rec
                VV = self.getVtotal(time2)
                phi = [grid.ifft(ekkp * grid.fft(p)) for p in phi]       # :72-74
                for _ in range(n_rec):                                   # :75-96
                    for i in range(ncomp):
                        tmp2[i] = VV[i] - mu
                        for k in range(ncomp):
                            tmp2[i] = tmp2[i] + g[i, k] * np.abs(phi[k]) ** 2
                    if self.nlincpl != 0:                                # :84-89
                        tmp3 = coupl + self.nlincpl * (np.abs(phi[0]) ** 2 + np.abs(phi[1]) ** 2)
                        cosom = np.cosh(dt * tmp3)
                        sinomm = np.sinh(dt * tmp3)
                        sinomp = sinomm
                    t0 = np.exp(-tmp2[0] * dt) * (cosom * phi[0] - sinomp * phi[1])  # :90-91
                    t1 = np.exp(-tmp2[1] * dt) * (cosom * phi[1] - sinomm * phi[0])
                    phi = [grid.ifft(ekk * grid.fft(t)) for t in (t0, t1)]  # :92-94
                phi = [grid.ifft(ekkm * grid.fft(p)) for p in phi]       # :97-99
                ncur = np.real(grid.integrate(phi[0] * np.conj(phi[0]) + phi[1] * np.conj(phi[1])))  # :105,111
                if gam > 0:                                              # :100-109
                    if tau > 0:
                        NNN = NN0 * math.exp(-time2 / tau)
                    phi = [p * math.sqrt(NNN / ncur) for p in phi]
                hphi = self.applyham(phi)     # at current_time (:107, :112)
                mu = self.inner(phi, hphi) / NNN
            self.ext_callback(phi, j, time2, mu, ncur)                   # :115
        return phi


class GPEtask2comp(GPEtaskSpinor):
    """GPEtask2comp (lib/@GPEtask2comp/GPEtask2comp.m:1-150): an incoherent
    mixture, components normalised separately to N1 and N2, masses M1, M2 in
    the imaginary-time kinetic factors; applyham/get_energy are the spinor's
    without coupling (GPEtask2comp.m:51-74, 107-118), the rotating frame
    through lap(phi, omega)."""

    def __init__(self, grid, trappot):
        super().__init__(grid, trappot)
        self.N1 = self.N2 = 0.0
        self.M1 = self.M2 = 1.0

    # GPEtask2comp.m:51-64: no coupling; the rotating frame enters through
    # lap(phi, omega) (:60), not through lz
    def applyham1c(self, phi, j, time=None):
        if time is None:
            time = self.current_time
        res = self.getVtotal(time)[j]
        for k in range(self.ncomp):
            res = res + self.g[j, k] * np.abs(phi[k]) ** 2
        return res * phi[j] + self.grid.lap(phi[j], self.omega)

    # lib/@GPEtask2comp/groundstate_itp.m:1-157 (scalar omega: the x/y half
    # steps of :31-36, 61-80 with each component's mass)
    def groundstate_itp(self, dt, eps, phi, nargout=4, max_iter=500000):
        """Returns (phi, MU1, MU2, EE); EE = get_energy/Ntotal when nargout >= 4,
        else MU2 (:98-102); the returned arrays drop the last iteration (:143-154)."""
        grid = self.grid
        VV = self.getVtotal(0)
        g = self.g
        phi = [np.asarray(p, dtype=np.complex128) for p in phi]
        ekk1 = np.exp(-grid.kk * dt * 0.5 / self.M1)                    # :29-30
        ekk2 = np.exp(-grid.kk * dt * 0.5 / self.M2)
        rot = self.omega != 0
        ek = (self._rot_factors(dt, self.M1), self._rot_factors(dt, self.M2)) if rot else None
        MU1, MU2, EE = [], [], []
        i = 1
        iswitch = 20
        while True:
            t1 = VV[0] + g[0, 0] * np.abs(phi[0]) ** 2 + g[0, 1] * np.abs(phi[1]) ** 2   # :58-59
            t2 = VV[1] + g[1, 0] * np.abs(phi[0]) ** 2 + g[1, 1] * np.abs(phi[1]) ** 2
            if rot:                                                                     # :61-65
                phi = [self._rot_half(phi[0], ek[0], "xy"), self._rot_half(phi[1], ek[1], "xy")]
            else:                                                                       # :67-68
                phi = [grid.ifft(ekk1 * grid.fft(phi[0])), grid.ifft(ekk2 * grid.fft(phi[1]))]
            phi = [np.exp(-t1 * dt) * phi[0], np.exp(-t2 * dt) * phi[1]]                # :70-71
            if rot:                                                                     # :72-76
                phi = [self._rot_half(phi[0], ek[0], "yx"), self._rot_half(phi[1], ek[1], "yx")]
            else:                                                                       # :78-79
                phi = [grid.ifft(ekk1 * grid.fft(phi[0])), grid.ifft(ekk2 * grid.fft(phi[1]))]
            n1c = np.real(grid.integrate(phi[0] * np.conj(phi[0])))                      # :82-90
            n2c = np.real(grid.integrate(phi[1] * np.conj(phi[1])))
            mu1 = math.sqrt(self.N1 / n1c)
            mu2 = math.sqrt(self.N2 / n2c)
            MU1.append(math.log(mu1) / dt)
            MU2.append(math.log(mu2) / dt)
            phi = [phi[0] * mu1, phi[1] * mu2]
            self.current_state = phi
            EE.append(self.get_energy(phi) / self.Ntotal if nargout >= 4 else MU2[-1])  # :98-102
            if (i - iswitch) > 10 and i % 10 == 0:                                      # :113-135
                delta = (abs(EE[i - 1] - EE[i - 10]) / 9 + abs(EE[i - 1] - EE[i - 2])) / dt
                if delta < eps:
                    if dt < eps or dt < 5e-6:
                        break
                    dt = dt / 1.5
                    ekk1 = np.exp(-grid.kk * dt * 0.5 / self.M1)
                    ekk2 = np.exp(-grid.kk * dt * 0.5 / self.M2)
                    if rot:
                        ek = (self._rot_factors(dt, self.M1), self._rot_factors(dt, self.M2))
                    iswitch = i
            if i >= max_iter:
                warnings.warn("Convergence not reached")
                break
            i += 1
        self.init_state = phi
        self.current_state = phi
        self.final_dt = dt
        return phi, np.array(MU1[:i - 1]), np.array(MU2[:i - 1]), np.array(EE[:i - 1])


# ---------------------------------------------------------------------------
# Vortex-core detection: lib/util/detect_core.m:1-67.  Arrays here are
# indexed [ix, iy] (the transpose of MATLAB's row = y, column = x matrix), so
# MATLAB's column-major find() order is this C order.
# ---------------------------------------------------------------------------
def _second_diff(U, h, axis):
    """One dimension of MATLAB's del2: central second differences inside,
    linear extrapolation to the two edge points (n > 3)."""
    n = U.shape[axis]
    g = np.zeros_like(U)

    def s(a, b):
        return tuple(slice(a, b) if k == axis else slice(None) for k in range(U.ndim))

    g[s(1, n - 1)] = (U[s(2, n)] - 2.0 * U[s(1, n - 1)] + U[s(0, n - 2)]) / h ** 2
    g[s(0, 1)] = 2.0 * g[s(1, 2)] - g[s(2, 3)]
    g[s(n - 1, n)] = 2.0 * g[s(n - 2, n - 1)] - g[s(n - 3, n - 2)]
    return g


def del2(U, hx, hy):
    """del2(U, hx, hy) of a 2D field: (d2/dx2 + d2/dy2)/4 (x along axis 0)."""
    return (_second_diff(U, hx, 0) + _second_diff(U, hy, 1)) / 4.0


def core_charges(phi, rx, ry):
    """res1 of detect_core.m:14-27: the winding of the phase around each
    plaquette (corners (i,j), (i-1,j), (i-1,j-1), (i,j-1) in MATLAB's row/column
    indices, circular), kept where |del2(|phi|^2)| > 1% of its maximum."""
    n_x, n_y = phi.shape
    dx = rx[n_x // 2, 0] - rx[n_x // 2 - 1, 0]                # :13
    dy = ry[0, n_y // 2] - ry[0, n_y // 2 - 1]                # :14
    an = np.angle(phi)
    ddphi = np.abs(del2(np.abs(phi) ** 2, dx, dy))            # :18
    a = [an, np.roll(an, 1, axis=1), np.roll(np.roll(an, 1, axis=1), 1, axis=0), np.roll(an, 1, axis=0)]
    dif = [a[k] - a[k - 1] for k in range(4)]                 # :24 (k = 0 wraps to the 4th corner)
    cnt = sum((d > math.pi).astype(int) for d in dif) - sum((d < -math.pi).astype(int) for d in dif)
    return cnt * (ddphi > 0.01 * np.max(ddphi)), dx, dy       # :25


def _refine_core(phi, rx, ry, dx, dy, jx, iy):
    """refine_core of detect_core.m:51-66 at MATLAB (row, column) = (iy, jx),
    1-based and already clamped to >= 2 (C.L. Phillips et al., Phys. Rev. E 91,
    023311 (2015))."""
    import scipy.linalg

    rep, imp = np.real(phi), np.imag(phi)

    def at(f, r, c):  # MATLAB f(r, c), 1-based
        return f[c - 1, r - 1]

    r, c = iy, jx
    A = -np.array([[at(rep, r - 1, c) - at(rep, r, c), at(rep, r, c)],
                   [at(imp, r - 1, c) - at(imp, r, c), at(imp, r, c)]])
    B = np.array([[at(rep, r, c) - at(rep, r - 1, c) - at(rep, r, c - 1) + at(rep, r - 1, c - 1),
                   at(rep, r, c - 1) - at(rep, r, c)],
                  [at(imp, r, c) - at(imp, r - 1, c) - at(imp, r, c - 1) + at(imp, r - 1, c - 1),
                   at(imp, r, c - 1) - at(imp, r, c)]])
    d, v = scipy.linalg.eig(A, B)
    v = v[0, :] / v[1, :]
    for i in range(2):
        if np.real(d[i]) > 0 and np.real(d[i]) < 1 and np.real(v[i]) > 0 and np.real(v[i]) < 1:
            return [at(rx, r, c) - dy * np.real(d[i]), at(ry, r, c) - dx * np.real(v[i])]
    return [0.0, 0.0]


def detect_core(phi, rx, ry, refine=0):
    """detect_core.m:1-49: (resp, resm), k x 2 arrays of [x, y] of the positive
    and negative cores in MATLAB's find() order."""
    res1, dx, dy = core_charges(phi, rx, ry)
    out = []
    for sign in (1, -1):
        res = res1 * sign > 0
        if refine > 0:
            jx, iy = np.nonzero(res)  # C order of [ix, iy] = MATLAB's column-major order
            pts = [_refine_core(phi, rx, ry, dx, dy, max(j + 1, 2), max(i + 1, 2)) for j, i in zip(jx, iy)]
            out.append(np.array(pts, dtype=np.float64).reshape(-1, 2))
        else:
            ydel = dy if sign > 0 else dx  # :45 subtracts dx from y for the negative cores
            out.append(np.stack([rx[res] - dx / 2, ry[res] - ydel / 2], axis=1))
    return out[0], out[1]


# ---------------------------------------------------------------------------
# Vortex imprint: examples/example1_vortex.m:26-30 (also README.md:93-97)
# ---------------------------------------------------------------------------
def imprint_vortex(grid: Grid, phi, g, x0, y0=0.0):
    """psi * tanh(r/xi) * exp(i*atan2(X - x0, Y - y0)), xi = 1/sqrt(2 g max|psi|^2).

    The argument order of atan2 follows example1_vortex.m:29 exactly.
    """
    xi = 1.0 / math.sqrt(2 * g * np.max(np.abs(phi)) ** 2)
    X, Y = grid.mesh["x"], grid.mesh["y"]
    rr = np.sqrt((X - x0) ** 2 + (Y - y0) ** 2)
    angs = np.arctan2(X - x0, Y - y0)
    return phi * np.tanh(rr / xi) * np.exp(1j * angs)
