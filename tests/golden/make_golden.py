"""Generate the golden fixtures under tests/golden/ from the FP64 oracle.

    python tests/golden/make_golden.py

Each case runs oracle/gpe_oracle.py on a small seeded input and stores the
inputs and outputs (.npz).  The reference itself (MATLAB) cannot run here, so
these fixtures pin the oracle against regressions and give the GPU parity
tests fixed inputs and expected outputs; the oracle is pinned to physics by
tests/test_oracle.py.

Inputs: psi0 = exp(-r^2/(2 sigma^2)) + 1e-3 (N(0,1) + i N(0,1))/sqrt(2) with
numpy default_rng(seed), as in gpe_workloads.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle import gpe_oracle as O  # noqa: E402


def path(name: str) -> Path:
    return HERE / f"{name}.npz"


def gaussian_noise(grid, sigma, seed, noise=1e-3):
    rng = np.random.default_rng(seed)
    X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
    r2 = X ** 2 + Y ** 2 + (Z ** 2 if grid.ndims == 3 else 0.0)
    phi = np.exp(-r2 / (2 * sigma ** 2)).astype(np.complex128)
    return phi + noise * (rng.standard_normal(grid.shape) + 1j * rng.standard_normal(grid.shape)) / np.sqrt(2)


def case_itp_vortex2d_64():
    """2D plain method at 64^2: ITP, vortex imprint at x0 = 5, 4 x 50 steps."""
    g = O.Grid(17, 64, 17, 64)
    t = O.GPEtask(g, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2))
    t.Ntotal = 1e5
    t.g = 0.06
    psi0 = gaussian_noise(g, 4.0, 1)
    phi, MU, MU2, EE = t.groundstate_itp(0.02, 1e-6, psi0)
    vort = O.imprint_vortex(g, phi, t.g, 5.0)
    t.init_state = vort
    t.solve_split(0.004, 50, 4)
    return {"psi0": psi0, "phi": phi, "MU": MU, "MU2": MU2, "EE": EE, "vortex": vort,
            "psi_t": t.current_state, "hist_mu": np.array(t.history["mu"]), "hist_n": np.array(t.history["n"]),
            "current_time": np.array(t.current_time)}


def case_split_damped2d_48():
    """48^2 (radix-3 lengths), gamma = 0.05, decay tau = 2, N = 50, anisotropic trap."""
    g = O.Grid(6, 48, 5, 48)
    t = O.GPEtask(g, lambda X, Y, Z: 0.5 * (X ** 2 + (1.3 * Y) ** 2))
    t.Ntotal = 50.0
    t.g = 1.0
    t.gamma = 0.05
    t.decay_rate = 2.0
    psi0 = gaussian_noise(g, 1.5, 2) * np.exp(0.3j * g.mesh["x"])
    t.init_state = np.sqrt(50.0) * g.normalize(psi0)
    t.solve_split(0.01, 10, 3)
    return {"psi0": t.init_state, "psi_t": t.current_state, "hist_mu": np.array(t.history["mu"]),
            "hist_n": np.array(t.history["n"])}


def case_split3d_24x32x16():
    """3D with unequal axes (nx=24, ny=32, nz=16), gamma = 0, Ntotal = 0."""
    g = O.Grid(5, 24, 6, 32, 4, 16)
    t = O.GPEtask(g, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2 + (1.5 * Z) ** 2))
    t.g = 1.0
    psi0 = gaussian_noise(g, 1.2, 3) * np.exp(0.5j * g.mesh["y"])
    t.init_state = psi0
    t.solve_split(0.005, 10, 2)
    return {"psi0": psi0, "psi_t": t.current_state, "hist_mu": np.array(t.history["mu"]),
            "hist_n": np.array(t.history["n"])}


def case_itp3d_adjust_16():
    """3D ITP at 16^3 with itp_adjust_stepsize (dt halving), lambda = (1, 1, 2)."""
    g = O.Grid(5, 16, 5, 16, 4, 16)
    t = O.GPEtask(g, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2 + (2 * Z) ** 2))
    t.Ntotal = 20.0
    t.g = 1.0
    t.itp_adjust_stepsize = True
    psi0 = gaussian_noise(g, 1.5, 4)
    phi, MU, MU2, EE = t.groundstate_itp(0.05, 1e-5, psi0)
    return {"psi0": psi0, "phi": phi, "MU": MU, "MU2": MU2, "EE": EE}


def _pair_start(g):
    X, Y = g.mesh["x"], g.mesh["y"]
    return [(np.exp(-((X - 0.4) ** 2 + Y ** 2) / 2) * np.exp(0.3j * Y)).astype(complex),
            (0.6 * np.exp(-(X ** 2 + (Y + 0.3) ** 2) / 2.5) * np.exp(-0.2j * X)).astype(complex)]


def case_spinor_split2d_32x24():
    """GPEtaskSpinor.solve_split at 32x24: asymmetric g, complex coupling,
    damping with decay, shifted second trap, 3 outer steps of 2 blocks."""
    g = O.Grid(4.0, 32, 3.5, 24)
    V1 = lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2)  # noqa: E731
    V2 = lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2) + 0.3 * X  # noqa: E731
    t = O.GPEtaskSpinor(g, [V1, V2])
    t.g = np.array([[1.0, 0.7], [0.5, 0.8]])
    t.coupling = 0.6 * np.exp(0.7j)
    t.gamma, t.decay_rate, t.Ntotal, t.n_recalc = 0.05, 2.0, 3.0, 5
    p0 = _pair_start(g)
    t.init_state = p0
    t.solve_split(0.004, 10, 3)
    return {"psi0_1": p0[0], "psi0_2": p0[1], "psi_1": t.current_state[0], "psi_2": t.current_state[1],
            "hist_mu": np.real(np.array(t.history["mu"])), "hist_n": np.array(t.history["n"])}


def case_itp_2comp2d_32x24():
    """GPEtask2comp.groundstate_itp at 32x24: N1 = 2, N2 = 1, masses 1 and
    2.5, EE with Ntotal = 3."""
    g = O.Grid(4.0, 32, 3.5, 24)
    V = lambda X, Y, Z: 0.5 * (X ** 2 + 1.3 * Y ** 2)  # noqa: E731
    t = O.GPEtask2comp(g, [V, V])
    t.g = np.array([[1.0, 0.6], [0.6, 0.8]])
    t.N1, t.N2, t.M1, t.M2, t.Ntotal = 2.0, 1.0, 1.0, 2.5, 3.0
    p0 = _pair_start(g)
    phi, MU1, MU2, EE = t.groundstate_itp(0.02, 1e-3, p0, nargout=4)
    return {"psi0_1": p0[0], "psi0_2": p0[1], "phi_1": phi[0], "phi_2": phi[1], "MU1": MU1, "MU2": MU2, "EE": EE}


CASES = {
    "itp_vortex2d_64": case_itp_vortex2d_64,
    "split_damped2d_48": case_split_damped2d_48,
    "split3d_24x32x16": case_split3d_24x32x16,
    "itp3d_adjust_16": case_itp3d_adjust_16,
    "spinor_split2d_32x24": case_spinor_split2d_32x24,
    "itp_2comp2d_32x24": case_itp_2comp2d_32x24,
}


def main():
    for name, fn in CASES.items():
        out = fn()
        np.savez_compressed(path(name), **out)
        print(name, {k: np.shape(v) for k, v in out.items()})


if __name__ == "__main__":
    main()
