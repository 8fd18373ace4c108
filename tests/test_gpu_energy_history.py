"""The energy history (an addition: get_energy at every outer step, evaluated on
the device from the block-end sums) against the oracle's get_energy of the
state its ext_callback receives (GPEtask.m:97-107, GPEtaskSpinor.m:98-110):
plain and renormalised (damped) runs, the graph-replayed small-grid path,
FP64 and FP32, and a spinor run."""
import numpy as np
import pytest

from oracle import gpe_oracle as O

pytestmark = pytest.mark.gpu


def energies_of(ot):
    out = []
    ot.user_callback = lambda t: out.append(t.get_energy(t.current_state))
    return out


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("damped", [False, True], ids=["gamma0", "damped"])
def test_energy_history_matches_oracle(gpe, precision, damped):
    axes = (5.0, 48, 4.0, 32)
    V = lambda X, Y, Z: 0.5 * (X ** 2 + 1.3 * Y ** 2)
    grid = gpe.grid2d(*axes, precision=precision)
    task = gpe.GPEtask(grid, V)
    og = O.Grid(*axes)
    ot = O.GPEtask(og, V)
    for t in (task, ot):
        t.g, t.Ntotal = 1.5, 4.0
        if damped:
            t.gamma, t.decay_rate = 0.05, 3.0
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = (np.exp(-((X - 0.3) ** 2 + Y ** 2) / 2) * np.exp(0.4j * Y)).astype(complex)
    task.init_state = psi0
    ot.init_state = psi0
    E = energies_of(ot)
    task.solve_split(0.005, 10, 3)   # no callback: small grid, replayed CUDA graphs
    ot.solve_split(0.005, 10, 3)
    tol = 1e-11 if precision == "double" else 2e-5
    np.testing.assert_allclose(task.history["energy"], E, rtol=tol)
    # with a callback (per-outer-step host path) the same values
    t2 = gpe.GPEtask(grid, V)
    for k in ("g", "Ntotal", "gamma", "decay_rate"):
        setattr(t2, k, getattr(task, k))
    t2.init_state = psi0
    seen = []
    t2.user_callback = lambda t: seen.append(t.history["energy"][t.current_iter - 1])
    t2.solve_split(0.005, 10, 3)
    np.testing.assert_allclose(seen, E, rtol=tol)


def test_spinor_energy_history_matches_oracle(gpe):
    axes = (5.0, 48, 4.0, 32)
    pots = [lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2), lambda X, Y, Z: 0.5 * ((X - 0.3) ** 2 + Y ** 2)]
    task = gpe.GPEtaskSpinor(gpe.grid2d(*axes, precision="double"), pots)
    og = O.Grid(*axes)
    ot = O.GPEtaskSpinor(og, pots)
    for t in (task, ot):
        t.g = np.array([[1.0, 0.6], [0.6, 0.9]])
        t.coupling, t.gamma, t.Ntotal, t.n_recalc = 0.4 + 0.1j, 0.02, 3.0, 5
    X, Y = og.mesh["x"], og.mesh["y"]
    p = np.exp(-(X ** 2 + Y ** 2) / 2).astype(complex)
    task.init_state = [p, 0.5 * p * np.exp(0.3j * X)]
    ot.init_state = [p, 0.5 * p * np.exp(0.3j * X)]
    E = energies_of(ot)
    task.solve_split(0.004, 10, 2)
    ot.solve_split(0.004, 10, 2)
    np.testing.assert_allclose(task.history["energy"], E, rtol=1e-11)
