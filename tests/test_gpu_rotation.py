"""Rotating frame (scalar omega): the x half / y / z / x half kinetic step of
ssft_kin_step.m:12-15 with the factors of set_kinop.m:5-7, and the rotating
Hamiltonian of lap.m:8-10 in the energy sums, against the FP64 oracle.

Tolerances: FP64 kernels rel. L2 / scalars <= 1e-11; FP32 <= 2e-5 (state),
1e-6 (energy and mu of a ground state).
"""
import numpy as np
import pytest

from oracle import gpe_oracle as O

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def pair(gpe, axes, precision, V, **props):
    grid = gpe.grid2d(*axes, precision=precision) if len(axes) == 4 else gpe.grid3d(*axes, precision=precision)
    task = gpe.GPEtask(grid, V)
    og = O.Grid(*axes)
    ot = O.GPEtask(og, V)
    for k, v in props.items():
        setattr(task, k, v)
        setattr(ot, k, v)
    return task, og, ot


def trap2(X, Y, Z):
    return 0.5 * (X ** 2 + 1.3 * Y ** 2)


def trap3(X, Y, Z):
    return 0.5 * (X ** 2 + 1.3 * Y ** 2 + (1.5 * Z) ** 2)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_rotating_itp_2d(gpe, precision):
    task, og, ot = pair(gpe, (4.0, 48, 3.5, 32), precision, trap2, Ntotal=20.0, g=1.0, omega=0.5,
                        itp_max_iter=400)
    X, Y = og.mesh["x"], og.mesh["y"]
    phi0 = (np.exp(-(X ** 2 + Y ** 2) / 2) * (1 + 0.3 * (X + 1j * Y))).astype(complex)
    phi, MU, MU2, EE = task.groundstate_itp(0.01, 1e-8, phi0, nargout=4)
    ophi, oMU, oMU2, oEE = ot.groundstate_itp(0.01, 1e-8, phi0, nargout=4)
    if precision == "double":
        assert len(MU) == len(oMU)
        np.testing.assert_allclose(MU, oMU, rtol=1e-11)
        chk = oMU2 != 0
        np.testing.assert_allclose(EE[chk], oEE[chk], rtol=1e-11)
        assert rel_l2(phi, ophi) < 1e-11
    else:
        assert EE[-1] == pytest.approx(oEE[-1], rel=1e-6)
        assert MU[-1] == pytest.approx(oMU[-1], rel=1e-6)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_rotating_damped_dynamics_3d(gpe, precision):
    """gamma > 0 feeds mu back every block, so the rotating-frame energy
    weights of the energy passes enter the result."""
    task, og, ot = pair(gpe, (4.0, 32, 3.5, 24, 2.5, 16), precision, trap3, Ntotal=15.0, g=1.0, omega=0.6,
                        gamma=0.02)
    X, Y, Z = og.mesh["x"], og.mesh["y"], og.mesh["z"]
    psi0 = (np.exp(-((X - 0.5) ** 2 + Y ** 2 + Z ** 2) / 2) * np.exp(0.4j * Y)).astype(complex)
    task.init_state = psi0
    ot.init_state = psi0
    task.solve_split(0.003, 10, 3)
    ot.solve_split(0.003, 10, 3)
    tol = 1e-11 if precision == "double" else 2e-5
    assert rel_l2(task.current_state, ot.current_state) < tol
    np.testing.assert_allclose(task.history["mu"], ot.history["mu"], rtol=tol)
    np.testing.assert_allclose(task.history["n"], ot.history["n"], rtol=tol)


def test_rotating_observables_match_applyham(gpe):
    task, og, ot = pair(gpe, (4.0, 32, 3.5, 24, 2.5, 16), "double", trap3, g=0.7, omega=-0.8)
    rng = np.random.default_rng(5)
    X, Y, Z = og.mesh["x"], og.mesh["y"], og.mesh["z"]
    psi = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2) * (1 + 0.1 * rng.standard_normal(og.shape)) * np.exp(0.3j * X)
    o = task.observables(psi)
    assert o["energy"] == pytest.approx(ot.get_energy(psi), rel=1e-12)
    assert o["mu_integral"] == pytest.approx(np.real(og.inner(psi, ot.applyham(psi))), rel=1e-12)


def test_rotating_frame_large_grid_and_adjoint_rejected(gpe):
    """A grid above the graph-replay size (separate launches per block) and
    the adjoint's refusal of omega != 0."""
    from gpe_gb300 import _lib as L

    task, og, ot = pair(gpe, (6.0, 128, 6.0, 128, 4.0, 64), "double", trap3, g=0.5, omega=0.3)
    X, Y, Z = og.mesh["x"], og.mesh["y"], og.mesh["z"]
    psi0 = (np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 3) * np.exp(0.2j * X)).astype(complex)
    task.init_state = psi0
    ot.init_state = psi0
    task.solve_split(0.002, 5, 1)
    ot.solve_split(0.002, 5, 1)
    assert rel_l2(task.current_state, ot.current_state) < 1e-11
    with pytest.raises(gpe.GPEError) as e:
        task.adjoint_grad(psi0, 0.002, 3, phi0=psi0)
    assert e.value.status == L.GPE_ERR_UNSUPPORTED
