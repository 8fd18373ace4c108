"""Incoherent two-component mixture (GPEtask2comp.groundstate_itp,
lib/@GPEtask2comp/groundstate_itp.m:1-157) through the C ABI
(gpe_groundstate_itp_2comp) against the FP64 oracle restatement
(oracle.GPEtask2comp), same seeded inputs:

* MU1, MU2 (each component's own normalisation factor) and EE of every
  iteration, and both ground-state components: FP64 to 1e-10, 2D and 3D;
* equal masses (one kinetic launch over both components) and unequal masses
  (one launch per component with its own exp(-kk dt/2/M_j) tables);
* nargout = 2, where the convergence test runs on MU2 instead of EE;
* FP32 reaches the FP64 ground-state energy;
* the rotating branch (scalar omega, 2D) with equal and unequal masses;
* the error statuses (coupling set, omega in 3D, a one-component context).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import gpe_oracle as O

pytestmark = pytest.mark.gpu

G = np.array([[1.0, 0.6], [0.6, 0.8]])


def rel_l2(a, b):
    a = np.concatenate([np.ravel(x) for x in a])
    b = np.concatenate([np.ravel(x) for x in b])
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def pots(nd):
    if nd == 2:
        return [lambda X, Y, Z: 0.5 * (X ** 2 + 1.3 * Y ** 2), lambda X, Y, Z: 0.5 * (X ** 2 + 1.3 * Y ** 2) + 0.2 * X]
    return [lambda X, Y, Z: 0.5 * (X ** 2 + 1.3 * Y ** 2 + (1.5 * Z) ** 2),
            lambda X, Y, Z: 0.5 * (X ** 2 + 1.3 * Y ** 2 + (1.5 * Z) ** 2) - 0.2 * Y]


def make_pair(gpe, axes, precision, **props):
    nd = 2 if len(axes) == 4 else 3
    grid = gpe.grid2d(*axes, precision=precision) if nd == 2 else gpe.grid3d(*axes, precision=precision)
    task = gpe.GPEtask2comp(grid, pots(nd))
    og = O.Grid(*axes)
    ot = O.GPEtask2comp(og, pots(nd))
    for k, v in dict(g=G, N1=2.0, N2=1.0, Ntotal=3.0, **props).items():
        setattr(task, k, v)
        setattr(ot, k, v)
    X, Y = og.mesh["x"], og.mesh["y"]
    p0 = [np.exp(-((X - 0.3) ** 2 + Y ** 2) / 2).astype(complex),
          (0.5 * np.exp(-(X ** 2 + (Y + 0.2) ** 2) / 3) * np.exp(0.2j * X)).astype(complex)]
    return task, og, ot, p0


@pytest.mark.parametrize("masses", [(1.0, 1.0), (1.0, 2.5)], ids=["equal_mass", "unequal_mass"])
@pytest.mark.parametrize("axes", [(4.0, 32, 3.5, 24), (4.0, 24, 3.5, 16, 3.0, 16)], ids=["2d", "3d"])
def test_2comp_itp_matches_oracle(gpe, axes, masses):
    task, og, ot, p0 = make_pair(gpe, axes, "double", M1=masses[0], M2=masses[1])
    phi, MU1, MU2, EE = task.groundstate_itp(0.02, 1e-5, p0, nargout=4)
    ophi, oMU1, oMU2, oEE = ot.groundstate_itp(0.02, 1e-5, p0, nargout=4)
    assert len(MU1) == len(oMU1) > 20
    np.testing.assert_allclose(MU1, oMU1, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(MU2, oMU2, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(EE, oEE, rtol=1e-10)
    assert rel_l2(phi, ophi) < 1e-10
    # each component normalised to its own N_j (groundstate_itp.m:82-90)
    np.testing.assert_allclose([og.integrate(np.abs(p) ** 2) for p in phi], [2.0, 1.0], rtol=1e-12)
    assert task.last_itp.converged and task.last_itp.final_dt == pytest.approx(ot.final_dt)


def test_2comp_itp_nargout2_tests_on_mu2(gpe):
    task, og, ot, p0 = make_pair(gpe, (4.0, 32, 3.5, 24), "double", M1=1.0, M2=1.7)
    phi, MU1 = task.groundstate_itp(0.02, 1e-5, p0, nargout=2)
    ophi, oMU1, oMU2, oEE = ot.groundstate_itp(0.02, 1e-5, p0, nargout=2)
    assert len(MU1) == len(oMU1)
    np.testing.assert_allclose(MU1, oMU1, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(oEE, oMU2)  # EE(i) = MU2(i) without nargout >= 4
    assert rel_l2(phi, ophi) < 1e-10


def test_2comp_itp_fp32_reaches_the_fp64_energy(gpe):
    task, og, ot, p0 = make_pair(gpe, (4.0, 32, 3.5, 24), "single", M1=1.0, M2=2.0)
    phi, MU1, MU2, EE = task.groundstate_itp(0.02, 1e-3, p0, nargout=4)
    _, oMU1, oMU2, oEE = ot.groundstate_itp(0.02, 1e-3, p0, nargout=4)
    assert EE[-1] == pytest.approx(oEE[-1], rel=1e-5)
    assert MU1[-1] == pytest.approx(oMU1[-1], rel=1e-4)


def test_2comp_error_statuses(gpe):
    from gpe_gb300 import _lib as L

    task, og, ot, p0 = make_pair(gpe, (4.0, 32, 3.5, 24), "double")
    task.coupling = 0.2
    with pytest.raises(ValueError):
        task.groundstate_itp(0.02, 1e-5, p0)
    task.coupling = 0.0
    one = gpe.GPEtask(gpe.grid2d(4.0, 32, 3.5, 24), lambda X, Y, Z: 0 * X)
    one.init_state = np.ones(one.grid.shape, complex)
    one._push_params()
    one._upload_V(one.Vtrap)
    one._upload_state(one.init_state)
    prm = L.gpe_itp_params()
    prm.dt, prm.eps = 0.02, 1e-5
    res = L.gpe_itp_result()
    st = L.lib.gpe_groundstate_itp_2comp(one._ctx, C.byref(prm), 1.0, 1.0, 1.0, 1.0, None, None, None, 0,
                                         C.byref(res))
    assert st == L.GPE_ERR_UNSUPPORTED


@pytest.mark.parametrize("masses", [(1.0, 1.0), (1.0, 2.5)], ids=["equal_mass", "unequal_mass"])
def test_2comp_rotating_itp_matches_oracle(gpe, masses):
    """The rotating branch of GPEtask2comp.groundstate_itp (groundstate_itp.m:
    31-36, 61-80, 2D): x then y half steps before the nonlinear factor, y then
    x after it, each with its component's mass; EE from lap(phi, omega)
    (GPEtask2comp.m:60).  FP64 against the oracle, iteration for iteration."""
    task, og, ot, p0 = make_pair(gpe, (4.0, 32, 3.5, 24), "double", M1=masses[0], M2=masses[1], omega=0.3)
    X = og.mesh["x"]
    p0 = [p0[0] * np.exp(0.25j * X), p0[1]]
    phi, MU1, MU2, EE = task.groundstate_itp(0.02, 1e-5, p0, nargout=4)
    ophi, oMU1, oMU2, oEE = ot.groundstate_itp(0.02, 1e-5, p0, nargout=4)
    assert len(MU1) == len(oMU1) > 20
    np.testing.assert_allclose(MU1, oMU1, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(MU2, oMU2, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(EE, oEE, rtol=1e-10)
    assert rel_l2(phi, ophi) < 1e-10


def test_2comp_rotating_itp_3d_is_refused(gpe):
    from gpe_gb300 import _lib as L

    task, og, ot, p0 = make_pair(gpe, (4.0, 24, 3.5, 16, 3.0, 16), "double", omega=0.3)
    with pytest.raises(gpe.GPEError) as e:
        task.groundstate_itp(0.02, 1e-5, p0)
    assert e.value.status == L.GPE_ERR_UNSUPPORTED


def test_2comp_itp_matches_the_golden_fixture(gpe):
    """The committed fixture tests/golden/itp_2comp2d_32x24.npz (the FP64
    oracle's GPEtask2comp.groundstate_itp on fixed inputs), FP64."""
    from tests.golden import make_golden as MG

    ref = np.load(MG.path("itp_2comp2d_32x24"))
    grid = gpe.grid2d(4.0, 32, 3.5, 24, precision="double")
    V = lambda X, Y, Z: 0.5 * (X ** 2 + 1.3 * Y ** 2)  # noqa: E731
    task = gpe.GPEtask2comp(grid, [V, V])
    task.g = np.array([[1.0, 0.6], [0.6, 0.8]])
    task.N1, task.N2, task.M1, task.M2, task.Ntotal = 2.0, 1.0, 1.0, 2.5, 3.0
    phi, MU1, MU2, EE = task.groundstate_itp(0.02, 1e-3, [ref["psi0_1"], ref["psi0_2"]], nargout=4)
    assert len(MU1) == len(ref["MU1"])
    np.testing.assert_allclose(MU1, ref["MU1"], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(MU2, ref["MU2"], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(EE, ref["EE"], rtol=1e-10)
    assert rel_l2(phi, [ref["phi_1"], ref["phi_2"]]) < 1e-10
