"""Coherently coupled two-component condensate (GPEtaskSpinor.solve_split,
lib/@GPEtaskSpinor/solve_split.m:1-119) through the C ABI against the FP64
oracle restatement (oracle.GPEtaskSpinor), same seeded inputs:

* states of both components and the mu / n history: FP64 <= 1e-11, FP32
  <= 2e-5 (relative L2), 2D and 3D, asymmetric g, complex coupling;
* damping with decay and renormalisation, the density-dependent coupling;
* a time-dependent potential (mu evaluated at current_time, as
  GPEtaskSpinor.applyham does) with the outer-step callback, and a resumed run;
* energies (get_energy, <psi|H psi>) and the error statuses;
* the spinor's own imaginary-time solver (groundstate_itp.m): MU, MU2, EE of
  every iteration and the ground state against the oracle (FP64), and the FP32
  ground-state energy.
"""
import numpy as np
import pytest

from oracle import gpe_oracle as O

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.concatenate([np.ravel(x) for x in a])
    b = np.concatenate([np.ravel(x) for x in b])
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def pots(ndims):
    if ndims == 2:
        return [lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2),
                lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2) + 0.3 * X]
    return [lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2 + (1.5 * Z) ** 2),
            lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2 + (1.5 * Z) ** 2) - 0.2 * Y]


def make_pair(gpe, axes, precision, **props):
    nd = 2 if len(axes) == 4 else 3
    grid = gpe.grid2d(*axes, precision=precision) if nd == 2 else gpe.grid3d(*axes, precision=precision)
    task = gpe.GPEtaskSpinor(grid, pots(nd))
    og = O.Grid(*axes)
    ot = O.GPEtaskSpinor(og, pots(nd))
    for k, v in props.items():
        setattr(task, k, v)
        setattr(ot, k, v)
    X, Y = og.mesh["x"], og.mesh["y"]
    p1 = (np.exp(-((X - 0.4) ** 2 + Y ** 2) / 2) * np.exp(0.3j * Y)).astype(complex)
    p2 = (0.6 * np.exp(-(X ** 2 + (Y + 0.3) ** 2) / 2.5) * np.exp(-0.2j * X)).astype(complex)
    task.init_state = [p1, p2]
    ot.init_state = [p1, p2]
    return task, og, ot


G = np.array([[1.0, 0.7], [0.5, 0.8]])
AXES = [(4.0, 48, 3.5, 32), (4.0, 32, 3.5, 24, 2.5, 16)]


@pytest.mark.parametrize("axes", AXES, ids=["2d", "3d"])
@pytest.mark.parametrize("precision", ["double", "single"])
def test_spinor_split_matches_oracle(gpe, axes, precision):
    task, og, ot = make_pair(gpe, axes, precision, g=G, coupling=0.6 * np.exp(0.7j), n_recalc=5)
    task.solve_split(0.004, 10, 3)
    ot.solve_split(0.004, 10, 3)
    tol = 1e-11 if precision == "double" else 2e-5
    assert rel_l2(task.current_state, ot.current_state) < tol
    np.testing.assert_allclose(task.history["n"], ot.history["n"], rtol=tol)
    np.testing.assert_allclose(task.history["mu"], np.real(ot.history["mu"]), rtol=10 * tol)
    assert task.current_iter == 3 and task.current_time == pytest.approx(ot.current_time)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_spinor_damping_decay_and_nonlinear_coupling(gpe, precision):
    task, og, ot = make_pair(gpe, AXES[0], precision, g=G, coupling=0.4, nlincpl=0.25, gamma=0.05,
                             decay_rate=2.0, Ntotal=3.0, n_recalc=5)
    task.solve_split(0.004, 10, 2)
    ot.solve_split(0.004, 10, 2)
    tol = 1e-11 if precision == "double" else 2e-5
    assert rel_l2(task.current_state, ot.current_state) < tol
    np.testing.assert_allclose(task.history["n"], ot.history["n"], rtol=tol)
    np.testing.assert_allclose(task.history["mu"], np.real(ot.history["mu"]), rtol=10 * tol)
    # renormalised to N(t) = Ntotal exp(-time2/tau) at the last block
    n_end = sum(og.integrate(np.abs(p) ** 2) for p in task.current_state)
    assert n_end == pytest.approx(3.0 * np.exp(-task.current_time / 2.0), rel=10 * tol)


def test_spinor_time_dependent_potential_callback_and_resume(gpe):
    task, og, ot = make_pair(gpe, AXES[0], "double", g=G, coupling=0.3 - 0.2j, n_recalc=5)
    vtd = lambda t, time: 0.2 * np.sin(3.0 * time) * og.mesh["x"]
    task.Vtd = vtd
    ot.Vtd = vtd
    seen = []
    task.user_callback = lambda t: seen.append((t.current_iter, t.current_mu))
    task.solve_split(0.004, 10, 2)
    ot.solve_split(0.004, 10, 2)
    assert rel_l2(task.current_state, ot.current_state) < 1e-11
    assert [s[0] for s in seen] == [1, 2]
    np.testing.assert_allclose([s[1] for s in seen], np.real(ot.history["mu"]), rtol=1e-10)
    # resume from current_iter = 2 to 4 (solve_split.m:23-27)
    task.solve_split(0.004, 10, 4)
    ot.solve_split(0.004, 10, 4)
    assert rel_l2(task.current_state, ot.current_state) < 1e-11
    np.testing.assert_allclose(task.history["n"], ot.history["n"], rtol=1e-11)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_spinor_energy_matches_oracle(gpe, precision):
    task, og, ot = make_pair(gpe, AXES[1], precision, g=G, coupling=0.5 + 0.3j)
    phi = ot.init_state
    obs = task.observables(phi)
    tol = 1e-11 if precision == "double" else 2e-6
    assert obs["energy"] == pytest.approx(ot.get_energy(phi), rel=tol)
    mu2 = np.real(ot.inner(phi, ot.applyham(phi)))
    assert obs["mu_integral"] == pytest.approx(mu2, rel=tol)
    c = 0.5 + 0.3j
    assert obs["ecpl"] == pytest.approx(2 * np.real(c * og.inner(phi[0], phi[1])), rel=max(tol, 1e-9))
    assert obs["norm"] == pytest.approx(sum(og.integrate(np.abs(p) ** 2) for p in phi), rel=tol)


def test_spinor_error_statuses(gpe):
    import ctypes as C

    from gpe_gb300 import _lib as L

    task, og, ot = make_pair(gpe, (4.0, 32, 3.5, 32), "single", g=G, n_recalc=10)
    with pytest.raises(gpe.GPEError) as e:
        task.solve_split(0.004, 5, 1)        # floor(5/10) = 0 blocks (solve_split.m:66)
    assert e.value.status == L.GPE_ERR_INVALID
    ch = (C.c_int * 3)()
    assert L.lib.gpe_autotune(task._ctx, 1, ch) == L.GPE_ERR_UNSUPPORTED


@pytest.mark.parametrize("nargout", [4, 2])
def test_spinor_itp_matches_oracle(gpe, nargout):
    """GPEtaskSpinor.groundstate_itp (groundstate_itp.m): MU, MU2, EE of every
    iteration (same count: the convergence decisions coincide) and the ground
    state, FP64; with nargout = 2 the test runs on MU alone."""
    axes = (4.0, 32, 3.5, 24)
    task, og, ot = make_pair(gpe, axes, "double", g=G, coupling=-0.3 + 0.1j, Ntotal=3.0)
    X, Y = og.mesh["x"], og.mesh["y"]
    p0 = [np.exp(-(X ** 2 + Y ** 2) / 2).astype(complex), 0.7 * np.exp(-((X - 0.3) ** 2 + Y ** 2) / 2).astype(complex)]
    out = task.groundstate_itp(0.02, 1e-5, p0, nargout=4)
    ref = ot.groundstate_itp(0.02, 1e-5, p0, nargout=nargout)
    if nargout == 2:
        out = task.groundstate_itp(0.02, 1e-5, p0, nargout=2)
    assert len(out[1]) == len(ref[1])
    np.testing.assert_allclose(out[1], ref[1], rtol=1e-9, atol=1e-11)
    if nargout == 4:
        np.testing.assert_allclose(out[2], ref[2], rtol=1e-10)
        np.testing.assert_allclose(out[3], ref[3], rtol=1e-10)
    assert rel_l2(out[0], ref[0]) < 1e-10
    assert task.last_itp.converged


def test_spinor_itp_fp32_reaches_the_fp64_energy(gpe):
    axes = (4.0, 32, 3.5, 24)
    task, og, ot = make_pair(gpe, axes, "single", g=G, coupling=-0.3, Ntotal=3.0)
    X, Y = og.mesh["x"], og.mesh["y"]
    p0 = [np.exp(-(X ** 2 + Y ** 2) / 2).astype(complex), 0.7 * np.exp(-(X ** 2 + Y ** 2) / 2).astype(complex)]
    phi, MU, MU2, EE = task.groundstate_itp(0.02, 1e-3, p0, nargout=4)
    _, oMU, oMU2, oEE = ot.groundstate_itp(0.02, 1e-3, p0, nargout=4)
    # the two runs may stop at different dt levels (FP32 noise in the test on
    # EE); the ground-state energy agrees to the splitting error there
    assert EE[-1] == pytest.approx(oEE[-1], rel=1e-5)


@pytest.mark.parametrize("nargout", [4, 3])
def test_spinor_rotating_itp_matches_oracle(gpe, nargout):
    """The rotating branch of GPEtaskSpinor.groundstate_itp (groundstate_itp.m:
    30-33, 61-80, 2D): x then y half-step factors with the kx*y*omega and
    ky*x*omega terms on both sides of the nonlinear + coupling factor; MU2 and
    EE add -omega <psi|lz psi> with grid1d's stencil (GPEtaskSpinor.m:72-74).
    FP64 against the oracle, iteration for iteration."""
    task, og, ot = make_pair(gpe, (4.0, 32, 3.5, 24), "double", g=G, coupling=-0.3 + 0.1j, Ntotal=3.0,
                             omega=0.35)
    X, Y = og.mesh["x"], og.mesh["y"]
    p0 = [(np.exp(-(X ** 2 + Y ** 2) / 2) * np.exp(0.3j * X)).astype(complex),
          (0.7 * np.exp(-((X - 0.3) ** 2 + Y ** 2) / 2) * np.exp(-0.2j * Y)).astype(complex)]
    out = task.groundstate_itp(0.02, 1e-5, p0, nargout=nargout)
    ref = ot.groundstate_itp(0.02, 1e-5, p0, nargout=nargout)
    assert len(out[1]) == len(ref[1]) > 20
    np.testing.assert_allclose(out[1], ref[1], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(out[2], ref[2], rtol=1e-10)
    if nargout == 4:
        np.testing.assert_allclose(out[3], ref[3], rtol=1e-10)
    assert rel_l2(out[0], ref[0]) < 1e-10


def test_spinor_rotating_itp_3d_is_refused(gpe):
    from gpe_gb300 import _lib as L

    task, og, ot = make_pair(gpe, AXES[1], "double", g=G, Ntotal=1.0, omega=0.3)
    with pytest.raises(gpe.GPEError) as e:
        task.groundstate_itp(0.02, 1e-5, task.init_state)
    assert e.value.status == L.GPE_ERR_UNSUPPORTED


@pytest.mark.parametrize("axes", AXES, ids=["2d", "3d"])
@pytest.mark.parametrize("precision", ["double", "single"])
def test_spinor_split_with_omega_matches_oracle(gpe, axes, precision):
    """GPEtaskSpinor.solve_split with a scalar omega: the step keeps the plain
    kinetic factor (solve_split.m has no omega) while mu = <psi|H psi>/N adds
    -omega <psi|lz psi> with grid1d's stencil (GPEtaskSpinor.m:72-74), which
    feeds back into the step through mu when gamma > 0."""
    task, og, ot = make_pair(gpe, axes, precision, g=G, coupling=0.4, gamma=0.02, Ntotal=2.0, n_recalc=5,
                             omega=0.3)
    task.solve_split(0.004, 10, 2)
    ot.solve_split(0.004, 10, 2)
    tol = 1e-11 if precision == "double" else 2e-5
    assert rel_l2(task.current_state, ot.current_state) < tol
    np.testing.assert_allclose(task.history["mu"], np.real(ot.history["mu"]), rtol=10 * tol)
    # the Lz term is visible in mu: the same run without it differs
    phi = ot.current_state
    mu_lz = np.real(ot.inner(phi, ot.applyham(phi))) / 2.0
    ot.omega = 0.0
    mu_plain = np.real(ot.inner(phi, ot.applyham(phi))) / 2.0
    assert abs(mu_lz - mu_plain) > 1e-3 * abs(mu_lz)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_spinor_energy_with_omega_matches_oracle(gpe, precision):
    task, og, ot = make_pair(gpe, AXES[0], precision, g=G, coupling=0.5 + 0.3j, omega=0.45)
    X = og.mesh["x"]
    phi = [ot.init_state[0] * np.exp(0.4j * og.mesh["y"]), ot.init_state[1] * np.exp(-0.3j * X)]
    obs = task.observables(phi)
    tol = 1e-11 if precision == "double" else 2e-6
    assert obs["energy"] == pytest.approx(ot.get_energy(phi), rel=tol)
    assert obs["mu_integral"] == pytest.approx(np.real(ot.inner(phi, ot.applyham(phi))), rel=tol)


def test_spinor_split_matches_the_golden_fixture(gpe):
    """The committed fixture tests/golden/spinor_split2d_32x24.npz (the FP64
    oracle's GPEtaskSpinor.solve_split on fixed inputs), FP64."""
    from tests.golden import make_golden as MG

    ref = np.load(MG.path("spinor_split2d_32x24"))
    grid = gpe.grid2d(4.0, 32, 3.5, 24, precision="double")
    task = gpe.GPEtaskSpinor(grid, [lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2),
                                    lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2) + 0.3 * X])
    task.g = np.array([[1.0, 0.7], [0.5, 0.8]])
    task.coupling = 0.6 * np.exp(0.7j)
    task.gamma, task.decay_rate, task.Ntotal, task.n_recalc = 0.05, 2.0, 3.0, 5
    task.init_state = [ref["psi0_1"], ref["psi0_2"]]
    task.solve_split(0.004, 10, 3)
    assert rel_l2(task.current_state, [ref["psi_1"], ref["psi_2"]]) < 1e-11
    np.testing.assert_allclose(task.history["mu"], ref["hist_mu"], rtol=1e-10)
    np.testing.assert_allclose(task.history["n"], ref["hist_n"], rtol=1e-11)
