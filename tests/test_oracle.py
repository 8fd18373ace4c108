"""CPU checks of the FP64 oracle (oracle/gpe_oracle.py).

The reference ships no tests or golden vectors and MATLAB is absent, so the
oracle is pinned to analytic known answers of the Gross-Pitaevskii equation
and of the reference's split-step scheme, plus the committed golden fixtures
(regression pins of the oracle itself, tests/golden/make_golden.py).
"""
import math

import numpy as np
import pytest

from oracle import gpe_oracle as O


def harmonic(lam=(1.0, 1.0, 1.0)):
    def V(X, Y, Z):
        return 0.5 * ((lam[0] * X) ** 2 + (lam[1] * Y) ** 2 + (lam[2] * Z) ** 2)
    return V


def test_grid_matches_matlab_definitions():
    g = O.Grid(17, 8, 5, 12)
    assert g.shape == (8, 12)
    x = np.linspace(-17, 17, 8)
    dx = x[1] - x[0]
    L = x[-1] - x[0] + dx
    np.testing.assert_allclose(g.kx1, np.array([0, 1, 2, 3, 4, -3, -2, -1]) * 2 * np.pi / L, rtol=0, atol=1e-15)
    assert g.weight == pytest.approx(dx * (10 / 11))
    # meshgrid layout: X varies along axis 0 (MATLAB columns), Y along axis 1 (rows, contiguous)
    assert np.all(g.mesh["x"][:, 0] == g.x) and np.all(g.mesh["y"][0, :] == g.y)
    g3 = O.Grid(1, 8, 2, 8, 3, 12)
    assert g3.shape == (12, 8, 8)
    assert g3.kk.shape == g3.shape
    assert g3.kk[0, 0, 1] == pytest.approx(g3.ky1[1] ** 2 / 2)


def test_fft_convention_unnormalised_forward():
    g = O.Grid(4, 16, 4, 16)
    a = np.ones(g.shape, dtype=complex)
    assert g.fft(a)[0, 0] == pytest.approx(256)
    np.testing.assert_allclose(g.ifft(g.fft(a)), a, atol=1e-14)


@pytest.mark.parametrize("dt", [0.01])
def test_itp_harmonic_2d_ground_state_energy(dt):
    # g = 0, omega = 1: mu = E/N = 1 (two 1/2 zero-point energies).
    g = O.Grid(8, 64, 8, 64)
    t = O.GPEtask(g, harmonic())
    t.Ntotal = 1.0
    t.g = 0.0
    phi0 = np.exp(-((g.mesh["x"] - 0.3) ** 2 + g.mesh["y"] ** 2) / 3.0).astype(complex)
    phi, MU, MU2, EE = t.groundstate_itp(dt, 1e-9, phi0)
    assert MU[-1] == pytest.approx(1.0, abs=5e-5)        # Strang error O(dt^2)
    assert EE[-1] == pytest.approx(1.0, abs=1e-7)        # variational: O(dt^4)
    assert MU2[-1] == pytest.approx(1.0, abs=1e-7)
    assert g.integrate(np.abs(phi) ** 2) == pytest.approx(1.0, rel=1e-12)


def test_itp_anisotropic_3d_ground_state_energy():
    # g = 0, lambda = 4: mu = (1 + 1 + 4)/2 = 3.
    g = O.Grid(6, 32, 6, 32, 6, 32)
    t = O.GPEtask(g, harmonic((1, 1, 4)))
    t.Ntotal = 1.0
    t.g = 0.0
    X, Y, Z = g.mesh["x"], g.mesh["y"], g.mesh["z"]
    phi0 = np.exp(-(X ** 2 + Y ** 2 + 4 * Z ** 2) / 1.5).astype(complex)
    phi, MU, MU2, EE = t.groundstate_itp(0.005, 1e-8, phi0)
    assert EE[-1] == pytest.approx(3.0, abs=1e-5)        # grid + convergence error
    assert MU[-1] == pytest.approx(3.0, abs=1e-4)


def test_itp_thomas_fermi_limit_2d():
    # Large gN: mu -> sqrt(g N / pi) for V = r^2/2 (loose, kinetic energy neglected).
    g = O.Grid(17, 128, 17, 128)
    t = O.GPEtask(g, harmonic())
    t.Ntotal = 1e5
    t.g = 0.06
    phi0 = np.exp(-(g.mesh["x"] ** 2 + g.mesh["y"] ** 2) / 32).astype(complex)
    phi, MU = t.groundstate_itp(0.02, 1e-6, phi0, nargout=2)[:2]
    assert MU[-1] == pytest.approx(math.sqrt(0.06 * 1e5 / math.pi), rel=2e-3)


def test_split_plane_wave_is_exact():
    # V = 0, g = 0: a grid plane wave only acquires exp(-i (k^2/2 - mu) t).
    g = O.Grid(5, 32, 5, 32)
    t = O.GPEtask(g, lambda X, Y, Z: 0 * X)
    kx, ky = g.kx1[3], g.ky1[-2]
    psi0 = np.exp(1j * (kx * g.mesh["x"] + ky * g.mesh["y"]))
    t.init_state = psi0
    t.mu_init = 0.3
    t.solve_split(0.01, 20, 3)
    T = 0.01 * 20 * 3
    expect = psi0 * np.exp(-1j * ((kx ** 2 + ky ** 2) / 2 - 0.3) * T)
    np.testing.assert_allclose(t.current_state, expect, rtol=0, atol=1e-12)


@pytest.mark.parametrize("axes", [(5.0, 32, 6.0, 24), (5.0, 16, 6.0, 24, 4.0, 12)])
def test_kinetic_step_factorises_over_axes_in_any_order(axes):
    """The kinetic step exp(-kk dt) applied in Fourier space
    (ssft_kin_step.m:17) equals one 1D transform / factor / inverse per axis,
    in any order of the axes: the property the CUDA passes rely on, one pass
    per axis and consecutive split steps taking the axes in opposite orders
    (the folded steps).  Complex dt of a damped run (gamma = 0.05)."""
    g = O.Grid(*axes)
    t = O.GPEtask(g, harmonic())
    dt = 0.01j / (1 + 0.05j)
    t.set_kinop(dt)
    rng = np.random.default_rng(7)
    psi = rng.standard_normal(g.shape) + 1j * rng.standard_normal(g.shape)
    full = t.ssft_kin_step(psi, dt)
    names = ["x", "y", "z"][: len(axes) // 2]
    k = {"x": g.KX, "y": g.KY, "z": g.KZ}
    for order in (names, names[::-1], names[1:] + names[:1]):
        phi = psi
        for ax in order:
            phi = g.ifft1(np.exp(-k[ax] ** 2 / 2 * dt) * g.fft1(phi, ax), ax)
        np.testing.assert_allclose(phi, full, rtol=0, atol=1e-12 * np.abs(full).max())


def test_split_gamma0_conserves_norm_and_is_time_reversible():
    g = O.Grid(6, 32, 6, 32)
    t = O.GPEtask(g, harmonic((1.0, 1.3, 1.0)))
    t.g = 2.0
    t.mu_init = 1.5  # a fixed mu: the state-derived mu is not time-symmetric
    rng = np.random.default_rng(5)
    psi0 = np.exp(-(g.mesh["x"] ** 2 + g.mesh["y"] ** 2) / 4) * (1 + 0.1 * rng.standard_normal(g.shape))
    psi0 = psi0 * np.exp(0.4j * g.mesh["x"])
    t.init_state = psi0
    t.solve_split(0.005, 10, 4)
    n0 = g.integrate(np.abs(psi0) ** 2)
    np.testing.assert_allclose(t.history["n"], n0, rtol=1e-12)
    # conj -> propagate -> conj returns the start (symmetric Strang, gamma = 0)
    back = O.GPEtask(g, harmonic((1.0, 1.3, 1.0)))
    back.g = 2.0
    back.mu_init = 1.5
    back.init_state = np.conj(t.current_state)
    back.solve_split(0.005, 10, 4)
    np.testing.assert_allclose(np.conj(back.current_state), psi0, rtol=0, atol=1e-11)


def test_split_damping_renormalises_and_decays():
    g = O.Grid(6, 32, 6, 32)
    t = O.GPEtask(g, harmonic())
    t.g = 1.0
    t.Ntotal = 50.0
    t.gamma = 0.05
    t.decay_rate = 2.0
    phi0 = np.exp(-(g.mesh["x"] ** 2 + g.mesh["y"] ** 2) / 4).astype(complex)
    t.init_state = math.sqrt(50) * g.normalize(phi0)
    t.solve_split(0.01, 10, 3)
    # after renormalisation the norm is NNN = N0 exp(-time2/tau) of the last block
    assert g.integrate(np.abs(t.current_state) ** 2) == pytest.approx(50 * math.exp(-t.current_time / 2.0),
                                                                     rel=1e-12)


def test_vortex_imprint_matches_example():
    g = O.Grid(8, 32, 8, 32)
    phi = np.ones(g.shape, complex) * 2.0
    out = O.imprint_vortex(g, phi, 0.5, 1.0)
    xi = 1 / math.sqrt(2 * 0.5 * 4.0)
    X, Y = g.mesh["x"], g.mesh["y"]
    np.testing.assert_allclose(np.abs(out), 2 * np.tanh(np.sqrt((X - 1) ** 2 + Y ** 2) / xi))
    np.testing.assert_allclose(np.angle(out[5, 20]), np.arctan2(X[5, 20] - 1, Y[5, 20]))


@pytest.mark.parametrize("axes", [(8, 32, 8, 32), (6, 16, 6, 12, 4, 8)], ids=["2d", "3d"])
def test_oracle_adjoint_matches_central_differences(axes):
    """The oracle's reverse sweep against central differences of its own
    forward (step 1e-5): directional derivatives within 1e-7 relative."""
    g = O.Grid(*axes)
    X, Y, Z = g.mesh["x"], g.mesh["y"], g.mesh["z"]
    V = 0.5 * (X ** 2 + Y ** 2 + (Z ** 2 if len(axes) == 6 else 0.0))
    psi0 = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 4).astype(complex) * (1 + 0.1j * X)
    tgt = np.exp(-((X - 1) ** 2 + Y ** 2) / 4).astype(complex) * np.exp(1j * np.arctan2(X - 1, Y))
    coupling, ddt, M = 0.5, 0.01, 20
    loss, dV = O.adjoint_grad(g, V, coupling, psi0, tgt, ddt, M)
    assert 0 < loss < 1
    rng = np.random.default_rng(7)
    eps = 1e-5
    for _ in range(3):
        d = rng.standard_normal(g.shape)
        lp = O.overlap_loss(g, tgt, O.split_forward(g, V + eps * d, coupling, psi0, ddt, M)[0], psi0)[0]
        lm = O.overlap_loss(g, tgt, O.split_forward(g, V - eps * d, coupling, psi0, ddt, M)[0], psi0)[0]
        ad = float(np.sum(dV * d))
        assert abs((lp - lm) / (2 * eps) - ad) < 1e-7 * abs(ad)


def test_rotating_frame_keeps_the_isotropic_ground_state():
    """Scalar omega (set_kinop.m:5-7, ssft_kin_step.m:12-15, lap.m:8-9): the
    nodeless ground state of an isotropic trap has Lz psi = 0, so a slowly
    rotating frame leaves the ITP fixed point and its energy unchanged."""
    g = O.Grid(6, 32, 6, 32)
    X, Y = g.mesh["x"], g.mesh["y"]
    out = []
    for om in (0.0, 0.3):
        t = O.GPEtask(g, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2))
        t.Ntotal, t.g, t.omega = 10.0, 1.0, om
        phi = t.groundstate_itp(0.01, 1e-9, np.exp(-(X ** 2 + Y ** 2) / 2).astype(complex), nargout=1)[0]
        out.append((phi, t.get_energy(phi)))
    assert np.linalg.norm(out[1][0] - out[0][0]) / np.linalg.norm(out[0][0]) < 1e-5
    assert out[1][1] == pytest.approx(out[0][1], rel=1e-9)


def test_rotating_frame_dynamics_conserve_norm_and_energy():
    """gamma = 0 in a rotating anisotropic trap: the split step conserves the
    norm exactly and the rotating-frame energy to the splitting error."""
    g = O.Grid(6, 32, 6, 32, 4, 16)
    t = O.GPEtask(g, lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2 + Z ** 2))
    t.g, t.omega = 1.0, 0.4
    X, Y, Z = g.mesh["x"], g.mesh["y"], g.mesh["z"]
    psi = np.exp(-((X - 1) ** 2 + Y ** 2 + Z ** 2) / 2).astype(complex) * np.exp(0.2j * Y)
    t.init_state = psi
    E0 = t.get_energy(psi)
    phi = t.solve_split(0.002, 20, 2)
    assert g.integrate(np.abs(phi) ** 2) == pytest.approx(g.integrate(np.abs(psi) ** 2), rel=1e-12)
    assert t.get_energy(phi) == pytest.approx(E0, rel=1e-6)


def test_sgpe_zero_temperature_is_gpe_up_to_a_global_phase():
    """SGPEtask at T = 0, gamma = 0 (lib/@SGPEtask/solve_split.m): mu stays at
    mu_init while GPEtask uses <psi|H psi>/N; mu only adds a global phase at
    gamma = 0, so |psi| agrees with GPEtask's."""
    g = O.Grid(5, 32, 4, 24)
    V = lambda X, Y, Z: 0.5 * (X ** 2 + 1.3 * Y ** 2)
    X, Y = g.mesh["x"], g.mesh["y"]
    psi0 = (np.exp(-((X - 0.5) ** 2 + Y ** 2) / 2) * np.exp(0.3j * Y)).astype(complex)
    a, b = O.GPEtask(g, V), O.SGPEtask(g, V)
    for t in (a, b):
        t.g = 1.0
        t.init_state = psi0
    pa = a.solve_split(0.005, 10, 2)
    pb = b.solve_split(0.005, 10, 2)
    np.testing.assert_allclose(np.abs(pb), np.abs(pa), rtol=0, atol=1e-12)
    assert b.history["mu"] == [0.0, 0.0]


def test_sgpe_energy_cutoff_masks_the_noise_spectrum():
    """With T > 0 and ecut > 0 (solve_split.m:40-42) one step of pure noise
    from psi = 0 (V = g = mu = 0) has no mode with kk >= ecut; with T = 0 the
    cut-off is not applied."""
    g = O.Grid(8, 32, 8, 32)
    t = O.SGPEtask(g, lambda X, Y, Z: 0 * X)
    t.gamma, t.T, t.ecut, t.n_recalc = 0.2, 2.0, 0.3 * g.kk.max(), 1
    t.init_state = np.zeros(g.shape, complex)
    spec = np.abs(g.fft(t.solve_split(0.01, 1, 1, rng=np.random.default_rng(3))))
    kept = g.kk < t.ecut
    assert 0 < kept.sum() < kept.size
    assert spec[~kept].max() < 1e-12 * spec[kept].max()
    t.T, t.current_iter = 0.0, 0
    psi0 = np.exp(-(g.mesh["x"] ** 2 + g.mesh["y"] ** 2)).astype(complex)
    t.init_state = psi0
    a = t.solve_split(0.01, 2, 1)
    t.ecut, t.current_iter = 0.0, 0
    np.testing.assert_array_equal(t.solve_split(0.01, 2, 1), a)


def test_spinor_rabi_oscillation_is_exact():
    """GPEtaskSpinor.solve_split (lib/@GPEtaskSpinor/solve_split.m) with V = 0,
    g = 0 and a uniform state: the kinetic factors leave k = 0 alone, mu is a
    common phase, and the coupling matrix of each step is exp(-i H_c ddt),
    H_c = [[0, c], [conj(c), 0]], so the populations follow cos^2(|c| t)."""
    g = O.Grid(4, 16, 4, 16)
    t = O.GPEtaskSpinor(g, [lambda X, Y, Z: 0 * X, lambda X, Y, Z: 0 * X])
    t.coupling = 0.7 * np.exp(0.4j)
    t.init_state = [np.ones(g.shape, complex), np.zeros(g.shape, complex)]
    ddt, nin, nout = 0.01, 10, 3
    t.solve_split(ddt, nin, nout)
    N = g.integrate(np.ones(g.shape))
    n1 = g.integrate(np.abs(t.current_state[0]) ** 2)
    assert n1 / N == pytest.approx(math.cos(0.7 * ddt * nin * nout) ** 2, abs=1e-12)
    ratio = t.current_state[1][3, 5] / t.current_state[0][3, 5]
    # phi2/phi1 = -i tan(|c| t) exp(-i arg c)
    assert ratio == pytest.approx(-1j * math.tan(0.7 * ddt * nin * nout) * np.exp(-0.4j), abs=1e-12)
    np.testing.assert_allclose(t.history["n"], N, rtol=1e-12)


def test_spinor_conserves_norm_and_matches_single_component_when_decoupled():
    """gamma = 0: the step is unitary (real coupling with nlincpl as well).
    Decoupled (coupling = nlincpl = 0, g diagonal, V2 = V1) with phi2 = 0, the
    first component evolves as GPEtask with the kinetic-first splitting
    K/2 (N K)^n K^-1/2 of solve_split.m:72-99."""
    g = O.Grid(5, 32, 5, 24)
    V = lambda X, Y, Z: 0.5 * (X ** 2 + 1.3 * Y ** 2)
    X, Y = g.mesh["x"], g.mesh["y"]
    p1 = np.exp(-((X - 0.4) ** 2 + Y ** 2) / 2) * np.exp(0.3j * Y)
    p2 = 0.5 * np.exp(-(X ** 2 + (Y - 0.5) ** 2) / 3)
    t = O.GPEtaskSpinor(g, [V, lambda X, Y, Z: V(X, Y, Z) + 0.2 * X])
    t.g = np.array([[1.0, 0.6], [0.6, 0.8]])
    t.coupling, t.nlincpl = 0.3, 0.2
    t.init_state = [p1, p2]
    t.solve_split(0.005, 10, 2)
    N0 = g.integrate(np.abs(p1) ** 2 + np.abs(p2) ** 2)
    np.testing.assert_allclose(t.history["n"], N0, rtol=1e-12)
    # decoupled: one component against a direct restatement of the splitting
    d = O.GPEtaskSpinor(g, [V, V])
    d.g = np.diag([1.0, 0.5])
    d.init_state = [p1, np.zeros(g.shape, complex)]
    d.solve_split(0.005, 10, 1)
    dt = 0.005j
    mu = np.real(g.inner(p1, g.lap(p1) + (V(X, Y, 0) + np.abs(p1) ** 2) * p1)) / g.integrate(np.abs(p1) ** 2)
    ph = g.ifft(np.exp(-g.kk * dt / 2) * g.fft(p1))
    for _ in range(10):
        ph = np.exp(-(V(X, Y, 0) - mu + np.abs(ph) ** 2) * dt) * ph
        ph = g.ifft(np.exp(-g.kk * dt) * g.fft(ph))
    ph = g.ifft(np.exp(g.kk * dt / 2) * g.fft(ph))
    np.testing.assert_allclose(d.current_state[0], ph, rtol=0, atol=1e-12)
    assert np.max(np.abs(d.current_state[1])) == 0


def vortex_field(g, cores, width=2.5):
    """A Gaussian with a core z/sqrt(1 + |z|^2), z = (x - x_k) + i s_k (y - y_k),
    at each (x_k, y_k, s_k)."""
    X, Y = g.mesh["x"], g.mesh["y"]
    phi = np.exp(-(X ** 2 + Y ** 2) / (2 * width ** 2)).astype(complex)
    for xk, yk, sk in cores:
        z = (X - xk) + 1j * sk * (Y - yk)
        phi = phi * z / np.sqrt(1.0 + np.abs(z) ** 2)
    return phi


def test_detect_core_finds_charges_and_refines_positions():
    """lib/util/detect_core.m: charges and positions of imprinted cores (the
    centre (x_j - dx/2, y_i - dy/2) of the plaquette holding the core);
    refine = 1 (Phillips et al.) recovers the zeros to a few % of a cell."""
    g = O.Grid(8, 64, 8, 64)
    cores = [(-2.03, 1.51, 1), (1.27, -0.88, -1), (2.55, 2.14, 1)]
    phi = vortex_field(g, cores)
    rx, ry = g.mesh["x"], g.mesh["y"]
    resp, resm = O.detect_core(phi, rx, ry)
    assert resp.shape == (2, 2) and resm.shape == (1, 2)
    for pts, sgn in ((resp, 1), (resm, -1)):
        for x, y in pts:
            near = [c for c in cores if c[2] == sgn and abs(c[0] - x) <= g.dx / 2 and abs(c[1] - y) <= g.dy / 2]
            assert len(near) == 1
    # MATLAB find() order: column-major over (row = y, column = x) -> ascending x first
    assert resp[0, 0] < resp[1, 0]
    rp, rm = O.detect_core(phi, rx, ry, refine=1)
    truth_p = sorted([c[:2] for c in cores if c[2] == 1])
    np.testing.assert_allclose(sorted(map(tuple, rp)), truth_p, atol=0.05 * g.dx)
    np.testing.assert_allclose(rm, [cores[1][:2]], atol=0.05 * g.dx)
    # no cores: empty k x 2 arrays
    e1, e2 = O.detect_core(vortex_field(g, []), rx, ry)
    assert e1.shape == (0, 2) and e2.shape == (0, 2)


def test_del2_matches_matlab_edge_extrapolation():
    """del2 of a quadratic is exact everywhere (edges included): for
    U = a x^2 + b y^2 it is (2a + 2b)/4."""
    g = O.Grid(3, 16, 2, 12)
    U = 0.7 * g.mesh["x"] ** 2 + 1.9 * g.mesh["y"] ** 2
    np.testing.assert_allclose(O.del2(U, g.dx, g.dy), (2 * 0.7 + 2 * 1.9) / 4, rtol=1e-10)
    U3 = g.mesh["x"] ** 3  # cubic: second difference 6x exact inside, linear extrapolation exact too
    np.testing.assert_allclose(O.del2(U3, g.dx, g.dy), 6 * g.mesh["x"] / 4, atol=1e-9)


def test_lz_of_an_angular_momentum_eigenstate():
    """grid2d/lz.m with the 4th-order stencil of grid1d.m:52-57: (x + i y) f(r)
    has Lz = +1 and (x - i y) f(r) Lz = -1, to the stencil's O(h^4) error;
    deriv1 is exact on cubics away from the zero-padded edges."""
    g = O.Grid(6, 96, 6, 96)
    X, Y = g.mesh["x"], g.mesh["y"]
    f = np.exp(-(X ** 2 + Y ** 2) / 2)
    for s in (1, -1):
        phi = (X + 1j * s * Y) * f
        assert np.max(np.abs(g.lz(phi) - s * phi)) < 3e-4 * np.max(np.abs(phi))  # h = 0.126
    cub = X ** 3 - 2 * X
    d = g.derivx(cub)
    np.testing.assert_allclose(d[2:-2], (3 * X ** 2 - 2)[2:-2], rtol=0, atol=1e-9)


def test_array_omega_keeps_the_isotropic_ground_state():
    """Array omega (the Crank-Nicolson Lz branch, ssft_kin_step.m:3-11): a
    nodeless ground state of an isotropic trap has Lz psi ~ 0, so a uniform
    omega array leaves the ITP fixed point as it is without rotation, and the
    -omega Lz energy (GPEtask.m:92-94) of an Lz = 1 state is -omega N."""
    g = O.Grid(6, 48, 6, 48)
    X, Y = g.mesh["x"], g.mesh["y"]
    out = []
    for om in (0.0, np.full(g.shape, 0.3)):
        t = O.GPEtask(g, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2))
        t.Ntotal, t.g, t.omega = 10.0, 1.0, om
        out.append(t.groundstate_itp(0.01, 1e-9, np.exp(-(X ** 2 + Y ** 2) / 2).astype(complex), nargout=1)[0])
    # the stencil's O(h^4) error on the radial profile (h = 0.26) is the difference
    assert np.linalg.norm(out[1] - out[0]) / np.linalg.norm(out[0]) < 1e-4
    t = O.GPEtask(g, lambda X, Y, Z: 0 * X)
    t.omega = np.full(g.shape, 0.3)
    phi = (X + 1j * Y) * np.exp(-(X ** 2 + Y ** 2) / 2)
    lz_energy = np.real(g.inner(phi, t.applyh0(phi) - g.lap(phi)))
    assert lz_energy == pytest.approx(-0.3 * g.integrate(np.abs(phi) ** 2), rel=2e-3)  # stencil error, h = 0.26


def test_golden_fixtures_reproduce():
    from tests.golden import make_golden as MG

    for name, fn in MG.CASES.items():
        ref = np.load(MG.path(name))
        out = fn()
        for k in ref.files:
            np.testing.assert_allclose(out[k], ref[k], rtol=1e-12, atol=1e-12, err_msg=f"{name}:{k}")


def test_spinor_itp_decoupled_matches_single_component_ground_state():
    """GPEtaskSpinor.groundstate_itp (lib/@GPEtaskSpinor/groundstate_itp.m)
    with coupling = 0, g = diag(g0, g0), identical traps and identical halves
    converges to the one-component ground state of N/2 per component: the
    harmonic g = 0 case has mu = E/N = 1 (2D, omega = 1)."""
    g = O.Grid(6, 48, 6, 48)
    V = lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2)
    t = O.GPEtaskSpinor(g, [V, V])
    t.g = np.zeros((2, 2))
    t.Ntotal = 2.0
    X, Y = g.mesh["x"], g.mesh["y"]
    p0 = np.exp(-((X - 0.3) ** 2 + Y ** 2) / 3).astype(complex)
    phi, MU, MU2, EE = t.groundstate_itp(0.01, 1e-7, [p0, p0])
    assert EE[-1] == pytest.approx(1.0, abs=1e-6)
    assert MU2[-1] == pytest.approx(1.0, abs=1e-6)
    assert len(MU) == len(EE) and len(MU) > 30
    np.testing.assert_allclose(g.integrate(np.abs(phi[0]) ** 2), 1.0, rtol=1e-12)
    # the coupling term 2 Re(c <phi1|phi2>) of the symmetric state is c N, so
    # E/N = 1 + c: c = -0.25 makes it the ground state (0.75), c = +0.25 the
    # excited one (1.25), which ITP keeps from a symmetric start
    for c in (-0.25, 0.25):
        t.coupling = c
        phi, MU, MU2, EE = t.groundstate_itp(0.01, 1e-7, [p0, p0])
        assert EE[-1] == pytest.approx(1.0 + c, abs=1e-5)


def test_two_component_itp_known_answers():
    """GPEtask2comp.groundstate_itp (lib/@GPEtask2comp/groundstate_itp.m):
    without interactions each component relaxes to the harmonic ground state
    of its own mass, mu_j = omega_j = 1/sqrt(M_j) in 2D for V = r^2/2 (each
    normalised to its own N_j); EE = get_energy/Ntotal then equals
    (N1 mu1 + N2 mu2)/Ntotal."""
    g = O.Grid(6, 48, 6, 48)
    V = lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2)
    t = O.GPEtask2comp(g, [V, V])
    t.g = np.zeros((2, 2))
    t.N1, t.N2, t.Ntotal = 1.0, 3.0, 4.0
    t.M1, t.M2 = 1.0, 4.0
    X, Y = g.mesh["x"], g.mesh["y"]
    p0 = np.exp(-((X - 0.2) ** 2 + Y ** 2) / 3).astype(complex)
    phi, MU1, MU2, EE = t.groundstate_itp(0.01, 1e-7, [p0, p0])
    assert MU1[-1] == pytest.approx(1.0, abs=1e-4)
    assert MU2[-1] == pytest.approx(0.5, abs=1e-4)  # 1/sqrt(4)
    np.testing.assert_allclose([g.integrate(np.abs(p) ** 2) for p in phi], [1.0, 3.0], rtol=1e-12)
    # get_energy uses lap without the mass (GPEtask2comp.m:45-63): E_j = N_j (w/4 + 1/(4w) ...)
    # for a Gaussian of width set by M_j; compare against the direct sum
    E = sum(np.real(g.inner(p, g.lap(p) + V(X, Y, 0) * p)) for p in phi) / 4.0
    assert EE[-1] == pytest.approx(E, rel=1e-10)


@pytest.mark.parametrize("cls", ["spinor", "2comp"])
def test_rotating_two_component_itp_reduces_to_the_plain_one(cls):
    """The rotating branches of the two-component ITPs
    (GPEtaskSpinor/groundstate_itp.m:30-33, GPEtask2comp/groundstate_itp.m:31-36)
    with a vanishing omega: the x and y half-step factors then multiply to
    exp(-kk dt/2/M) exactly (the 1D transforms along x and y commute), so the
    run matches the omega = 0 branch iteration for iteration."""
    g = O.Grid(4.0, 32, 3.5, 24)
    V = [lambda X, Y, Z: 0.5 * (X ** 2 + 1.3 * Y ** 2)] * 2
    X, Y = g.mesh["x"], g.mesh["y"]
    p0 = [np.exp(-((X - 0.3) ** 2 + Y ** 2) / 2).astype(complex), 0.6 * np.exp(-(X ** 2 + Y ** 2) / 3).astype(complex)]
    out = []
    for om in (0.0, 1e-300):
        t = O.GPEtaskSpinor(g, V) if cls == "spinor" else O.GPEtask2comp(g, V)
        t.g = np.array([[1.0, 0.5], [0.5, 0.8]])
        t.Ntotal = 3.0
        if cls == "spinor":
            t.coupling = 0.2
        else:
            t.N1, t.N2, t.M1, t.M2 = 2.0, 1.0, 1.0, 1.7
        t.omega = om
        out.append(t.groundstate_itp(0.02, 1e-4, p0, nargout=4))
    (a, *ha), (b, *hb) = out
    assert len(ha[0]) == len(hb[0])
    for x, y in zip(ha, hb):
        np.testing.assert_allclose(x, y, rtol=1e-10, atol=1e-12)
    for x, y in zip(a, b):
        np.testing.assert_allclose(x, y, rtol=1e-10, atol=1e-12)


def test_rotating_2comp_energy_is_the_rotating_frame_laplacian():
    """GPEtask2comp.get_energy with omega (GPEtask2comp.m:60, grid2d/lap.m:8-10):
    for a state that is a function of r only (Lz psi = 0), the rotating terms
    cancel in <psi|lap(psi, omega)>, and the energy equals the omega = 0 one."""
    g = O.Grid(6.0, 48, 6.0, 48)
    X, Y = g.mesh["x"], g.mesh["y"]
    p = [np.exp(-(X ** 2 + Y ** 2) / 3).astype(complex), 0.5 * np.exp(-(X ** 2 + Y ** 2) / 2).astype(complex)]
    V = [lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2)] * 2
    e = []
    for om in (0.0, 0.4):
        t = O.GPEtask2comp(g, V)
        t.g = np.array([[1.0, 0.5], [0.5, 0.8]])
        t.omega = om
        e.append(t.get_energy(p))
    assert e[1] == pytest.approx(e[0], rel=1e-10)


def test_spinor_lz_energy_is_the_one_component_array_omega_term():
    """GPEtaskSpinor.applyham with a scalar omega subtracts omega*lz(phi_j)
    with grid1d's stencil (GPEtaskSpinor.m:72-74), the operator that
    GPEtask.applyh0 applies for an omega array (GPEtask.m:92-94).  With the
    coupling and g zero, the spinor's energy is therefore the sum of the two
    one-component energies with a uniform omega array."""
    g = O.Grid(4.0, 32, 3.5, 24)
    X, Y = g.mesh["x"], g.mesh["y"]
    V = [lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2), lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2) + 0.2 * X]
    phi = [((X + 0.5j * Y) * np.exp(-(X ** 2 + Y ** 2) / 2)).astype(complex),
           (np.exp(-(X ** 2 + Y ** 2) / 3) * np.exp(0.4j * Y)).astype(complex)]
    s = O.GPEtaskSpinor(g, V)
    s.g = np.zeros((2, 2))
    s.omega = 0.35
    e_sp = s.get_energy(phi)
    e_one = 0.0
    for j in range(2):
        t = O.GPEtask(g, V[j])
        t.omega = np.full(g.shape, 0.35)
        e_one += t.get_energy(phi[j])
    assert e_sp == pytest.approx(e_one, rel=1e-12)
    s.omega = 0.0
    assert abs(s.get_energy(phi) - e_sp) > 1e-3 * abs(e_sp)  # the term is not negligible here
