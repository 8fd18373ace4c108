"""Stochastic GPE (SGPEtask.solve_split, lib/@SGPEtask/solve_split.m:1-81).

* The noise generator (Philox4x32-10 keyed by the seed, counter = (grid point,
  global step), Box-Muller on 24-bit uniforms) against a restatement in
  Python integers: <= 3e-6 absolute (FP32 log/sqrt/sincospi).
* T = 0: the deterministic SGPE step (mu = mu_init, damping without
  renormalisation) against the FP64 oracle: FP64 <= 1e-11, FP32 <= 2e-5.
* T > 0: the oracle fed the device's own noise variates: FP32 <= 2e-5.
* The noise amplitude of one step from a zero state: within 5% of
  sqrt(T gamma ddt / weight) propagated through the kinetic factor.
* Rotating SGPE (scalar omega: the Lz Crank-Nicolson update after each
  kinetic step, solve_split.m:61-67): T = 0 FP64 and T > 0 FP32 with the
  device noise, against the oracle.
* Energy cut-off (ecut > 0 with T > 0, solve_split.m:40-42): the oracle fed
  the device's noise (a numpy restatement of the generator in FP64), 2D and
  3D, FP64 <= 1e-11 and FP32 <= 2e-5; one step of pure noise leaves no mode
  with kk >= ecut.
"""
import math

import numpy as np
import pytest

from oracle import gpe_oracle as O

pytestmark = pytest.mark.gpu

M0, M1, W0, W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(c, k0, k1):
    c = list(c)
    for _ in range(10):
        p0, p1 = M0 * c[0], M1 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & MASK, p1 & MASK, ((p0 >> 32) ^ c[3] ^ k1) & MASK, p0 & MASK]
        k0, k1 = (k0 + W0) & MASK, (k1 + W1) & MASK
    return c


def gauss2(seed, step, idx):
    r = philox4x32_10((idx & MASK, idx >> 32, step & MASK, step >> 32), seed & MASK, seed >> 32)
    u1 = ((r[0] >> 8) + 1) * 2.0 ** -24
    u2 = (r[1] >> 8) * 2.0 ** -24
    rad = math.sqrt(-2.0 * math.log(u1))
    return rad * math.cos(2 * math.pi * u2), rad * math.sin(2 * math.pi * u2)


def gauss2_np(seed, step, n):
    """gauss2 for points 0..n-1 in FP64 (numpy uint64 products)."""
    i = np.arange(n, dtype=np.uint64)
    m32 = np.uint64(MASK)
    c = [i & m32, i >> np.uint64(32), np.full(n, step & MASK, np.uint64), np.full(n, step >> 32, np.uint64)]
    k0, k1 = seed & MASK, seed >> 32
    for _ in range(10):
        p0, p1 = np.uint64(M0) * c[0], np.uint64(M1) * c[2]
        c = [((p1 >> np.uint64(32)) ^ c[1] ^ np.uint64(k0)) & m32, p1 & m32,
             ((p0 >> np.uint64(32)) ^ c[3] ^ np.uint64(k1)) & m32, p0 & m32]
        k0, k1 = (k0 + W0) & MASK, (k1 + W1) & MASK
    u1 = ((c[0] >> np.uint64(8)) + np.uint64(1)).astype(np.float64) * 2.0 ** -24
    u2 = (c[1] >> np.uint64(8)).astype(np.float64) * 2.0 ** -24
    rad = np.sqrt(-2.0 * np.log(u1))
    return rad * np.cos(2 * np.pi * u2) + 1j * rad * np.sin(2 * np.pi * u2)


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def test_noise_generator_matches_its_definition(gpe):
    seed, step, n = 0x123456789ABCDEF, 77, 3000
    z = gpe.noise_variates(seed, step, n)
    ref = np.array([gauss2(seed, step, i) for i in range(n)])
    assert np.max(np.abs(z - ref)) < 3e-6
    big = gpe.noise_variates(7, 1, 1 << 18)
    assert abs(big.mean()) < 0.01 and abs(big.var() - 1.0) < 0.01


def make_pair(gpe, axes, precision, **props):
    V = (lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2)) if len(axes) == 4 else \
        (lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2 + (1.5 * Z) ** 2))
    grid = gpe.grid2d(*axes, precision=precision) if len(axes) == 4 else gpe.grid3d(*axes, precision=precision)
    task = gpe.SGPEtask(grid, V)
    og = O.Grid(*axes)
    ot = O.SGPEtask(og, V)
    for k, v in props.items():
        setattr(task, k, v)
        setattr(ot, k, v)
    return task, og, ot


@pytest.mark.parametrize("axes", [(4.0, 48, 3.5, 32), (4.0, 32, 3.5, 24, 2.5, 16)], ids=["2d", "3d"])
@pytest.mark.parametrize("precision", ["double", "single"])
def test_sgpe_zero_temperature_matches_oracle(gpe, axes, precision):
    task, og, ot = make_pair(gpe, axes, precision, g=1.0, gamma=0.05, mu_init=1.7, T=0.0)
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = (np.exp(-((X - 0.5) ** 2 + Y ** 2) / 2) * np.exp(0.3j * Y)).astype(complex)
    task.init_state = psi0
    ot.init_state = psi0
    task.solve_split(0.004, 10, 3)
    ot.solve_split(0.004, 10, 3)
    tol = 1e-11 if precision == "double" else 2e-5
    assert rel_l2(task.current_state, ot.current_state) < tol
    np.testing.assert_allclose(task.history["mu"], [1.7, 1.7, 1.7])
    np.testing.assert_allclose(task.history["n"], ot.history["n"], rtol=tol)


def test_sgpe_finite_temperature_matches_oracle_with_the_device_noise(gpe):
    task, og, ot = make_pair(gpe, (4.0, 48, 3.5, 32), "single", g=0.8, gamma=0.1, mu_init=2.0, T=0.5)
    task.seed = 2024
    steps = iter(range(10 ** 6))
    P = og.nx * og.ny

    def noise(shape):
        z = gpe.noise_variates(task.seed, next(steps), P).astype(np.float64)
        return (z[:, 0] + 1j * z[:, 1]).reshape(shape)

    ot.noise = noise
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = np.exp(-(X ** 2 + Y ** 2) / 2).astype(complex)
    task.init_state = psi0
    ot.init_state = psi0
    task.solve_split(0.004, 10, 2)
    ot.solve_split(0.004, 10, 2)
    assert rel_l2(task.current_state, ot.current_state) < 2e-5
    np.testing.assert_allclose(task.history["n"], ot.history["n"], rtol=2e-5)
    # same seed, same run; another seed, another run
    task2, _, _ = make_pair(gpe, (4.0, 48, 3.5, 32), "single", g=0.8, gamma=0.1, mu_init=2.0, T=0.5)
    task2.seed = 2024
    task2.init_state = psi0
    task2.solve_split(0.004, 10, 2)
    np.testing.assert_array_equal(task2.current_state, task.current_state)
    task2.seed, task2.current_iter = 2025, 0
    task2.init_state = psi0
    task2.solve_split(0.004, 10, 2)
    assert rel_l2(task2.current_state, task.current_state) > 1e-3


def test_sgpe_noise_amplitude(gpe):
    """One step of pure noise (V = 0, g = 0, mu = 0) from psi = 0:
    psi = ifft(ekk fft(sigma (n1 + i n2))), so <|psi|^2> = 2 sigma^2 <|ekk|^2>."""
    axes = (8.0, 128, 8.0, 128)
    grid = gpe.grid2d(*axes, precision="single")
    task = gpe.SGPEtask(grid, lambda X, Y, Z: 0 * X)
    task.gamma, task.T, task.seed = 0.2, 3.0, 11
    task.init_state = np.zeros(grid.shape, complex)
    ddt = 0.01
    task.n_recalc = 1
    task.solve_split(ddt, 1, 1)
    og = O.Grid(*axes)
    dt = ddt * 1j / (1 + 1j * task.gamma)
    ekk2 = np.mean(np.abs(np.exp(-og.kk * dt)) ** 2)
    sigma2 = task.T * task.gamma * ddt / og.weight
    measured = np.mean(np.abs(task.current_state) ** 2)
    assert measured == pytest.approx(2 * sigma2 * ekk2, rel=0.05)


def test_sgpe_unsupported_options(gpe):
    from gpe_gb300 import _lib as L

    task, og, ot = make_pair(gpe, (4.0, 32, 3.5, 32), "single", g=1.0, gamma=0.1, T=1.0)
    task.omega = 0.5 + 0.0 * og.mesh["x"]  # an omega array: the reference's SGPE takes a scalar
    task.init_state = np.ones(og.shape, complex)
    with pytest.raises(gpe.GPEError) as e:
        task.solve_split(0.004, 10, 1)
    assert e.value.status == L.GPE_ERR_UNSUPPORTED
    task.omega, task.ecut = 0.0, float("nan")
    with pytest.raises(gpe.GPEError) as e:
        task.solve_split(0.004, 10, 1)
    assert e.value.status == L.GPE_ERR_INVALID


def cut_between_modes(og, frac):
    """An ecut at the given fraction of max(kk), moved to the middle of the gap
    between the two distinct mode energies around it (no mode within rounding)."""
    kk = np.unique(np.round(og.kk.ravel(), 9))
    i = np.searchsorted(kk, frac * kk[-1])
    return 0.5 * (kk[i - 1] + kk[i])


@pytest.mark.parametrize("axes", [(4.0, 48, 3.5, 32), (4.0, 32, 3.5, 24, 2.5, 16)], ids=["2d", "3d"])
@pytest.mark.parametrize("precision", ["double", "single"])
def test_sgpe_energy_cutoff_matches_oracle(gpe, axes, precision):
    task, og, ot = make_pair(gpe, axes, precision, g=0.8, gamma=0.1, mu_init=2.0, T=0.5, n_recalc=5)
    ecut = cut_between_modes(og, 0.3)
    task.ecut = ot.ecut = ecut
    task.seed = 99
    steps = iter(range(10 ** 6))

    def noise(shape):
        return gauss2_np(task.seed, next(steps), int(np.prod(shape))).reshape(shape)

    ot.noise = noise
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = (np.exp(-((X - 0.3) ** 2 + Y ** 2) / 2) * np.exp(0.5j * X)).astype(complex)
    task.init_state = psi0
    ot.init_state = psi0
    task.solve_split(0.004, 10, 2)
    ot.solve_split(0.004, 10, 2)
    tol = 1e-11 if precision == "double" else 2e-5
    assert rel_l2(task.current_state, ot.current_state) < tol
    np.testing.assert_allclose(task.history["n"], ot.history["n"], rtol=tol)


@pytest.mark.parametrize("axes", [(8.0, 64, 8.0, 64), (8.0, 32, 8.0, 32, 8.0, 32)], ids=["2d", "3d"])
def test_sgpe_energy_cutoff_empties_the_high_modes(gpe, axes):
    """One step of pure noise (V = g = mu = 0) from psi = 0: psi =
    ifft(ekk .* mask .* fft(noise)), so fft(psi) vanishes where kk >= ecut."""
    grid = gpe.grid2d(*axes, precision="single") if len(axes) == 4 else gpe.grid3d(*axes, precision="single")
    task = gpe.SGPEtask(grid, lambda X, Y, Z: 0 * X)
    og = O.Grid(*axes)
    task.gamma, task.T, task.seed, task.n_recalc = 0.2, 3.0, 5, 1
    task.ecut = cut_between_modes(og, 0.25)
    task.init_state = np.zeros(grid.shape, complex)
    task.solve_split(0.01, 1, 1)
    spec = np.abs(og.fft(task.current_state))
    kept = og.kk < task.ecut
    assert 0 < kept.sum() < kept.size
    assert spec[~kept].max() < 1e-5 * spec[kept].max()
    assert spec[kept].min() > 0


def test_sgpe_block_count_follows_sgpe_solve_split(gpe):
    """@SGPEtask/solve_split.m:54 loops jj = 1:niter_inner/n_recalc without
    GPEtask's n_recalc = 1 fallback: 15 inner steps at n_recalc = 10 run one
    block of 10 (time still advances by 15 ddt); 5 < 10 runs none (an error)."""
    from gpe_gb300 import _lib as L

    task, og, ot = make_pair(gpe, (4.0, 32, 3.5, 24), "double", g=1.0, gamma=0.05, mu_init=1.2, n_recalc=10)
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = np.exp(-(X ** 2 + Y ** 2) / 2).astype(complex)
    task.init_state = psi0
    ot.init_state = psi0
    task.solve_split(0.004, 15, 2)
    ot.solve_split(0.004, 15, 2)
    assert rel_l2(task.current_state, ot.current_state) < 1e-11
    assert task.current_time == pytest.approx(ot.current_time)
    task.current_iter = 0
    with pytest.raises(gpe.GPEError) as e:
        task.solve_split(0.004, 5, 1)
    assert e.value.status == L.GPE_ERR_INVALID


@pytest.mark.parametrize("precision,T", [("double", 0.0), ("single", 0.4)])
def test_rotating_sgpe_matches_oracle(gpe, precision, T):
    task, og, ot = make_pair(gpe, (4.0, 48, 3.5, 32), precision, g=0.8, gamma=0.05, mu_init=2.0, T=T,
                             omega=0.45, n_crank=3, n_recalc=5)
    task.seed = 31
    steps = iter(range(10 ** 6))

    def noise(shape):
        return gauss2_np(task.seed, next(steps), int(np.prod(shape))).reshape(shape)

    ot.noise = noise
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = (np.exp(-((X - 0.5) ** 2 + Y ** 2) / 2) * (1 + 0.2 * (X + 1j * Y))).astype(complex)
    task.init_state = psi0
    ot.init_state = psi0
    task.solve_split(0.004, 10, 2)
    ot.solve_split(0.004, 10, 2)
    tol = 1e-11 if precision == "double" else 2e-5
    assert rel_l2(task.current_state, ot.current_state) < tol
    np.testing.assert_allclose(task.history["n"], ot.history["n"], rtol=tol)


def test_sgpe_user_callback_term_ends_the_run(gpe):
    """@SGPEtask/solve_split.m:77-80: a user_callback that returns 'TERM'
    ends the run after that outer step (the library's on_step stop); the
    state and history are those of the oracle stopped at the same step."""
    task, og, ot = make_pair(gpe, (4.0, 48, 3.5, 32), "double", g=1.0, gamma=0.05, mu_init=1.7, T=0.0)
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = (np.exp(-((X - 0.5) ** 2 + Y ** 2) / 2) * np.exp(0.3j * Y)).astype(complex)
    cb = lambda t: "TERM" if t.current_iter == 2 else ""  # noqa: E731
    for t in (task, ot):
        t.init_state = psi0
        t.user_callback = cb
        t.solve_split(0.004, 10, 5)
    assert task.current_iter == ot.current_iter == 2
    assert len(task.history["n"]) == 2
    assert rel_l2(task.current_state, ot.current_state) < 1e-11
    # GPEtask ignores the callback's result (@GPEtask/solve_split.m:80)
    plain = gpe.GPEtask(task.grid, lambda X, Y, Z: 0.5 * (X ** 2 + 1.2 * Y ** 2))
    plain.init_state = psi0
    plain.user_callback = cb
    plain.solve_split(0.004, 10, 3)
    assert plain.current_iter == 3
