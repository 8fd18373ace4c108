"""Size-independent properties at the benchmark sizes (256^3, 512^3), where the
oracle is too slow to run: a grid plane wave propagates exactly (the per-axis
kinetic factors are exp(-i k^2/2 t) exactly), gamma = 0 steps with a fixed mu
are time-reversible (conj -> propagate -> conj returns the start) and conserve
the norm, and the FP32 kernels follow the FP64 ones on the same start."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def test_plane_wave_is_exact_at_256cube(gpe):
    grid = gpe.grid3d(12.0, 256, 12.0, 256, 12.0, 256, precision="double")
    task = gpe.GPEtask(grid, lambda X, Y, Z: 0 * X)
    X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
    L = 24.0 + 24.0 / 255  # period span + dx of each axis
    kx, ky, kz = 2 * np.pi * 5 / L, -2 * np.pi * 3 / L, 2 * np.pi * 7 / L
    psi0 = np.exp(1j * (kx * X + ky * Y + kz * Z))
    task.mu_init = 0.4
    task.init_state = psi0
    task.solve_split(0.002, 10, 2)
    T = 0.002 * 10 * 2
    expect = psi0 * np.exp(-1j * ((kx ** 2 + ky ** 2 + kz ** 2) / 2 - 0.4) * T)
    assert np.max(np.abs(task.current_state - expect)) < 1e-11


def test_time_reversal_at_256cube_fp64(gpe):
    grid = gpe.grid3d(12.0, 256, 12.0, 256, 12.0, 256, precision="double")
    V = lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2 + (4 * Z) ** 2)
    X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
    psi0 = (10 * np.exp(-(X ** 2 + Y ** 2 + 16 * Z ** 2) / 8) * np.exp(0.3j * X)).astype(complex)
    fwd = gpe.GPEtask(grid, V)
    fwd.g, fwd.mu_init = 0.5, 30.0  # a fixed mu: the state-derived one is not time-symmetric
    fwd.init_state = psi0
    fwd.solve_split(0.002, 10, 2)
    back = gpe.GPEtask(grid, V)
    back.g, back.mu_init = 0.5, 30.0
    back.init_state = np.conj(fwd.current_state)
    back.solve_split(0.002, 10, 2)
    assert rel_l2(np.conj(back.current_state), psi0) < 1e-10
    n0 = np.sum(np.abs(psi0) ** 2) * grid.weight
    np.testing.assert_allclose(fwd.history["n"], n0, rtol=1e-12)


def test_norm_conservation_at_256cube_fp32(gpe):
    grid = gpe.grid3d(12.0, 256, 12.0, 256, 12.0, 256, precision="single")
    task = gpe.GPEtask(grid, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2 + (4 * Z) ** 2))
    X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
    psi0 = (10 * np.exp(-(X ** 2 + Y ** 2 + 16 * Z ** 2) / 8) * np.exp(0.3j * Y)).astype(np.complex64)
    task.g = 0.5
    task.init_state = psi0
    task.solve_split(0.002, 100, 1)
    n0 = np.sum(np.abs(psi0.astype(np.complex128)) ** 2) * grid.weight
    assert abs(task.history["n"][-1] / n0 - 1) < 1e-5  # ~3e-8 per step


def test_fp32_follows_fp64_at_512cube(gpe):
    axes = (24.0, 512, 24.0, 512, 24.0, 512)
    V = lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2 + (2 * Z) ** 2)
    out = {}
    for prec in ("double", "single"):
        grid = gpe.grid3d(*axes, precision=prec)
        X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
        psi0 = (20 * np.exp(-(X ** 2 + Y ** 2 + 4 * Z ** 2) / 50) * np.exp(0.2j * X)).astype(complex)
        task = gpe.GPEtask(grid, V)
        task.g, task.gamma, task.Ntotal = 1.0, 0.01, 1e6
        task.init_state = psi0
        task.solve_split(0.001, 10, 1)
        out[prec] = (task.current_state.astype(np.complex128), task.history["mu"][-1])
        task.close()
        del psi0, X, Y, Z
    assert rel_l2(out["single"][0], out["double"][0]) < 2e-5
    assert out["single"][1] == pytest.approx(out["double"][1], rel=1e-5)
