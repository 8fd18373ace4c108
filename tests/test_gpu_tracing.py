"""Tracing hook: with GPE_NVTX=1 every kernel launch sits inside a host NVTX
range named by its kernel class (for ncu --nvtx filters and timeline tools).
The ranges change nothing the device computes: a run with them matches the
run without them bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(gpe):
    grid = gpe.grid2d(6.0, 64, 6.0, 48, precision="single")
    task = gpe.GPEtask(grid, lambda X, Y, Z: 0.5 * (X ** 2 + (1.2 * Y) ** 2))
    task.g, task.gamma, task.Ntotal = 0.5, 0.01, 50.0
    X, Y = grid.mesh["x"], grid.mesh["y"]
    task.init_state = np.exp(-(X ** 2 + Y ** 2) / 4 + 0.3j * X).astype(np.complex64)
    task.solve_split(0.004, 20, 2)
    out = task.current_state.copy(), np.array(task.history["mu"])
    task.close()
    return out


def test_nvtx_ranges_leave_the_results_unchanged(gpe, monkeypatch):
    monkeypatch.delenv("GPE_NVTX", raising=False)
    a = run(gpe)
    monkeypatch.setenv("GPE_NVTX", "1")
    b = run(gpe)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
