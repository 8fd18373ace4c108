"""The persistent kernels of small 2D grids (solve_split of one context, or
solve_split_batch of many, one launch per outer step for all of them): the
cluster kernel (state in distributed shared memory, one cluster per grid)
the grid-wide kernel (FP32, GPE_SMALL2D=grid: every pass spread over all
SMs, grid barriers between passes) and the multi-grid pass kernels (FP32,
GPE_SMALL2D=multi: one launch per pass over the tiles of all grids of one
shape, a stream per shape, one graph per outer step), against the per-pass path (pass variant
2: two axis-pass launches per step and grid) and against the FP64 oracle,
through the C ABI.

The per-point arithmetic of both paths is the same code (the axis passes'
FFT, kinetic factor, prologue and epilogue; both fold consecutive steps,
except the grid-wide kernel, which is compared with folding off), so the
states agree to the
rounding of the norm / energy sums, which are summed in a different order:
FP64 <= 1e-12 relative, FP32 <= 1e-6 (2e-6 with mu feedback, where those sums
steer the next block).
"""
import numpy as np
import pytest

from oracle import gpe_oracle as O

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def harmonic(lam):
    return lambda X, Y, Z: 0.5 * ((lam[0] * X) ** 2 + (lam[1] * Y) ** 2)


# (xmax, nx, ymax, ny), g, gamma: every cluster axis length, square and not
SPECS = [((4.0, 64, 4.0, 64), 0.8, 0.0), ((5.0, 96, 4.0, 128), 1.5, 0.02),
         ((6.0, 192, 6.0, 64), 0.5, 0.0), ((6.0, 256, 6.0, 256), 1.0, 0.01),
         ((7.0, 384, 7.0, 96), 0.3, 0.0), ((5.0, 128, 5.0, 192), 2.0, 0.05)]


def make(gpe, spec, precision, variant):
    axes, g, gam = spec
    grid = gpe.grid2d(*axes, precision=precision)
    t = gpe.GPEtask(grid, harmonic((1.0, 1.3)))
    t.set_pass_variant(variant)
    t.g, t.gamma, t.Ntotal = g, gam, 5.0
    X, Y = grid.mesh["x"], grid.mesh["y"]
    t.init_state = np.sqrt(5.0) * grid.normalize(np.exp(-(X ** 2 + Y ** 2) / 2 + 0.4j * X + 0.2j * Y))
    return t


PATHS = [("cluster", "double"), ("cluster", "single"), ("grid", "single"), ("multi", "single")]


@pytest.mark.parametrize("path,precision", PATHS)
def test_cluster_batch_matches_per_pass_path(gpe, monkeypatch, path, precision):
    monkeypatch.setenv("GPE_SMALL2D", path)
    if path == "grid":  # the grid-wide kernel runs unfolded steps: so does the reference path
        monkeypatch.setenv("GPE_FOLD", "0")
    # the per-pass path on the FFT plans the persistent kernel runs (FP32:
    # the cluster kernel takes the alternative plan where a length has one,
    # the grid kernel the default plans), so that both paths do the same
    # arithmetic and differ only in the order of the block-end sums
    ref = [make(gpe, s, precision, 2) for s in SPECS]
    ref_launched = 0
    for t in ref:
        t.autotune(3 if path == "cluster" else 0)
        k = t.kernel_launches()
        t.solve_split(0.003, 20, 3)
        ref_launched += t.kernel_launches() - k
    batch = [make(gpe, s, precision, 0) for s in SPECS]
    k0 = sum(t.kernel_launches() for t in batch)
    gpe.solve_split_batch(batch, 0.003, 20, 3)
    tol = 1e-12 if precision == "double" else 2e-6
    for a, b in zip(ref, batch):
        assert b.current_iter == 3 and b.current_time == pytest.approx(a.current_time)
        assert rel_l2(b.current_state, a.current_state) < tol
        np.testing.assert_allclose(b.history["mu"], a.history["mu"], rtol=tol)
        np.testing.assert_allclose(b.history["n"], a.history["n"], rtol=tol)
    # persistent kernels: one launch per outer step for the whole batch, plus
    # each context's setup (state upload and initial mu: a few kernels); the
    # per-pass path launches the passes of every step and grid plus the block
    # ends.  The multi-grid pass kernels launch one pass per shape of grid
    # (here every grid has its own shape): no more than the per-pass path.
    launched = sum(t.kernel_launches() for t in batch) - k0
    if path == "multi":
        assert launched <= ref_launched, (launched, ref_launched)
    else:
        assert launched <= 3 + 8 * len(SPECS), launched
    for t in ref + batch:
        t.close()


@pytest.mark.parametrize("path,precision", PATHS)
def test_cluster_single_context_with_feedback_decay_and_callbacks(gpe, monkeypatch, path, precision):
    monkeypatch.setenv("GPE_SMALL2D", path)
    if path == "grid":
        monkeypatch.setenv("GPE_FOLD", "0")
    """gamma > 0 with the mu feedback, a decaying target norm and an outer-step
    callback, on one 128 x 96 context, against the FP64 oracle."""
    V = harmonic((1.0, 1.4))
    grid = gpe.grid2d(5.0, 128, 4.0, 96, precision=precision)
    task = gpe.GPEtask(grid, V)
    og = O.GPEtask(O.Grid(5.0, 128, 4.0, 96), V)
    X, Y = og.grid.mesh["x"], og.grid.mesh["y"]
    psi0 = np.exp(-(X ** 2 + (1.2 * Y) ** 2) / 3 + 0.5j * X)
    seen = []
    for t in (task, og):
        t.Ntotal, t.g, t.gamma, t.decay_rate = 40.0, 1.2, 0.03, 0.5
        t.init_state = psi0
    task.user_callback = lambda tk: seen.append((tk.current_iter, tk.current_mu))
    task.solve_split(0.004, 30, 3)
    og.solve_split(0.004, 30, 3)
    tol = 1e-11 if precision == "double" else 2e-5
    assert rel_l2(task.current_state, og.current_state) < tol
    np.testing.assert_allclose(task.history["mu"], og.history["mu"], rtol=tol)
    np.testing.assert_allclose(task.history["n"], og.history["n"], rtol=tol)
    assert [s[0] for s in seen] == [1, 2, 3]
    np.testing.assert_allclose([s[1] for s in seen], og.history["mu"], rtol=tol)
    task.close()


@pytest.mark.parametrize("path", ["cluster", "grid", "multi"])
def test_cluster_kernel_is_the_launched_kernel(gpe, monkeypatch, path):
    """With per-launch profiling the persistent path launches directly: one
    cluster_step launch per outer step and no axis-pass launch."""
    monkeypatch.setenv("GPE_SMALL2D", path)
    grid = gpe.grid2d(6.0, 256, 6.0, 256, precision="single")
    task = gpe.GPEtask(grid, harmonic((1.0, 1.0)))
    task.g, task.Ntotal = 0.5, 10.0
    X, Y = grid.mesh["x"], grid.mesh["y"]
    task.init_state = np.exp(-(X ** 2 + Y ** 2) / 4).astype(complex)
    task.solve_split(0.002, 10, 1)
    task.profile(True)
    task.solve_split(0.002, 50, int(task.current_iter) + 4)
    stats = {s["name"]: s["launches"] for s in task.profile_read()}
    task.profile(False)
    assert stats.get("cluster_step") == 4, stats
    assert "pass_y" not in stats and "pass_x" not in stats, stats
    task.close()
