"""GPU discrete adjoint (gpe_adjoint_grad) against the FP64 oracle's reverse
sweep (oracle.gpe_oracle.adjoint_grad) and central finite differences.

Tolerances (written per test):
* FP64 kernels: dloss/dV relative L2 error <= 1e-9 against the oracle adjoint,
  loss <= 1e-12 absolute; identical results for every checkpoint spacing.
* FP32 kernels: dloss/dV relative L2 error <= 1e-4 against the FP64 oracle
  adjoint over 40 steps.  Over the 2000-step 256^2 window the FP32 sweep is
  held to 2e-3: the gradient there is a small response on top of a large
  stationary background, and rounding the state to FP32 alone moves it by
  2.5e-4 (a complex64 pocketfft sweep lands at 4.6e-4); the FP64 sweep of an
  FP32 context (precision="double") is held to 1e-4.
* Finite differences (FP64 forward on the GPU, step 1e-4): directional
  derivatives within 1e-6 of the FP64 adjoint and within 1e-4 of the FP64
  sweep of the FP32 context, both relative to |grad| |d|.
"""
import numpy as np
import pytest

from oracle import gpe_oracle as O

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def small_case(gpe, axes, precision, g=0.5):
    grid = gpe.grid2d(*axes, precision=precision) if len(axes) == 4 else gpe.grid3d(*axes, precision=precision)
    og = O.Grid(*axes)
    X, Y, Z = og.mesh["x"], og.mesh["y"], og.mesh["z"]
    V = 0.5 * (X ** 2 + Y ** 2) + (2.0 * Z ** 2 if len(axes) == 6 else 0.0) + 0.3 * np.exp(-((X - 1) ** 2 + Y ** 2))
    psi0 = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 4).astype(complex) * (1 + 0.2j * X)
    tgt = np.exp(-((X - 0.5) ** 2 + Y ** 2 + Z ** 2) / 4).astype(complex) * np.exp(1j * np.arctan2(X - 0.5, Y))
    task = gpe.GPEtask(grid, lambda X, Y, Z: V)
    task.g = g
    return task, og, V, psi0, tgt


@pytest.mark.parametrize("axes", [(8, 48, 6, 32), (6, 16, 6, 24, 4, 32)], ids=["2d", "3d"])
def test_fp64_adjoint_matches_oracle_for_every_checkpoint_spacing(gpe, axes):
    task, og, V, psi0, tgt = small_case(gpe, axes, "double")
    M, ddt = 24, 0.01
    ref_loss, ref = O.adjoint_grad(og, V, task.g, psi0, tgt, ddt, M)
    first = None
    for K in (0, 1, 5, 7, M):
        loss, dV = task.adjoint_grad(tgt, ddt, M, phi0=psi0, checkpoint_every=K)
        assert abs(loss - ref_loss) < 1e-12
        assert rel_l2(dV, ref) < 1e-9, K
        if first is None:
            first = dV
        else:
            np.testing.assert_array_equal(dV, first)  # recompute is bit-exact


@pytest.mark.parametrize("axes", [(8, 48, 6, 32), (6, 16, 6, 24, 4, 32)], ids=["2d", "3d"])
def test_fp32_adjoint_within_1e4_of_fp64_oracle(gpe, axes):
    task, og, V, psi0, tgt = small_case(gpe, axes, "single")
    M, ddt = 40, 0.01
    ref_loss, ref = O.adjoint_grad(og, V, task.g, psi0, tgt, ddt, M)
    loss, dV = task.adjoint_grad(tgt, ddt, M, phi0=psi0, checkpoint_every=8)
    assert abs(loss - ref_loss) < 1e-5
    assert rel_l2(dV, ref) < 1e-4


def test_adjoint_leaves_the_state_alone_and_checks_arguments(gpe):
    from gpe_gb300 import _lib as L

    task, og, V, psi0, tgt = small_case(gpe, (8, 32, 8, 32), "double")
    task.init_state = psi0
    task.solve_split(0.01, 5, 1)
    before = task.current_state.copy()
    task.adjoint_grad(tgt, 0.01, 3, phi0=task.current_state)
    np.testing.assert_array_equal(task._download(), before)
    with pytest.raises(gpe.GPEError) as e:
        task.adjoint_grad(tgt, 0.01, 0, phi0=psi0)
    assert e.value.status == L.GPE_ERR_INVALID
    with pytest.raises(gpe.GPEError) as e:  # 18 states of 16 KB
        task.adjoint_grad(tgt, 0.01, 50, phi0=psi0, mem_budget=1e5)
    assert e.value.status == L.GPE_ERR_ALLOC
    task.gamma = 0.01
    with pytest.raises(gpe.GPEError) as e:
        task.adjoint_grad(tgt, 0.01, 3, phi0=psi0)
    assert e.value.status == L.GPE_ERR_UNSUPPORTED


@pytest.mark.slow
def test_adjoint2d_256_gradient_of_bump_amplitudes(gpe):
    """256^2, 16 Gaussian bumps, 2000 steps of 0.002, checkpoints every 50:
    dloss/da_j from the FP32 context (FP32 and FP64 sweeps) against the FP64
    oracle adjoint and against central differences on 32 random directions."""
    from gpe_gb300.imprint import imprint_vortex
    from gpe_workloads import ADJOINT2D as W

    g64 = W.make_grid("double")
    t64 = gpe.GPEtask(g64, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2))
    t64.Ntotal, t64.g = W.Ntotal, W.g
    X, Y = g64.mesh["x"], g64.mesh["y"]
    psi0 = np.asarray(t64.groundstate_itp(W.itp_dt, W.itp_eps, np.exp(-(X ** 2 + Y ** 2) / 32).astype(complex)),
                      dtype=np.complex128)
    tgt = imprint_vortex(g64, psi0, W.g, W.vortex_x0)
    a, basis = W.bumps(g64)
    V0 = W.trap(g64)
    Va = V0 + sum(aj * b for aj, b in zip(a, basis))

    t32 = gpe.GPEtask(W.make_grid("single"), lambda X, Y, Z: V0)
    t32.g = W.g
    loss32, dV32 = t32.adjoint_grad(tgt, W.dt, W.steps, phi0=psi0, V=Va, checkpoint_every=W.checkpoint_every)
    ga32 = t32.project_gradient(dV32, basis)

    og = O.Grid(W.box, W.n, W.box, W.n)
    loss_o, dVo = O.adjoint_grad(og, Va, W.g, psi0, tgt, W.dt, W.steps)
    gao = np.array([np.sum(dVo * b) for b in basis])
    assert abs(loss32 - loss_o) < 1e-4
    assert rel_l2(dV32, dVo) < 2e-3
    assert rel_l2(ga32, gao) < 2e-3
    loss_m, dVm = t32.adjoint_grad(tgt, W.dt, W.steps, phi0=psi0, V=Va, checkpoint_every=W.checkpoint_every,
                                   precision="double")
    gam = t32.project_gradient(dVm, basis)
    assert abs(loss_m - loss_o) < 1e-6
    assert rel_l2(dVm, dVo) < 1e-4
    assert rel_l2(gam, gao) < 1e-4

    loss64, dV64 = t64.adjoint_grad(tgt, W.dt, W.steps, phi0=psi0, V=Va, checkpoint_every=W.checkpoint_every)
    ga64 = t64.project_gradient(dV64, basis)
    assert rel_l2(ga64, gao) < 1e-9

    rng = np.random.default_rng(40)
    eps = 1e-4
    scale = np.linalg.norm(gao)
    for _ in range(32):
        d = rng.standard_normal(len(a))
        d /= np.linalg.norm(d)
        Vd = sum(dj * b for dj, b in zip(d, basis))
        lp = t64.adjoint_grad(tgt, W.dt, W.steps, phi0=psi0, V=Va + eps * Vd)[0]
        lm = t64.adjoint_grad(tgt, W.dt, W.steps, phi0=psi0, V=Va - eps * Vd)[0]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - ga64 @ d) < 1e-6 * scale
        assert abs(fd - gam @ d) < 1e-4 * scale


def test_adjoint_500_step_window_with_recompute_matches_oracle(gpe):
    """The checkpoint/recompute path of config 5's window (500 steps of 0.001)
    on a grid the oracle runs: FP64, 48 x 48 x 32, a memory budget of 60
    states, which refuses storing every step (K = 1: 505 states) and leaves
    the sqrt rule (K = 20: 26 checkpoints, 20 segment states and the sweep's
    arrays, 49 states) and K = 25 (also 49); both match the oracle adjoint
    and each other bit for bit."""
    from gpe_gb300 import _lib as L

    axes = (6, 48, 6, 48, 4, 32)
    task, og, V, psi0, tgt = small_case(gpe, axes, "double")
    M, ddt = 500, 0.001
    S = og.mesh["x"].size * 16
    budget = 60 * S
    ref_loss, ref = O.adjoint_grad(og, V, task.g, psi0, tgt, ddt, M)
    with pytest.raises(gpe.GPEError) as e:
        task.adjoint_grad(tgt, ddt, M, phi0=psi0, checkpoint_every=1, mem_budget=budget)
    assert e.value.status == L.GPE_ERR_ALLOC
    loss_a, dV_a = task.adjoint_grad(tgt, ddt, M, phi0=psi0, checkpoint_every=0, mem_budget=budget)
    loss_b, dV_b = task.adjoint_grad(tgt, ddt, M, phi0=psi0, checkpoint_every=25, mem_budget=budget)
    assert abs(loss_a - ref_loss) < 1e-12
    assert rel_l2(dV_a, ref) < 1e-9
    np.testing.assert_array_equal(dV_a, dV_b)
    assert loss_a == loss_b
    task.close()


@pytest.mark.slow
def test_adjoint3d_512_window_within_60GB(gpe):
    """Config 5's adjoint: 512^3 FP32 (lambda = (1, 1, 2), g = 1), a vortex
    ring on a Thomas-Fermi-like start, the 500-step window of 0.001 against
    the ring-free target under the 60 GB budget.  Storing every state (537
    GB) is refused; the sqrt rule (K = 20, 49 states, 54 GB with the FP64
    gradient) and K = 25 give the same loss and gradient bit for bit (the
    recompute is exact), and the gradient is finite and nonzero."""
    from gpe_gb300 import _lib as L
    from gpe_workloads import RING3D as W

    grid, task = W.make_task("single")
    X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
    r_tf = 18.0
    n = np.clip(1.0 - (X ** 2 + Y ** 2 + (2.0 * Z) ** 2) / r_tf ** 2, 0.0, None)
    phi = np.sqrt(n + 1e-4).astype(np.complex128)
    psi0 = gpe.imprint_vortex_ring(grid, phi, W.g, 0.5 * r_tf)
    with pytest.raises(gpe.GPEError) as e:
        task.adjoint_grad(phi, W.dt, 500, phi0=psi0, checkpoint_every=1, mem_budget=60e9)
    assert e.value.status == L.GPE_ERR_ALLOC
    loss_a, dV_a = task.adjoint_grad(phi, W.dt, 500, phi0=psi0, checkpoint_every=0, mem_budget=60e9)
    loss_b, dV_b = task.adjoint_grad(phi, W.dt, 500, phi0=psi0, checkpoint_every=25, mem_budget=60e9)
    assert np.isfinite(loss_a) and 0.0 < loss_a < 1.0
    assert np.all(np.isfinite(dV_a)) and np.linalg.norm(dV_a) > 0
    assert loss_a == loss_b
    np.testing.assert_array_equal(dV_a, dV_b)
    task.close()


@pytest.mark.slow
def test_adjoint2d_256_fp32_error_sources(gpe, monkeypatch):
    """Where the FP32 context's gradient error on config 4 (256^2, 2000 steps,
    checkpoints every 50) comes from, against the FP64 oracle adjoint: the
    FP32 sweep; the FP64 sweep fed an FP32-arithmetic forward trajectory
    (GPE_ADJ_FORWARD=fp32); the FP64 sweep of an FP64 forward whose states
    are rounded to FP32 after every step (GPE_ADJ_FORWARD=round32); the FP64
    sweep of the FP64 forward; and the two halves of the FP32 forward apart
    (GPE_ADJ_FORWARD=kin32: FP32 kinetic passes, FP64 nonlinear phases;
    nl32: the converse).  Printed as an ADJOINT-ERRORS line.  Measured on a
    GB300 (dL/da): 9.4e-4, 4.5e-4, 6.6e-7, 2.9e-9; kin32 4.4e-4, nl32 4.3e-5.
    Storing the trajectory in FP32 costs nothing measurable; the floor is the
    FP32 kinetic step, whose rounded twiddle and kinetic-factor tables are the
    same at every step, so their errors add up coherently over the window.
    The bounds below pin that attribution."""
    import json

    from gpe_gb300.imprint import imprint_vortex
    from gpe_workloads import ADJOINT2D as W

    g64 = W.make_grid("double")
    t64 = gpe.GPEtask(g64, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2))
    t64.Ntotal, t64.g = W.Ntotal, W.g
    X, Y = g64.mesh["x"], g64.mesh["y"]
    psi0 = np.asarray(t64.groundstate_itp(W.itp_dt, W.itp_eps, np.exp(-(X ** 2 + Y ** 2) / 32).astype(complex)),
                      dtype=np.complex128)
    tgt = imprint_vortex(g64, psi0, W.g, W.vortex_x0)
    a, basis = W.bumps(g64)
    V0 = W.trap(g64)
    Va = V0 + sum(aj * b for aj, b in zip(a, basis))
    og = O.Grid(W.box, W.n, W.box, W.n)
    _, dVo = O.adjoint_grad(og, Va, W.g, psi0, tgt, W.dt, W.steps)
    gao = np.array([np.sum(dVo * b) for b in basis])

    t32 = gpe.GPEtask(W.make_grid("single"), lambda X, Y, Z: V0)
    t32.g = W.g
    kw = dict(phi0=psi0, V=Va, checkpoint_every=W.checkpoint_every)
    errs = {}
    for name, env, prec in (("fp32_sweep", None, None), ("fp64_sweep_fp32_forward", "fp32", "double"),
                            ("fp64_sweep_fp32_kinetic_forward", "kin32", "double"),
                            ("fp64_sweep_fp32_nonlinear_forward", "nl32", "double"),
                            ("fp64_sweep_fp64_forward_states_rounded_to_fp32", "round32", "double"),
                            ("fp64_sweep_fp64_forward", None, "double")):
        if env:
            monkeypatch.setenv("GPE_ADJ_FORWARD", env)
        else:
            monkeypatch.delenv("GPE_ADJ_FORWARD", raising=False)
        _, dV = t32.adjoint_grad(tgt, W.dt, W.steps, precision=prec, **kw)
        errs[name] = {"dLdV_rel_l2": rel_l2(dV, dVo), "dLda_rel_l2": rel_l2(t32.project_gradient(dV, basis), gao)}
    monkeypatch.delenv("GPE_ADJ_FORWARD", raising=False)
    print("ADJOINT-ERRORS " + json.dumps(errs), flush=True)
    e = {k: v["dLda_rel_l2"] for k, v in errs.items()}
    assert e["fp64_sweep_fp64_forward"] < 1e-8
    assert e["fp64_sweep_fp64_forward_states_rounded_to_fp32"] < 1e-5  # FP32 storage: harmless
    assert e["fp64_sweep_fp32_nonlinear_forward"] < 1e-4
    assert e["fp64_sweep_fp32_kinetic_forward"] > 2e-4  # the floor: FP32 kinetic arithmetic
    assert 0.7 < e["fp64_sweep_fp32_kinetic_forward"] / e["fp64_sweep_fp32_forward"] < 1.3
    assert e["fp32_sweep"] < 2e-3
    t32.close()
    t64.close()
