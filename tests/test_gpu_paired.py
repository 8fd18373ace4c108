"""The paired FP32 step passes (two pencils per thread on packed FP32x2
arithmetic: plan variant 2 on the alternative plans, 3 on the default plans,
gpe_autotune modes 4 and 5) against the FP64 oracle, on both pass layouts
and every axis length that has them, through the C ABI.

Tolerances: FP32 kernels, relative L2 state error <= 2e-5 and history mu / n
<= 2e-5 relative after a few split steps (the bound of the scalar FP32
passes); ground-state MU/EE <= 1e-6 relative of the oracle's (the FP32 ITP
finishes in FP64 once FP32 rounding stalls its residual).  Against the scalar
pass on the same plan (both FP32): <= 2e-6 (rounding-level: the same
arithmetic, different contraction and reduction order).
"""
import numpy as np
import pytest

from tests.test_gpu_parity import harmonic, make_pair, rel_l2

pytestmark = pytest.mark.gpu

ALT = [128, 192, 256, 384, 512]
DEF = [128, 256, 512]  # lengths with a paired pass on the default plan
CASES = [(n, 4) for n in ALT] + [(n, 5) for n in DEF]
VAR = {4: 2, 5: 3}  # autotune mode -> plan variant reported per axis


def gauss_state(og, rng, k=0.3):
    X, Y = og.mesh["x"], og.mesh["y"]
    r2 = X ** 2 + Y ** 2
    if "z" in og.mesh:
        r2 = r2 + og.mesh["z"] ** 2
    return np.exp(-r2) * (1 + 0.05 * rng.standard_normal(og.shape)) * np.exp(1j * k * X)


@pytest.mark.parametrize("n,mode", CASES)
@pytest.mark.parametrize("gamma", [0.0, 0.02])
def test_paired_passes_2d_contig_and_strided(gpe, n, mode, gamma):
    """y pass (contiguous, prologue) and x pass (strided, epilogue) of 2D
    grids n x 8 and 8 x n, with and without damping (the damping factor takes
    the packed exponential)."""
    rng = np.random.default_rng(n + 7)
    for nx, ny in ((n, 8), (8, n)):
        grid, task, og, ot = make_pair(gpe, (3.0, nx, 2.0, ny), harmonic((1.0, 1.7)), "single", g=0.7, gamma=gamma)
        chosen = task.autotune(mode)
        assert chosen[0] == (VAR[mode] if nx == n else -1) and chosen[1] == (VAR[mode] if ny == n else -1)
        psi0 = gauss_state(og, rng)
        task.init_state = psi0
        ot.init_state = psi0
        task.solve_split(0.002, 3, 2)  # 3 % n_recalc != 0 -> n_rec = 1 (solve_split.m:25-27)
        ot.solve_split(0.002, 3, 2)
        assert rel_l2(task.current_state, ot.current_state) < 2e-5, (nx, ny)
        np.testing.assert_allclose(task.history["mu"], ot.history["mu"], rtol=2e-5)
        np.testing.assert_allclose(task.history["n"], ot.history["n"], rtol=2e-5)
        task.close()


@pytest.mark.parametrize("n,mode", CASES)
def test_paired_passes_3d_z_axis(gpe, n, mode):
    """z pass (strided by nx*ny) of an 8 x 16 x n grid, 20 steps in 2 blocks."""
    rng = np.random.default_rng(n + 11)
    grid, task, og, ot = make_pair(gpe, (3.0, 8, 3.0, 16, 4.0, n), harmonic((1.0, 1.2, 1.5)), "single", g=0.5,
                                   gamma=0.01)
    chosen = task.autotune(mode)
    assert chosen[2] == VAR[mode]
    psi0 = gauss_state(og, rng)
    task.init_state = psi0
    ot.init_state = psi0
    task.solve_split(0.002, 20, 1)
    ot.solve_split(0.002, 20, 1)
    assert rel_l2(task.current_state, ot.current_state) < 2e-5
    np.testing.assert_allclose(task.history["mu"], ot.history["mu"], rtol=2e-5)
    task.close()


@pytest.mark.parametrize("axes,modes,chosen", [
    ((5.0, 128, 5.0, 256, 4.0, 192), (4, 3), ((2, 2, 2), (1, 1, 1))),
    ((5.0, 256, 5.0, 128, 4.0, 128), (5, 0), ((3, 3, 3), (0, 0, 0))),
], ids=["alternative", "default"])
def test_paired_3d_all_axes_match_scalar_passes(gpe, axes, modes, chosen):
    """Every axis paired: the paired passes against the scalar passes of the
    same plans, and both against the oracle."""
    V = harmonic((1.0, 1.1, 1.3))
    rng = np.random.default_rng(5)
    grid, tp, og, ot = make_pair(gpe, axes, V, "single", g=0.4, gamma=0.01)
    _, ts, _, _ = make_pair(gpe, axes, V, "single", g=0.4, gamma=0.01)
    assert tp.autotune(modes[0]) == chosen[0]
    assert ts.autotune(modes[1]) == chosen[1]
    psi0 = gauss_state(og, rng)
    for t in (tp, ts, ot):
        t.init_state = psi0
        t.solve_split(0.002, 10, 1)
    assert rel_l2(tp.current_state, ts.current_state) < 2e-6
    assert rel_l2(tp.current_state, ot.current_state) < 2e-5
    np.testing.assert_allclose(tp.history["mu"], ot.history["mu"], rtol=2e-5)
    tp.close()
    ts.close()


@pytest.mark.parametrize("mode", [4, 5])
def test_paired_itp_ground_state(gpe, mode):
    """Imaginary time on paired passes (ITP prologue and epilogue: the factor
    array, the packed exponential at large arguments): MU/EE and the ground
    state against the oracle."""
    axes = (6.0, 128, 6.0, 256)
    grid, task, og, ot = make_pair(gpe, axes, harmonic((1.0, 1.3)), "single", Ntotal=50.0, g=0.8)
    assert task.autotune(mode) == (VAR[mode], VAR[mode], -1)
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = np.exp(-(X ** 2 + Y ** 2) / 4).astype(complex)
    phi, MU, MU2, EE = task.groundstate_itp(0.01, 1e-6, psi0, nargout=4)
    ophi, oMU, oMU2, oEE = ot.groundstate_itp(0.01, 1e-6, psi0, nargout=4)
    assert task.last_itp.converged
    assert abs(MU[-1] - oMU[-1]) / abs(oMU[-1]) < 1e-6
    assert abs(EE[-1] - oEE[-1]) / abs(oEE[-1]) < 1e-6
    assert rel_l2(phi, ophi) < 1e-5
    task.close()


def test_autotuner_may_choose_paired(gpe):
    """The tuner's choice is one of the three variants per axis, and the tuned
    context reproduces the oracle."""
    axes = (6.0, 256, 6.0, 256, 4.0, 128)
    grid, task, og, ot = make_pair(gpe, axes, harmonic((1.0, 1.0, 1.5)), "single", g=0.5)
    chosen = task.autotune(1)
    assert all(c in (0, 1, 2, 3) for c in chosen)
    psi0 = gauss_state(og, np.random.default_rng(2))
    task.init_state = psi0
    ot.init_state = psi0
    task.solve_split(0.002, 10, 1)
    ot.solve_split(0.002, 10, 1)
    assert rel_l2(task.current_state, ot.current_state) < 2e-5
    task.close()
