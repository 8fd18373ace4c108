"""GPU parity: libgpe (through the C ABI, via the gpe_gb300 host mirror)
against the FP64 oracle and the committed golden fixtures.

Tolerances (written per test):
* FP64 kernels: relative L2 state error <= 1e-11 after tens to hundreds of
  steps, scalars (MU, mu, n) <= 1e-11 relative - rounding-level agreement
  (different FFT factorisation and summation order than pocketfft).
* FP32 kernels: relative L2 <= 2e-5 per 100 steps of smooth states,
  ground-state energy / mu <= 1e-6 relative.
"""
import math

import numpy as np
import pytest

from oracle import gpe_oracle as O
from tests.golden import make_golden as MG

pytestmark = pytest.mark.gpu

SIZES = [8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024]


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def harmonic(lam):
    def V(X, Y, Z):
        v = 0.5 * ((lam[0] * X) ** 2 + (lam[1] * Y) ** 2)
        if len(lam) == 3:
            v = v + 0.5 * (lam[2] * Z) ** 2
        return v
    return V


def make_pair(gpe, axes_args, V, precision, **props):
    """The same task in the product (GPU) and in the oracle (CPU)."""
    if len(axes_args) == 4:
        grid = gpe.grid2d(*axes_args, precision=precision)
    else:
        grid = gpe.grid3d(*axes_args, precision=precision)
    task = gpe.GPEtask(grid, V)
    og = O.Grid(*axes_args)
    ot = O.GPEtask(og, V)
    for k, v in props.items():
        setattr(task, k, v)
        setattr(ot, k, v)
    return grid, task, og, ot


# ---- golden fixtures --------------------------------------------------------
@pytest.mark.parametrize("precision", ["double", "single"])
def test_golden_itp_then_vortex_dynamics_2d(gpe, precision):
    ref = np.load(MG.path("itp_vortex2d_64"))
    grid = gpe.grid2d(17, 64, 17, 64, precision=precision)
    task = gpe.GPEtask(grid, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2))
    task.Ntotal, task.g = 1e5, 0.06
    phi, MU, MU2, EE = task.groundstate_itp(0.02, 1e-6, ref["psi0"], nargout=4)
    assert task.last_itp.converged
    if precision == "double":
        assert len(MU) == len(ref["MU"])
        np.testing.assert_allclose(MU, ref["MU"], rtol=1e-11)
        chk = ref["MU2"] != 0
        np.testing.assert_allclose(MU2[chk], ref["MU2"][chk], rtol=1e-11)
        np.testing.assert_allclose(EE[chk], ref["EE"][chk], rtol=1e-11)
        assert rel_l2(phi, ref["phi"]) < 1e-11
    else:
        # FP32 phase + FP64 polish: same fixed point, energy/mu within 1e-6.
        assert task.last_itp.fp32_iters > 0
        assert MU[-1] == pytest.approx(ref["MU"][-1], rel=1e-6)
        assert EE[-1] == pytest.approx(ref["EE"][-1], rel=1e-6)
        assert rel_l2(phi, ref["phi"]) < 1e-5
    # vortex imprint (host, example1_vortex.m:26-30) is the oracle's bit for bit
    vort = gpe.imprint_vortex(grid, ref["phi"], 0.06, 5.0)
    np.testing.assert_allclose(vort, ref["vortex"], rtol=1e-14, atol=1e-12)
    task.init_state = ref["vortex"]
    task.current_iter = 0
    task.solve_split(0.004, 50, 4)
    tol = 1e-11 if precision == "double" else 2e-4
    assert rel_l2(task.current_state, ref["psi_t"]) < tol
    np.testing.assert_allclose(task.history["mu"], ref["hist_mu"], rtol=tol)
    np.testing.assert_allclose(task.history["n"], ref["hist_n"], rtol=tol)
    assert task.current_time == pytest.approx(float(ref["current_time"]))
    assert task.current_iter == 4


@pytest.mark.parametrize("precision", ["double", "single"])
def test_golden_damped_decay_radix3_2d(gpe, precision):
    ref = np.load(MG.path("split_damped2d_48"))
    grid = gpe.grid2d(6, 48, 5, 48, precision=precision)
    task = gpe.GPEtask(grid, lambda X, Y, Z: 0.5 * (X ** 2 + (1.3 * Y) ** 2))
    task.Ntotal, task.g, task.gamma, task.decay_rate = 50.0, 1.0, 0.05, 2.0
    task.init_state = ref["psi0"]
    task.solve_split(0.01, 10, 3)
    tol = 1e-11 if precision == "double" else 2e-5
    assert rel_l2(task.current_state, ref["psi_t"]) < tol
    np.testing.assert_allclose(task.history["mu"], ref["hist_mu"], rtol=tol)
    np.testing.assert_allclose(task.history["n"], ref["hist_n"], rtol=tol)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_golden_3d_unequal_axes(gpe, precision):
    ref = np.load(MG.path("split3d_24x32x16"))
    grid = gpe.grid3d(5, 24, 6, 32, 4, 16, precision=precision)
    task = gpe.GPEtask(grid, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2 + (1.5 * Z) ** 2))
    task.g = 1.0
    task.init_state = ref["psi0"]
    task.solve_split(0.005, 10, 2)
    tol = 1e-11 if precision == "double" else 2e-5
    assert rel_l2(task.current_state, ref["psi_t"]) < tol
    np.testing.assert_allclose(task.history["mu"], ref["hist_mu"], rtol=tol)
    np.testing.assert_allclose(task.history["n"], ref["hist_n"], rtol=tol)


def test_golden_itp_adjust_stepsize_3d(gpe):
    ref = np.load(MG.path("itp3d_adjust_16"))
    grid = gpe.grid3d(5, 16, 5, 16, 4, 16, precision="double")
    task = gpe.GPEtask(grid, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2 + (2 * Z) ** 2))
    task.Ntotal, task.g, task.itp_adjust_stepsize = 20.0, 1.0, True
    phi, MU, MU2, EE = task.groundstate_itp(0.05, 1e-5, ref["psi0"], nargout=4)
    assert len(MU) == len(ref["MU"])
    np.testing.assert_allclose(MU, ref["MU"], rtol=1e-11)
    assert rel_l2(phi, ref["phi"]) < 1e-11


# ---- every FFT length on both pass layouts -------------------------------------
@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("precision", ["double", "single"])
def test_every_axis_length_contig_and_strided(gpe, n, precision):
    rng = np.random.default_rng(n)
    for nx, ny in ((n, 8), (8, n)):
        grid, task, og, ot = make_pair(gpe, (3.0, nx, 2.0, ny), harmonic((1.0, 1.7)), precision, g=0.7)
        X, Y = og.mesh["x"], og.mesh["y"]
        psi0 = np.exp(-(X ** 2 + Y ** 2)) * (1 + 0.05 * rng.standard_normal(og.shape)) * np.exp(0.3j * X)
        task.init_state = psi0
        ot.init_state = psi0
        task.solve_split(0.002, 3, 2)   # 3 % n_recalc != 0 -> n_rec = 1 (solve_split.m:25-27)
        ot.solve_split(0.002, 3, 2)
        tol = 1e-11 if precision == "double" else 2e-5
        assert rel_l2(task.current_state, ot.current_state) < tol, (nx, ny)
        np.testing.assert_allclose(task.history["mu"], ot.history["mu"], rtol=tol)


@pytest.mark.parametrize("n", [128, 192, 256, 384, 512])
def test_alternative_fft_plans_contig_and_strided(gpe, n):
    """The autotuner's alternative plans (twice the threads per pencil) give
    the same step as the oracle on both pass layouts (FP32 tolerance)."""
    rng = np.random.default_rng(n + 1)
    for nx, ny in ((n, 8), (8, n)):
        grid, task, og, ot = make_pair(gpe, (3.0, nx, 2.0, ny), harmonic((1.0, 1.7)), "single", g=0.7)
        chosen = task.autotune(3)
        assert chosen[0] == (1 if nx == n else -1) and chosen[1] == (1 if ny == n else -1)
        X, Y = og.mesh["x"], og.mesh["y"]
        psi0 = np.exp(-(X ** 2 + Y ** 2)) * (1 + 0.05 * rng.standard_normal(og.shape)) * np.exp(0.3j * X)
        task.init_state = psi0
        ot.init_state = psi0
        task.solve_split(0.002, 3, 2)
        ot.solve_split(0.002, 3, 2)
        assert rel_l2(task.current_state, ot.current_state) < 2e-5, (nx, ny)
        np.testing.assert_allclose(task.history["mu"], ot.history["mu"], rtol=2e-5)


def test_autotuner_choices_and_results(gpe):
    """Tuning picks a plan per axis (cached per shape), and the tuned context
    reproduces the oracle; mode 0 restores the default plans."""
    axes = (6.0, 128, 6.0, 256, 4.0, 64)
    grid, task, og, ot = make_pair(gpe, axes, harmonic((1.0, 1.0, 1.5)), "single", g=0.5)
    chosen = task.autotune(1)
    assert chosen[0] in (0, 1, 2, 3) and chosen[1] in (0, 1, 2, 3) and chosen[2] == -1
    assert task.autotune(1) == chosen  # cached per device and shape
    X, Y, Z = og.mesh["x"], og.mesh["y"], og.mesh["z"]
    psi0 = (np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2) * np.exp(0.2j * Y)).astype(complex)
    task.init_state = psi0
    ot.init_state = psi0
    task.solve_split(0.002, 10, 1)
    ot.solve_split(0.002, 10, 1)
    assert rel_l2(task.current_state, ot.current_state) < 2e-5
    assert task.autotune(0) == (0, 0, -1)  # x = 128 and y = 256 have two plans, z = 64 one


# ---- semantics -----------------------------------------------------------------
def test_observables_match_applyham_and_get_energy(gpe):
    grid, task, og, ot = make_pair(gpe, (4.0, 32, 3.0, 48, 2.0, 24), harmonic((1.0, 1.2, 2.0)), "double", g=1.3)
    rng = np.random.default_rng(3)
    X, Y, Z = og.mesh["x"], og.mesh["y"], og.mesh["z"]
    psi = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2) * (1 + 0.1 * rng.standard_normal(og.shape)) * np.exp(0.2j * Y)
    o = task.observables(psi)
    assert o["energy"] == pytest.approx(ot.get_energy(psi), rel=1e-12)
    assert o["mu_integral"] == pytest.approx(np.real(og.inner(psi, ot.applyham(psi))), rel=1e-12)
    assert o["norm"] == pytest.approx(og.integrate(np.abs(psi) ** 2), rel=1e-13)


def test_time_dependent_potential_and_callbacks(gpe):
    lam = (1.0, 1.0)
    grid, task, og, ot = make_pair(gpe, (5.0, 32, 5.0, 32), harmonic(lam), "double", g=0.5, Ntotal=10.0,
                                   gamma=0.02)

    def Vtd(t_, time):
        return 0.3 * math.sin(2.0 * time) * t_.grid.mesh["x"]

    task.Vtd = Vtd
    ot.Vtd = Vtd
    seen_gpu, seen_ref = [], []
    task.user_callback = lambda t_: seen_gpu.append((t_.current_iter, t_.current_time, t_.current_state.copy()))
    ot.user_callback = lambda t_: seen_ref.append((t_.current_iter, t_.current_time, t_.current_state.copy()))
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = math.sqrt(10.0) * og.normalize(np.exp(-((X - 0.5) ** 2 + Y ** 2) / 2).astype(complex))
    task.init_state = psi0
    ot.init_state = psi0
    task.solve_split(0.01, 20, 3)
    ot.solve_split(0.01, 20, 3)
    assert [s[0] for s in seen_gpu] == [1, 2, 3]
    for (ig, tg, pg), (ir, tr, pr) in zip(seen_gpu, seen_ref):
        assert ig == ir and tg == pytest.approx(tr)
        assert rel_l2(pg, pr) < 1e-11
    np.testing.assert_allclose(task.history["mu"], ot.history["mu"], rtol=1e-11)


def test_resume_matches_reference_restart_semantics(gpe):
    grid, task, og, ot = make_pair(gpe, (6.0, 32, 6.0, 32), harmonic((1.0, 1.4)), "double", g=2.0)
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = np.exp(-(X ** 2 + Y ** 2) / 3) * np.exp(0.2j * X)
    for t_ in (task, ot):
        t_.init_state = psi0
        t_.solve_split(0.005, 10, 2)
        t_.solve_split(0.005, 10, 5)  # resumes at current_iter = 2 (solve_split.m:29,34-38)
    assert task.current_iter == 5 and len(task.history["mu"]) == 5
    assert rel_l2(task.current_state, ot.current_state) < 1e-11
    np.testing.assert_allclose(task.history["n"], ot.history["n"], rtol=1e-11)


def test_itp_without_ntotal_uses_mu_init_branch(gpe):
    grid, task, og, ot = make_pair(gpe, (5.0, 32, 5.0, 32), harmonic((1.0, 1.0)), "double", g=1.0, mu_init=3.0)
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = (2.0 * np.exp(-(X ** 2 + Y ** 2) / 4)).astype(complex)
    task.itp_max_iter = ot.itp_max_iter = 300
    phi, MU, MU2, EE = task.groundstate_itp(0.01, 1e-9, psi0, nargout=4)
    with pytest.warns(UserWarning):
        ophi, oMU, oMU2, oEE = ot.groundstate_itp(0.01, 1e-9, psi0)
    assert len(MU) == len(oMU)
    np.testing.assert_allclose(MU, oMU, rtol=1e-11)
    assert rel_l2(phi, ophi) < 1e-11


def test_gamma0_conserves_norm_fp32(gpe):
    grid = gpe.grid3d(6, 64, 6, 64, 6, 64, precision="single")
    task = gpe.GPEtask(grid, harmonic((1.0, 1.0, 2.0)))
    task.g = 1.0
    X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
    psi0 = np.exp(-(X ** 2 + Y ** 2 + 2 * Z ** 2) / 2) * np.exp(0.3j * X)
    task.init_state = psi0
    task.solve_split(0.002, 50, 4)
    n0 = grid.integrate(np.abs(psi0) ** 2)
    # FP32 rounding of unit-modulus factors leaves a drift of a few 1e-8 per
    # step (the FP64 path conserves to ~1e-17 per step): bound 1e-7 per step.
    np.testing.assert_allclose(task.history["n"], n0, rtol=200 * 1e-7)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_batched_uneven_grids_match_individual_runs(gpe, precision):
    """solve_split_batch (one CUDA graph per block, chains of all grids run
    concurrently) gives each task exactly what its own solve_split gives."""
    specs = [((4.0, 32, 4.0, 32), 0.8, 0.0), ((5.0, 48, 4.0, 64), 1.5, 0.02),
             ((6.0, 64, 6.0, 24), 0.5, 0.0), ((3.0, 24, 3.0, 32), 2.0, 0.05)]

    def make(spec):
        axes, g, gam = spec
        grid = gpe.grid2d(*axes, precision=precision)
        t = gpe.GPEtask(grid, harmonic((1.0, 1.3)))
        t.g, t.gamma, t.Ntotal = g, gam, 5.0
        X, Y = grid.mesh["x"], grid.mesh["y"]
        t.init_state = np.sqrt(5.0) * grid.normalize(np.exp(-(X ** 2 + Y ** 2) / 2 + 0.4j * X))
        return t

    singles = [make(s) for s in specs]
    for t in singles:
        t.solve_split(0.003, 20, 3)
    batch = [make(s) for s in specs]
    gpe.solve_split_batch(batch, 0.003, 20, 3)
    tol = 1e-12 if precision == "double" else 1e-6
    for a, b in zip(singles, batch):
        assert b.current_iter == 3 and b.current_time == pytest.approx(a.current_time)
        assert rel_l2(b.current_state, a.current_state) < tol
        np.testing.assert_allclose(b.history["mu"], a.history["mu"], rtol=tol)
        np.testing.assert_allclose(b.history["n"], a.history["n"], rtol=tol)


def test_batched_rejects_host_callbacks(gpe):
    grid = gpe.grid2d(3, 16, 3, 16)
    t = gpe.GPEtask(grid, harmonic((1.0, 1.0)))
    t.init_state = np.ones(grid.shape, complex)
    t.decay_rate = 1.0
    with pytest.raises(gpe.GPEError):
        gpe.solve_split_batch([t], 0.01, 10, 1)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_tma_pass_variant_matches_direct(gpe, precision):
    """The TMA-staged passes run the same per-point arithmetic as the direct
    passes; only the order of the norm/energy sums differs, so results agree
    to rounding (3D, damping, renormalisation, ITP)."""
    out = []
    for variant in (0, 1):
        grid = gpe.grid3d(6, 32, 6, 64, 6, 48, precision=precision)
        task = gpe.GPEtask(grid, harmonic((1.0, 1.2, 1.7)))
        task.set_pass_variant(variant)
        task.Ntotal, task.g, task.gamma = 30.0, 1.0, 0.02
        X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
        psi0 = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 3).astype(complex)
        task.itp_max_iter = 200
        phi = task.groundstate_itp(0.01, 1e-12, psi0)
        task.init_state = phi * np.exp(0.3j * X)
        task.solve_split(0.002, 20, 2)
        out.append((phi, task.current_state, np.array(task.history["mu"])))
    tol = 1e-12 if precision == "double" else 2e-5
    assert rel_l2(out[1][0], out[0][0]) < tol
    assert rel_l2(out[1][1], out[0][1]) < tol
    np.testing.assert_allclose(out[1][2], out[0][2], rtol=tol)


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("tensor", ["1", "0"], ids=["tensor_boxes", "row_copies"])
def test_tma_strided_tiles_512_match_direct(gpe, monkeypatch, precision, tensor):
    """The TMA pass's strided tiles as tensor-map boxes (two boxes of 256
    positions per pencil at N = 512) and as per-row bulk copies: x pass of
    length 512 and z pass of length 256 on a 512 x 32 x 256 grid, against the
    direct passes (rounding of the sums only)."""
    monkeypatch.setenv("GPE_TMA_TENSOR", tensor)
    out = []
    for variant in (0, 1):
        grid = gpe.grid3d(8, 512, 4, 32, 6, 256, precision=precision)
        task = gpe.GPEtask(grid, harmonic((1.0, 1.5, 1.2)))
        task.set_pass_variant(variant)
        task.Ntotal, task.g, task.gamma = 30.0, 0.8, 0.01
        X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
        task.init_state = (np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 3) * np.exp(0.3j * X)).astype(complex)
        task.solve_split(0.002, 10, 2)
        out.append((task.current_state, np.array(task.history["mu"])))
        task.close()
    tol = 1e-12 if precision == "double" else 2e-6
    assert rel_l2(out[1][0], out[0][0]) < tol
    np.testing.assert_allclose(out[1][1], out[0][1], rtol=tol)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_l2_prefetch_variant_is_bit_identical(gpe, precision):
    """Variant 0 only adds L2 prefetch hints to variant 2's passes: the
    arithmetic and the reduction order are those of the direct passes, so the
    results are identical.  The grid is large enough that every axis pass
    launches more CTAs than one resident wave (the prefetch path runs)."""
    out = []
    for variant in (0, 2):
        grid = gpe.grid3d(8, 256, 8, 256, 8, 64, precision=precision)
        task = gpe.GPEtask(grid, harmonic((1.0, 1.0, 2.0)))
        task.set_pass_variant(variant)
        task.Ntotal, task.g, task.gamma = 1e3, 0.5, 0.01
        X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
        psi0 = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 4).astype(complex)
        task.itp_max_iter = 60
        task.itp_min_iter = 10
        phi = task.groundstate_itp(0.005, 1e-12, psi0)
        task.init_state = phi * np.exp(0.3j * X)
        task.solve_split(0.002, 20, 2)
        out.append((phi, task.current_state, np.array(task.history["mu"])))
    np.testing.assert_array_equal(out[1][0], out[0][0])
    np.testing.assert_array_equal(out[1][1], out[0][1])
    np.testing.assert_array_equal(out[1][2], out[0][2])


@pytest.mark.parametrize("axes,n_rec", [((4.0, 64, 5.0, 48), 10), ((4.0, 64, 5.0, 48), 5),
                                         ((5.0, 24, 6.0, 32, 4.0, 16), 10), ((5.0, 24, 6.0, 32, 4.0, 16), 3)])
def test_folded_steps_match_unfolded_and_oracle(gpe, monkeypatch, axes, n_rec):
    """Folded steps (consecutive steps take the axes in opposite orders and
    share one pass, the default) against the same run with GPE_FOLD=0 (y x z
    every step) and against the FP64 oracle: the kinetic factors commute, so
    the two orders agree to rounding.  FP64 with gamma > 0 (mu feeds back
    every block) and an even and an odd n_recalc (the block ends on the y or
    on the last axis)."""
    V = harmonic((1.0, 1.3, 1.6)[: len(axes) // 2])
    out = []
    for fold in ("1", "0"):
        monkeypatch.setenv("GPE_FOLD", fold)
        monkeypatch.setenv("GPE_CLUSTER", "0")  # the per-pass path (2D grids this small take the cluster kernel)
        grid, task, og, ot = make_pair(gpe, axes, V, "double", g=0.7, gamma=0.02, Ntotal=20.0)
        task.n_recalc = n_rec
        ot.n_recalc = n_rec
        X = og.mesh["x"]
        psi0 = np.exp(-sum(og.mesh[k] ** 2 for k in og.mesh) / 3) * np.exp(0.4j * X)
        task.init_state = psi0
        task.solve_split(0.003, 2 * n_rec, 2)
        out.append((task.current_state, np.array(task.history["mu"])))
        if fold == "1":
            ot.init_state = psi0
            ot.solve_split(0.003, 2 * n_rec, 2)
            assert rel_l2(task.current_state, ot.current_state) < 1e-11
            np.testing.assert_allclose(task.history["mu"], ot.history["mu"], rtol=1e-11)
        task.close()
    assert rel_l2(out[0][0], out[1][0]) < 1e-12
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-12)


def test_device_sincos_error_bound(gpe):
    """The FP32 phase factors' sin/cos: absolute error <= 2 ulp(1) = 2.4e-7
    against FP64 over the bounded range and beyond it (library fallback)."""
    from gpe_gb300 import _lib as L

    rng = np.random.default_rng(7)
    x = np.concatenate([np.linspace(-7e4, 7e4, 20001), np.linspace(-10, 10, 200001),
                        rng.uniform(-3.5, 3.5, 100000), np.array([0.0, 1e-30, -1e-8, 65536.0, -65536.0])])
    x = x.astype(np.float32)
    s = np.empty_like(x)
    c = np.empty_like(x)
    L.check(None, L.lib.gpe_selftest_trig(L.fptr(x), L.fptr(s), L.fptr(c), x.size))
    xd = x.astype(np.float64)
    assert np.max(np.abs(s - np.sin(xd))) <= 2.4e-7
    assert np.max(np.abs(c - np.cos(xd))) <= 2.4e-7
    # no systematic modulus bias over phases of one step's typical range
    m = s.astype(np.float64) ** 2 + c.astype(np.float64) ** 2 - 1
    assert abs(np.mean(m[20001:220002])) < 2e-8


def test_errors_are_reported_not_crashing(gpe):
    from gpe_gb300 import _lib as L

    grid = gpe.grid2d(3, 16, 3, 16)
    task = gpe.GPEtask(grid, lambda X, Y, Z: 0 * X)
    with pytest.raises(gpe.GPEError) as e:
        task.solve_split(-1.0, 10, 1)
    assert e.value.status == L.GPE_ERR_INVALID
    # non-finite input state is detected by the reductions, not propagated silently
    bad = np.ones(grid.shape, complex)
    bad[3, 3] = np.nan
    task.init_state = bad
    task.g = 1.0
    with pytest.raises(gpe.GPEError) as e:
        task.solve_split(0.01, 10, 1)
    assert e.value.status == L.GPE_ERR_NONFINITE
