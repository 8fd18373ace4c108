"""Parity on the benchmark configurations themselves, at their real sizes,
against the FP64 oracle (the restatement of groundstate_itp.m:19-111 and
solve_split.m:13-84), through the C ABI.

* vortex2d_256 (the 2D example, example1_vortex.m:11-35 with the seeded
  Gaussian start): the whole workload - ITP at dt 0.02 / eps 1e-6 with
  MU/MU2/EE, the vortex at x0 = 5, then 20 outer x 50 inner steps of 0.004.
* damped3d_256 (256^3, +-12, lambda 4, g 0.5, N 1e5): the whole ITP to
  convergence (E and mu of the ground state), 50 ITP iterations from the
  seeded start, and 100 damped real-time steps (gamma 0.01, dt 0.002).
* ring3d_512 (512^3, +-24, lambda (1,1,2), g 1, N 1e6): 10 ITP iterations
  from the seeded start, the vortex ring at 0.5 R_TF, 10 real-time steps.

Tolerances (written per case):
* FP64 kernels: state rel. L2 <= 1e-11, MU / history mu and n <= 1e-11
  relative (rounding-level: a different FFT factorisation and summation order
  than pocketfft).
* FP32 kernels: ground-state energy and mu <= 1e-6 relative of the oracle's
  (north star; measured 4e-12 / 1e-10 at 256^2 and 1e-13 / 2e-11 at 256^3,
  the FP64 polish of the FP32 ITP); the FP32 state error at the fixed
  horizons is printed (``CONFIG-PARITY`` lines) and bounded per case below.

The oracle runs on the host cores (scipy.fft, all workers); the 256^3 and
512^3 cases take a few minutes of CPU time in all.
"""
import json
import math

import numpy as np
import pytest

from gpe_workloads import DAMPED3D, RING3D, VORTEX2D
from oracle import gpe_oracle as O

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def rel(a, b):
    return float(abs(a - b) / abs(b))


def report(case, precision, **errs):
    print("CONFIG-PARITY " + json.dumps({"case": case, "precision": precision, **errs}), flush=True)


def oracle_task(W):
    gargs = [v for pair in zip(W.box, W.n) for v in pair]
    og = O.Grid(*gargs)
    ot = O.GPEtask(og, W.potential())
    ot.Ntotal, ot.g, ot.gamma = W.Ntotal, W.g, W.gamma
    return og, ot


def gpu_task(gpe, W, precision):
    grid, task = W.make_task(precision)
    return grid, task


# ---- vortex2d_256: the whole 2D example ------------------------------------------
@pytest.fixture(scope="module")
def vortex2d_oracle():
    W = VORTEX2D
    og, ot = oracle_task(W)
    psi0 = W.initial_state(og)
    phi, MU, MU2, EE = ot.groundstate_itp(W.itp_dt, W.itp_eps, psi0, nargout=4)
    vort = O.imprint_vortex(og, phi, W.g, W.vortex_x0)
    ot.init_state = vort
    ot.current_iter = 0
    ot.solve_split(W.dt, W.niter_inner, W.niter_outer)
    return {"psi0": psi0, "phi": phi, "MU": MU, "MU2": MU2, "EE": EE, "vortex": vort,
            "psi_t": ot.current_state, "hist_mu": np.array(ot.history["mu"]), "hist_n": np.array(ot.history["n"]),
            "time": ot.current_time}


@pytest.mark.parametrize("precision", ["double", "single"])
def test_vortex2d_256_whole_workload_against_oracle(gpe, vortex2d_oracle, precision):
    W, ref = VORTEX2D, vortex2d_oracle
    grid, task = gpu_task(gpe, W, precision)
    phi, MU, MU2, EE = task.groundstate_itp(W.itp_dt, W.itp_eps, ref["psi0"], nargout=4)
    assert task.last_itp.converged
    chk = ref["MU2"] != 0
    e_itp = {"itp_iters": int(len(MU)), "oracle_itp_iters": int(len(ref["MU"])),
             "E_rel": rel(EE[-1], ref["EE"][-1]), "mu_rel": rel(MU[-1], ref["MU"][-1]),
             "MU2_rel": rel(MU2[-1], ref["MU2"][-1]), "ground_state_rel_l2": rel_l2(phi, ref["phi"])}
    # the dynamics start from the oracle's vortex state on both sides
    task.init_state = ref["vortex"]
    task.current_iter = 0
    task.solve_split(W.dt, W.niter_inner, W.niter_outer)
    e_dyn = {"state_rel_l2_after_1000_steps": rel_l2(task.current_state, ref["psi_t"]),
             "hist_mu_max_rel": float(np.max(np.abs(np.array(task.history["mu"]) - ref["hist_mu"]) / np.abs(ref["hist_mu"]))),
             "hist_n_max_rel": float(np.max(np.abs(np.array(task.history["n"]) - ref["hist_n"]) / np.abs(ref["hist_n"])))}
    report("vortex2d_256", precision, **e_itp, **e_dyn)
    assert task.current_iter == W.niter_outer and task.current_time == pytest.approx(ref["time"])
    if precision == "double":
        assert len(MU) == len(ref["MU"])
        np.testing.assert_allclose(MU, ref["MU"], rtol=1e-11)
        np.testing.assert_allclose(MU2[chk], ref["MU2"][chk], rtol=1e-11)
        np.testing.assert_allclose(EE[chk], ref["EE"][chk], rtol=1e-11)
        assert e_itp["ground_state_rel_l2"] < 1e-11
        assert e_dyn["state_rel_l2_after_1000_steps"] < 1e-11
        assert e_dyn["hist_mu_max_rel"] < 1e-11 and e_dyn["hist_n_max_rel"] < 1e-11
    else:
        assert e_itp["E_rel"] < 1e-6 and e_itp["mu_rel"] < 1e-6 and e_itp["MU2_rel"] < 1e-6
        assert e_itp["ground_state_rel_l2"] < 1e-5
        # FP32 vortex dynamics over 1000 steps: measured 6.2e-4 (state), 9.4e-6
        # (mu) and 2.0e-5 (norm drift, ~2e-8 per step)
        assert e_dyn["state_rel_l2_after_1000_steps"] < 5e-3
        assert e_dyn["hist_mu_max_rel"] < 5e-5 and e_dyn["hist_n_max_rel"] < 5e-5
    task.close()


# ---- damped3d_256 ------------------------------------------------------------------
@pytest.fixture(scope="module")
def damped3d_oracle():
    """50 ITP iterations from the seeded start, then 100 damped steps (one outer
    step of 100, n_recalc 10) from that state."""
    W = DAMPED3D
    og, ot = oracle_task(W)
    psi0 = W.initial_state(og)
    ot.itp_max_iter = 50
    with pytest.warns(UserWarning):
        phi50, MU50, _, _ = ot.groundstate_itp(W.itp_dt, W.itp_eps, psi0, nargout=2)
    ot.init_state = phi50
    ot.current_iter = 0
    ot.solve_split(W.dt, 100, 1)
    return {"psi0": psi0, "phi50": phi50, "MU50": MU50, "psi_t": ot.current_state,
            "mu": ot.history["mu"][0], "n": ot.history["n"][0]}


@pytest.mark.parametrize("precision", ["double", "single"])
def test_damped3d_256_short_horizons_against_oracle(gpe, damped3d_oracle, precision):
    W, ref = DAMPED3D, damped3d_oracle
    grid, task = gpu_task(gpe, W, precision)
    task.itp_max_iter = 50
    with pytest.warns(UserWarning):
        phi50, MU50 = task.groundstate_itp(W.itp_dt, W.itp_eps, ref["psi0"], nargout=2)
    assert len(MU50) == 50
    e = {"itp50_state_rel_l2": rel_l2(phi50, ref["phi50"]), "itp50_MU_max_rel":
         float(np.max(np.abs(MU50 - ref["MU50"]) / np.abs(ref["MU50"])))}
    task.init_state = ref["phi50"]
    task.current_iter = 0
    task.solve_split(W.dt, 100, 1)
    e.update({"state_rel_l2_after_100_steps": rel_l2(task.current_state, ref["psi_t"]),
              "mu_rel_after_100_steps": rel(task.history["mu"][0], ref["mu"]),
              "n_rel_after_100_steps": rel(task.history["n"][0], ref["n"])})
    report("damped3d_256", precision, **e)
    if precision == "double":
        assert e["itp50_state_rel_l2"] < 1e-11 and e["itp50_MU_max_rel"] < 1e-11
        assert e["state_rel_l2_after_100_steps"] < 1e-11
        assert e["mu_rel_after_100_steps"] < 1e-11 and e["n_rel_after_100_steps"] < 1e-11
    else:
        assert e["itp50_state_rel_l2"] < 1e-4 and e["itp50_MU_max_rel"] < 1e-5
        assert e["state_rel_l2_after_100_steps"] < 1e-4
        assert e["mu_rel_after_100_steps"] < 1e-5 and e["n_rel_after_100_steps"] < 1e-5
    task.close()


@pytest.fixture(scope="module")
def damped3d_ground_oracle():
    """The converged ITP ground state of the 256^3 workload (MU, MU2, EE)."""
    W = DAMPED3D
    og, ot = oracle_task(W)
    psi0 = W.initial_state(og)
    phi, MU, MU2, EE = ot.groundstate_itp(W.itp_dt, W.itp_eps, psi0, nargout=4)
    return {"psi0": psi0, "phi": phi, "MU": MU, "MU2": MU2, "EE": EE}


@pytest.mark.parametrize("precision", ["double", "single"])
def test_damped3d_256_ground_state_energy_against_oracle(gpe, damped3d_ground_oracle, precision):
    W, ref = DAMPED3D, damped3d_ground_oracle
    grid, task = gpu_task(gpe, W, precision)
    phi, MU, MU2, EE = task.groundstate_itp(W.itp_dt, W.itp_eps, ref["psi0"], nargout=4)
    assert task.last_itp.converged
    e = {"itp_iters": int(len(MU)), "oracle_itp_iters": int(len(ref["MU"])),
         "fp32_iters": int(task.last_itp.fp32_iters),
         "E_rel": rel(EE[-1], ref["EE"][-1]), "mu_rel": rel(MU[-1], ref["MU"][-1]),
         "MU2_rel": rel(MU2[-1], ref["MU2"][-1]), "ground_state_rel_l2": rel_l2(phi, ref["phi"])}
    report("damped3d_256_ground_state", precision, **e)
    if precision == "double":
        assert len(MU) == len(ref["MU"])
        np.testing.assert_allclose(MU, ref["MU"], rtol=1e-11)
        assert e["E_rel"] < 1e-11 and e["MU2_rel"] < 1e-11 and e["ground_state_rel_l2"] < 1e-11
    else:
        assert e["E_rel"] < 1e-6 and e["mu_rel"] < 1e-6 and e["MU2_rel"] < 1e-6
        assert e["ground_state_rel_l2"] < 1e-5
    task.close()


# ---- ring3d_512 ---------------------------------------------------------------------
@pytest.fixture(scope="module")
def ring3d_oracle():
    """10 ITP iterations from the seeded start, the vortex ring at 0.5 R_TF
    (R_TF from the workload's Thomas-Fermi mu), then one block of 10 steps."""
    W = RING3D
    og, ot = oracle_task(W)
    psi0 = W.initial_state(og)
    ot.itp_max_iter = 10
    with pytest.warns(UserWarning):
        phi10, MU10, _, _ = ot.groundstate_itp(W.itp_dt, W.itp_eps, psi0, nargout=2)
    return {"og": og, "ot": ot, "psi0": psi0, "phi10": phi10, "MU10": MU10}


@pytest.mark.parametrize("precision", ["double", "single"])
def test_ring3d_512_short_horizons_against_oracle(gpe, ring3d_oracle, precision):
    W, ref = RING3D, ring3d_oracle
    grid, task = gpu_task(gpe, W, precision)
    task.itp_max_iter = 10
    with pytest.warns(UserWarning):
        phi10, MU10 = task.groundstate_itp(W.itp_dt, W.itp_eps, ref["psi0"], nargout=2)
    e = {"itp10_state_rel_l2": rel_l2(phi10, ref["phi10"]),
         "itp10_MU_max_rel": float(np.max(np.abs(MU10 - ref["MU10"]) / np.abs(ref["MU10"])))}
    del phi10
    if "psi_t" not in ref:
        # the ring on the oracle's state (host FP64 imprint, shared by both sides)
        mu_tf = 0.5 * (15 * W.Ntotal * W.g * W.trap[0] * W.trap[1] * W.trap[2] / (8 * math.pi)) ** 0.4
        r_tf = math.sqrt(2.0 * mu_tf) / W.trap[0]
        ref["start"] = gpe.imprint_vortex_ring(grid, ref["phi10"], W.g, W.ring_frac * r_tf)
        ot = ref["ot"]
        ot.init_state = ref["start"]
        ot.current_iter = 0
        ot.solve_split(W.dt, 10, 1)
        ref["psi_t"], ref["mu"], ref["n"] = ot.current_state, ot.history["mu"][0], ot.history["n"][0]
    task.init_state = ref["start"]
    task.current_iter = 0
    task.solve_split(W.dt, 10, 1)
    e.update({"state_rel_l2_after_10_steps": rel_l2(task.current_state, ref["psi_t"]),
              "mu_rel_after_10_steps": rel(task.history["mu"][0], ref["mu"]),
              "n_rel_after_10_steps": rel(task.history["n"][0], ref["n"])})
    report("ring3d_512", precision, **e)
    if precision == "double":
        assert e["itp10_state_rel_l2"] < 1e-11 and e["itp10_MU_max_rel"] < 1e-11
        assert e["state_rel_l2_after_10_steps"] < 1e-11
        assert e["mu_rel_after_10_steps"] < 1e-11 and e["n_rel_after_10_steps"] < 1e-11
    else:
        assert e["itp10_state_rel_l2"] < 1e-4 and e["itp10_MU_max_rel"] < 1e-5
        assert e["state_rel_l2_after_10_steps"] < 1e-4
        assert e["mu_rel_after_10_steps"] < 1e-5 and e["n_rel_after_10_steps"] < 1e-5
    task.close()
