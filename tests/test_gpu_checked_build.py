"""The bounds-checked build (-DGPE_CHECK=1, libgpe_check.so) on the small
parity cases.

In that build every global index of the axis-pass kernels (scalar, paired,
TMA-staged, cluster, grid-wide and multi-grid) is checked against the extent of its
pass, and every shared-memory exchange index against its buffer; a
violation is recorded, the access skipped, and the run returns
GPE_ERR_BOUNDS.  The cases below run in a child process that loads the
checked library (GPE_LIB) and compare against the FP64 oracle and the golden
fixtures with the ordinary tolerances (FP64 1e-11, FP32 2e-5): no index may
leave its range and the results must stay right.  The checked library is
built on first use (about two minutes of nvcc).
"""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "gpe-matlab_gb300"
CHECK_LIB = PKG / "libgpe_check.so"

pytestmark = pytest.mark.gpu


def build_checked():
    import importlib.util

    spec = importlib.util.spec_from_file_location("gpe_build_lib_check", PKG / "build_lib.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(out=CHECK_LIB, build_dir=PKG / "_build_check", defines=["GPE_CHECK=1"])


def run_cases():
    """Runs in the child process (GPE_LIB = the checked library)."""
    for p in (str(ROOT), str(PKG)):
        if p not in sys.path:
            sys.path.insert(0, p)
    import gpe_gb300 as gpe
    from oracle import gpe_oracle as O
    from tests.golden import make_golden as MG
    from tests.test_gpu_parity import harmonic, make_pair, rel_l2

    assert os.environ.get("GPE_LIB", "").endswith("libgpe_check.so")
    n = 0
    rng = np.random.default_rng(0)

    def gauss(og, k=0.3):
        X, Y = og.mesh["x"], og.mesh["y"]
        r2 = X ** 2 + Y ** 2 + (og.mesh["z"] ** 2 if "z" in og.mesh else 0.0)
        return np.exp(-r2) * (1 + 0.05 * rng.standard_normal(og.shape)) * np.exp(1j * k * X)

    def split_case(axes, precision, mode=None, variant=0, gamma=0.01, steps=(6, 2)):
        grid, task, og, ot = make_pair(gpe, axes, harmonic((1.0, 1.3, 1.7)[: len(axes) // 2]), precision,
                                       g=0.6, gamma=gamma)
        if mode is not None:
            task.autotune(mode)
        task.set_pass_variant(variant)
        psi0 = gauss(og)
        task.init_state = psi0
        ot.init_state = psi0
        task.solve_split(0.002, *steps)
        ot.solve_split(0.002, *steps)
        tol = 1e-11 if precision == "double" else 2e-5
        err = rel_l2(task.current_state, ot.current_state)
        assert err < tol, (axes, precision, mode, variant, err)
        task.close()

    # every pass layout on the smallest plans and on the benchmark's lengths
    for precision in ("double", "single"):
        split_case((3.0, 8, 2.0, 12), precision)
        split_case((3.0, 16, 3.0, 16, 2.0, 16), precision)
        n += 2
    # the golden 3D fixture with unequal axes
    ref = np.load(MG.path("split3d_24x32x16"))
    for precision, tol in (("double", 1e-11), ("single", 2e-5)):
        grid = gpe.grid3d(5, 24, 6, 32, 4, 16, precision=precision)
        task = gpe.GPEtask(grid, lambda X, Y, Z: 0.5 * (X ** 2 + Y ** 2 + (1.5 * Z) ** 2))
        task.g = 1.0
        task.init_state = ref["psi0"]
        task.solve_split(0.005, 10, 2)
        assert rel_l2(task.current_state, ref["psi_t"]) < tol
        task.close()
        n += 1
    # FP32 plan variants: alternative plans, paired passes on both plans
    for mode in (3, 4, 5):
        split_case((3.0, 128, 2.0, 8), "single", mode=mode)
        split_case((3.0, 8, 2.0, 256), "single", mode=mode)
        split_case((3.0, 8, 3.0, 16, 4.0, 256), "single", mode=mode)
        n += 3
    # the TMA-staged passes (tensor boxes on the strided axes)
    split_case((6.0, 32, 6.0, 64, 6.0, 48), "single", variant=1)
    n += 1
    # imaginary time (ITP prologue/epilogue, FP64 polish) and the observables
    grid, task, og, ot = make_pair(gpe, (6.0, 32, 6.0, 48), harmonic((1.0, 1.3)), "single", Ntotal=20.0, g=0.8)
    X, Y = og.mesh["x"], og.mesh["y"]
    psi0 = np.exp(-(X ** 2 + Y ** 2) / 4).astype(complex)
    phi, MU = task.groundstate_itp(0.01, 1e-6, psi0, nargout=2)
    ophi, oMU = ot.groundstate_itp(0.01, 1e-6, psi0, nargout=2)[:2]
    assert abs(MU[-1] - oMU[-1]) / abs(oMU[-1]) < 1e-6
    o = task.observables(phi)
    assert o["energy"] == o["energy"]
    task.close()
    n += 1
    # the kernels of small 2D grids: cluster (FP64), multi-grid pass kernels
    # and grid-wide (FP32) batches
    for precision, path in (("double", "cluster"), ("single", "multi"), ("single", "grid")):
        os.environ["GPE_SMALL2D"] = path
        tasks, refs = [], []
        for axes in ((4.0, 64, 4.0, 64), (5.0, 96, 4.0, 128), (6.0, 256, 6.0, 256)):
            grid, task, og, ot = make_pair(gpe, axes, harmonic((1.0, 1.3)), precision, g=0.8, gamma=0.01, Ntotal=5.0)
            psi0 = gauss(og)
            task.init_state = psi0
            ot.init_state = psi0
            tasks.append(task)
            refs.append(ot)
        gpe.solve_split_batch(tasks, 0.003, 20, 2)
        tol = 1e-11 if precision == "double" else 2e-5
        for t, ot in zip(tasks, refs):
            ot.solve_split(0.003, 20, 2)
            assert rel_l2(t.current_state, ot.current_state) < tol
            t.close()
        n += 1
    os.environ.pop("GPE_SMALL2D", None)
    print(f"CHECKED-BUILD ok {n}", flush=True)


def test_checked_build_small_parity_cases():
    build_checked()
    env = dict(os.environ, GPE_LIB=str(CHECK_LIB))
    r = subprocess.run([sys.executable, "-c", "import tests.test_gpu_checked_build as m; m.run_cases()"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "CHECKED-BUILD ok" in r.stdout
