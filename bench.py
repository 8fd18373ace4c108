"""Benchmark: split-step grid-point-steps/s of GPEtask.solve_split on one GB300.

Workload (the damped 3D configuration): grid3d 256^3, box +-12, V = 0.5 (x^2 + y^2 +
(4 z)^2), g = 0.5, Ntotal = 1e5, ground state by imaginary-time propagation
(FP32 + FP64 polish, untimed), then real-time steps of dt = 0.002 with damping
gamma = 0.01.  One bench step = one outer step of solve_split = 100 split
steps (10 blocks of n_recalc = 10, mu feedback every block).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  `value` is complex-FP32 throughput with the state
resident in HBM; `fp64` is the same kernels in FP64 on the same start state;
`error` states the FP32 result against the FP64 one after 100 steps; `e2e`
runs each step through the C ABI (the drop-in boundary) with pinned host
buffers: gpe_set_state from the host, one outer step of gpe_solve_split,
gpe_get_state to the host.  `--impl reference` times the FP64 CPU
restatement of the reference's solve_split (the reference is MATLAB, which
this machine does not have) on the same workload, all host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (str(ROOT), str(ROOT / "gpe-matlab_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "split-step grid-pt-steps/s (complex FP32, vs FP64 same kernels)"
UNIT = "grid-pt-steps/s"
INNER = 100  # split steps per bench step (outer step of solve_split)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    """Barrier + max/sum over ranks (gloo on host tensors); no data-path collective."""

    def __init__(self):
        self.rank, self.world, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td

            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def reduce(self, x: float, op: str) -> float:
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX if op == "max" else self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi needs a moment to start: wait for its first sample so
            # that short timed regions still get one
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def flop_roofline(grid_points, steps, seconds, sm_max_mhz, sms_used=None):
    """Arithmetic roofline of an L2-resident workload: 10 log2(P) + 30 flops
    per grid-point-step for a grid of P points (FFTs of both directions on
    every axis, the kinetic factor, the phases), against the nominal FP32
    CUDA-core peak (SMs x 128 lanes x 2 flops x the maximum SM clock)."""
    import torch

    flops = sum(p * (10.0 * math.log2(p) + 30.0) for p in grid_points) * steps
    achieved = flops / seconds / 1e12
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = sm_max_mhz or 2070.0
    peak = sms * 128 * 2 * mhz * 1e6 / 1e12
    out = {"bound": "fp32 (CUDA cores)", "flops_per_point_step": "10 log2(P) + 30",
           "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
           "peak_kind": f"nominal: {sms} SMs x 128 lanes x 2 x {mhz:.0f} MHz"}
    if sms_used:
        out["sms_used"] = sms_used
        out["frac_of_sms_used"] = achieved / (peak * sms_used / sms)
    return out


def ground_state(gpe, W, precision="single", device=0):
    """Untimed setup: FP32 ITP with FP64 polish from the seeded Gaussian."""
    grid, task = W.make_task(precision, device=device)
    psi0 = W.initial_state(grid)
    phi = task.groundstate_itp(W.itp_dt, W.itp_eps, psi0)
    return grid, task, phi


def oracle_task(W, phi, cores: int):
    """The FP64 oracle's GPEtask (the restatement of the reference's solve_split)
    on the workload's grid, potential and parameters, holding phi.  Built from
    the oracle and the library-free workload tables only: nothing here loads
    libgpe.so."""
    from oracle import gpe_oracle as O

    O.set_workers(cores)
    gargs = [v for pair in zip(W.box, W.n) for v in pair]
    og = O.Grid(*gargs)
    ot = O.GPEtask(og, W.potential())
    ot.Ntotal, ot.g, ot.gamma = W.Ntotal, W.g, W.gamma
    ot.init_state = np.asarray(phi, dtype=np.complex128)
    return og, ot


def cpu_reference_run(W, phi, cores: int, warm: int, samples: int, per_sample=None, budget_s: float = 150.0):
    """Times the FP64 oracle's solve_split on the workload: `warm` untimed
    samples, then `samples` timed samples of `per_sample` split steps each.
    The clock starts after the warm-up samples, so solve_split's setup (the
    kinetic table and the applyham of solve_split.m:41) and the first steps
    are outside it.  per_sample None: chosen from the first split step's time
    so that the whole run stays near budget_s (1 .. niter_inner steps).
    Returns (grid-pt-steps/s, timed split steps, timed seconds, per_sample)."""
    og, ot = oracle_task(W, phi, cores)
    stamps = []
    plan = {"per": per_sample, "total": None}

    class Done(Exception):
        pass

    def on_inner(_j):
        stamps.append(time.perf_counter())
        if plan["total"] is None:
            if plan["per"] is None:
                t1 = stamps[0] - t0  # one split step plus the setup
                plan["per"] = int(max(1, min(W.niter_inner, budget_s / max(1, warm + samples) / t1)))
            plan["total"] = (warm + samples) * plan["per"]
        if len(stamps) >= plan["total"]:
            raise Done

    t0 = time.perf_counter()
    try:
        ot.solve_split(W.dt, W.niter_inner, 10 ** 6, inner_callback=on_inner)
    except Done:
        pass
    per = plan["per"]
    i0 = warm * per - 1
    n = len(stamps) - 1 - i0
    t = stamps[-1] - stamps[i0]
    return W.npoints * n / t, n, t, per


def oracle_block(W, phi, cores: int):
    """One block (10 split steps, n_recalc 10) of the FP64 oracle's solve_split
    from phi: (state, mu, n, grid-pt-steps/s of steps 2..10, 9, seconds)."""
    og, ot = oracle_task(W, phi, cores)
    stamps = []
    ot.solve_split(W.dt, 10, 1, inner_callback=lambda _j: stamps.append(time.perf_counter()))
    t = stamps[-1] - stamps[0]
    return (np.asarray(ot.current_state), ot.history["mu"][0], ot.history["n"][0], W.npoints * 9 / t, 9, t)


def workload_config(W):
    """The workload's description, identical in both arms' JSON lines."""
    return {"workload": W.name, "grid": list(W.n), "box": W.box[0], "trap_lambda": list(W.trap), "g": W.g,
            "Ntotal": W.Ntotal, "dt": W.dt, "gamma": W.gamma, "niter_inner": W.niter_inner, "n_recalc": 10,
            "l2": l2_note(W)}


def run_reference(args, dist):
    """--impl reference: the FP64 oracle (the restatement of the reference's
    solve_split; the reference itself is MATLAB, absent here) on the host
    cores, on the same workload as the gb300 arm.  One bench step is a
    bounded sample of split steps.  The grid, potential and start state come
    from the oracle and the library-free workload tables: this arm never
    loads libgpe.so."""
    from gpe_workloads import WORKLOADS

    if dist.rank != 0:
        return
    if args.workload not in WORKLOADS:
        print(json.dumps({"impl": "reference", "unavailable": f"{args.workload}: the reference has no gradient or "
                          "batched path; the FP64 oracle adjoint is timed as cpu_baseline of the gb300 arm"}))
        return
    W = WORKLOADS[args.workload]
    cores = os.cpu_count() or 1
    from oracle import gpe_oracle as O

    gargs = [v for pair in zip(W.box, W.n) for v in pair]
    # Start state: the seeded Gaussian (the FFT/elementwise work per step does
    # not depend on the state).
    phi = W.initial_state(O.Grid(*gargs)) * 10.0
    val, n, t, per = cpu_reference_run(W, phi, cores, args.warmup, args.steps)
    line = {
        "metric": METRIC, "value": val, "unit": UNIT, "impl": "reference", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian start)",
        "config": workload_config(W),
        "step": f"a sample of {per} split steps of solve_split (of the gb300 arm's {W.niter_inner}-step outer "
                f"step); value = grid points x split steps / s",
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.warmup} warm-up and {args.steps} timed samples of {per} split steps "
                                   f"({n} timed) of the {'x'.join(map(str, W.n))} FP64 oracle solve_split "
                                   f"(numpy + scipy.fft, {cores} workers); clock started after the warm-up"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def l2_note(W):
    mb = W.npoints * 12 / 1e6  # complex64 state + float32 potential
    if mb > 129:
        return f"inputs larger than L2 (state + V = {mb:.0f} MB > 129 MB L2)"
    return f"inputs ({mb:.1f} MB) fit in L2: an L2-resident workload, not an HBM measurement"


def imprint(gpe, W, grid, task, phi):
    """The workload's defect on the ground state: a vortex at x0 (2D,
    example1_vortex.m:26-30) or a vortex ring at ring_frac * R_TF (3D)."""
    if W.vortex_x0 is not None:
        return gpe.imprint_vortex(grid, phi, W.g, W.vortex_x0)
    if W.ring_frac is not None:
        r_tf = math.sqrt(2.0 * task.current_mu) / W.trap[0]
        return gpe.imprint_vortex_ring(grid, phi, W.g, W.ring_frac * r_tf)
    return phi


def e2e_abi(task, host_in, host_out, ddt, inner, steps):
    """`steps` outer steps, each through the C ABI with host buffers: the
    state uploaded from host_in, one outer step of `inner` split steps from
    current_iter 0 (gpe_solve_split), the state downloaded into host_out.
    Returns the wall seconds."""
    import ctypes as C

    from gpe_gb300 import _lib as L

    task._push_params()
    ctx = task._ctx
    prm = L.gpe_split_params()
    prm.ddt, prm.niter_inner, prm.niter_outer = float(ddt), int(inner), 1
    cur = L.gpe_current()
    fin = host_in.view(np.float32) if host_in.dtype == np.complex64 else host_in.view(np.float64)
    fout = host_out.view(np.float32) if host_out.dtype == np.complex64 else host_out.view(np.float64)
    set_state = L.lib.gpe_set_state_f32 if host_in.dtype == np.complex64 else L.lib.gpe_set_state
    get_state = L.lib.gpe_get_state_f32 if host_out.dtype == np.complex64 else L.lib.gpe_get_state
    ptr = L.fptr if host_in.dtype == np.complex64 else L.dptr

    def one():
        L.check(ctx, L.lib.gpe_set_current(ctx, C.byref(cur)))   # current_iter = 0
        L.check(ctx, set_state(ctx, ptr(fin)))
        L.check(ctx, L.lib.gpe_solve_split(ctx, C.byref(prm)))
        L.check(ctx, get_state(ctx, ptr(fout)))

    one()  # warm
    t0 = time.perf_counter()
    for _ in range(steps):
        one()
    return time.perf_counter() - t0


def run_gpu(args, dist):
    global INNER
    import gpe_gb300 as gpe
    from gpe_workloads import WORKLOADS

    W = WORKLOADS[args.workload]
    INNER = W.niter_inner
    dev = dist.local
    P = W.npoints
    grid, task, phi = ground_state(gpe, W, "single", device=dev)
    task.set_pass_variant(args.pass_variant)
    if args.plans >= 0:
        task.autotune(args.plans)  # fixed plans (measurement of one variant)
    plans = task.autotune(2)  # the plan per axis the autotuner chose on the first call (-1: one plan)
    itp = task.last_itp
    phi = np.asarray(imprint(gpe, W, grid, task, np.asarray(phi, dtype=np.complex128)))
    # ---- FP32 timed region ------------------------------------------------
    task.init_state = phi
    task.current_iter = 0
    task.solve_split(W.dt, INNER, 1)                  # first warm-up step
    psi32_1 = task.current_state.astype(np.complex128)
    mu32 = task.history["mu"][0]
    task.solve_split(W.dt, INNER, max(1, args.warmup))
    k0 = task.kernel_launches()
    dist.barrier()
    from gpe_gb300 import _lib as L
    import ctypes as C

    # Timed region: no per-launch events (each event record between two
    # kernels adds a gap of its own on the stream).
    with ClockSampler(dev) as clk:
        t0 = time.perf_counter()
        L.check(task._ctx, L.lib.gpe_timer_start(task._ctx))
        task.solve_split(W.dt, INNER, int(task.current_iter) + args.steps)
        ms = C.c_double()
        L.check(task._ctx, L.lib.gpe_timer_stop(task._ctx, C.byref(ms)))
        wall = time.perf_counter() - t0
    launches = task.kernel_launches() - k0
    t_s = dist.reduce(ms.value / 1e3, "max")
    work = dist.reduce(float(P) * INNER * args.steps, "sum")
    value = work / t_s
    # Per-kernel durations: the same steps again with CUDA events around every
    # launch (on the context stream), right after the timed region.
    task.profile(True)
    task.solve_split(W.dt, INNER, int(task.current_iter) + min(args.steps, 2))
    stats = task.profile_read()
    task.profile(False)
    # ---- roofline of the dominant kernel ------------------------------------
    hbm, peak_kind = peaks()
    top = max(stats, key=lambda s: s["total_ms"])
    avg_ms = top["total_ms"] / top["launches"]
    achieved = top["bytes_per_launch"] / (avg_ms / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "pass_traffic_damped3d_256.json"
    if tf.exists() and W.name == "damped3d_256":  # captured on this grid only
        d = json.loads(tf.read_text())
        traffic = d.get(top["name"], {}).get("bytes_per_launch_256cube")
    if args.quick:
        prof_ms = sum(k["total_ms"] for k in stats)
        print(json.dumps({"value": value, "ms_per_step": ms.value / args.steps, "fft_plans_xyz": plans,
                          "profiled_ms_per_step": prof_ms / min(args.steps, 2),
                          "roofline_kernel": top["name"], "frac": achieved / hbm,
                          "kernels": [(k["name"], k["launches"], round(1e3 * k["total_ms"] / k["launches"], 1))
                                      for k in stats]}))
        task.close()
        return
    # ---- FP64 arm (same kernels, same start) ----------------------------------
    g64, t64 = W.make_task("double", device=dev)
    t64.init_state = phi.astype(np.complex128)
    t64.solve_split(W.dt, INNER, 1)
    psi64_1 = t64.current_state
    mu64 = t64.history["mu"][0]
    k64 = max(1, min(args.steps, 3))
    L.check(t64._ctx, L.lib.gpe_timer_start(t64._ctx))
    t64.solve_split(W.dt, INNER, 1 + k64)
    ms64 = C.c_double()
    L.check(t64._ctx, L.lib.gpe_timer_stop(t64._ctx, C.byref(ms64)))
    value64 = float(P) * INNER * k64 / (ms64.value / 1e3)
    err_l2 = float(np.linalg.norm(psi32_1 - psi64_1) / np.linalg.norm(psi64_1))
    # ---- error against the FP64 oracle: one block (10 split steps) from the same
    # start, FP32 and FP64 kernels; the oracle run is also the CPU baseline sample
    cpu, vs_oracle = None, None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu:
        cores = os.cpu_count() or 1
        ostate, omu, on, cval, csteps, ct = oracle_block(W, phi, cores)
        blk = {}
        for name, tk in (("fp32", task), ("fp64", t64)):
            tk.init_state = phi
            tk.current_iter = 0
            tk.solve_split(W.dt, 10, 1)
            st = np.asarray(tk.current_state, dtype=np.complex128)
            blk[name] = {"state_rel_l2": float(np.linalg.norm(st - ostate) / np.linalg.norm(ostate)),
                         "mu_rel": abs(tk.history["mu"][0] - omu) / abs(omu),
                         "n_rel": abs(tk.history["n"][0] - on) / abs(on)}
        vs_oracle = {"horizon": "10 split steps (one n_recalc block) from the imprinted ground state", **blk,
                     "ground_state": "E and mu of the FP32 ITP vs the oracle's converged ITP: tests/test_gpu_configs.py "
                                     "(1e-13 / 2e-11 relative on this grid)"}
        cpu = {"value": cval, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{csteps} split steps of the same {'x'.join(map(str, W.n))} workload in the FP64 "
                         f"oracle (numpy + scipy.fft with {cores} workers), {ct:.1f} s, after one untimed step and "
                         f"the setup, the block-end mu included"}
    t64.close()
    # ---- e2e through the public API with pinned host buffers --------------------
    host_in = np.ascontiguousarray(phi.astype(np.complex64))
    host_out = np.empty_like(host_in)
    e2e_steps = max(1, min(args.steps, 5))
    with gpe.pinned(host_in), gpe.pinned(host_out):
        e2e_t = e2e_abi(task, host_in, host_out, W.dt, INNER, e2e_steps)
    e2e_t = dist.reduce(e2e_t, "max")
    e2e_val = dist.reduce(float(P) * INNER * e2e_steps, "sum") / e2e_t
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms.value / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 (FP64 reductions)", "data": "synthetic (seeded Gaussian -> ITP ground state)",
        "config": workload_config(W),
        "step": f"{INNER} split steps (1 outer step of solve_split)",
        "fft_plans_xyz": {"chosen_by": ("autotuner" if args.plans < 0 else f"fixed (gpe_autotune mode {args.plans})")
                          + " (0 default plan, 1 alternative, 2 / 3 paired passes on the alternative / default plan,"
                          " -1 single plan)",
                          "x": plans[0], "y": plans[1], "z": plans[2]},
        "parallelism": f"replicas x{dist.world}" if dist.world > 1 else "1 GPU",
        "fp64": {"value": value64, "unit": UNIT, "steps": INNER * k64, "ratio_fp32_over_fp64": value / dist.world / value64},
        "error": {"fp32_vs_fp64_rel_l2_after_outer_step": err_l2,
                  "mu_rel_after_outer_step": abs(mu32 - mu64) / abs(mu64),
                  "itp_iters": itp.iters, "itp_fp32_iters": itp.fp32_iters, "itp_converged": bool(itp.converged),
                  "itp_ms_fp32": itp.ms_main, "itp_ms_fp64_polish": itp.ms_fp64,
                  "vs_oracle": vs_oracle},
        "roofline": {"bound": "hbm", "kernel": top["name"], "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": top["bytes_per_launch"], "avg_launch_ms": avg_ms,
                     "timing": "CUDA events around every launch on the context stream, in a profiled "
                               "window of the same work right after the timed region"},
        "kernels": stats,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(host_in.nbytes),
                "d2h_bytes_per_step": int(host_out.nbytes), "steps": e2e_steps},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "wall_s_timed": wall,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if W.npoints * 12 / 1e6 <= 129:  # L2-resident: the arithmetic roofline
        cl = line["clocks"] if isinstance(line["clocks"], dict) else {}
        line["flop_roofline"] = flop_roofline([P], INNER * args.steps, t_s, cl.get("sm_max_mhz"),
                                              sms_used=16 if top["name"] == "cluster_step" else None)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    task.close()


def run_batch(args, dist):
    """The batched workload: 64 uneven 2D grids advanced by solve_split_batch
    (CUDA graph per block, grids' chains concurrent); device-timed with the
    first task's CUDA events."""
    import ctypes as C

    import gpe_gb300 as gpe
    from gpe_gb300 import _lib as L
    from gpe_workloads import BATCH2D as B

    tasks = B.make_tasks("single", device=dist.local, rank=dist.rank, world=dist.world)  # realisations sharded
    P = sum(t.grid.npoints for t in tasks)
    inner = B.niter_inner
    gpe.solve_split_batch(tasks, B.dt, inner, args.warmup)
    k0 = sum(t.kernel_launches() for t in tasks)
    dist.barrier()
    t0c = tasks[0]._ctx
    with ClockSampler(dist.local) as clk:
        L.check(t0c, L.lib.gpe_timer_start(t0c))
        gpe.solve_split_batch(tasks, B.dt, inner, args.warmup + args.steps)
        ms = C.c_double()
        L.check(t0c, L.lib.gpe_timer_stop(t0c, C.byref(ms)))
    launches = sum(t.kernel_launches() for t in tasks) - k0
    t_s = dist.reduce(ms.value / 1e3, "max")
    value = dist.reduce(float(P) * inner * args.steps, "sum") / t_s
    sizes = {}
    for t in tasks:
        sizes[t.grid.nx] = sizes.get(t.grid.nx, 0) + 1
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms.value / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 (FP64 reductions)", "data": "synthetic (seeded realisations -> ITP)",
        "config": {"workload": B.name, "realisations": B.count, "realisations_per_rank": len(tasks),
                   "sharding": "realisations dealt round-robin over ranks, no data-path collective",
                   "sizes_rank0": {f"{k}^2": v for k, v in sorted(sizes.items())},
                   "points_total": P, "dt": B.dt, "step": f"{inner} split steps of every realisation",
                   "execution": "one CUDA graph per outer step: per shape of grid a stream of pass kernels over "
                                "the tiles of all its grids (folded steps: 11 pass launches, 2 kinetic-sum "
                                "launches and 1 finalizer per block of 10 steps)",
                   "l2": f"all states ({P * 12 / 1e6:.0f} MB with V) fit in L2: L2-resident workload"},
        "gpu_launches": int(launches), "clocks": clk.summary(),
    }
    cl = line["clocks"] if isinstance(line["clocks"], dict) else {}
    line["flop_roofline"] = flop_roofline([t.grid.npoints for t in tasks], inner * args.steps, t_s,
                                          cl.get("sm_max_mhz"))
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    for t in tasks:
        t.close()


ADJ_METRIC = "adjoint grid-pt-steps/s (loss + dloss/dV through the window, per second)"


def adjoint_case(gpe, name, dev):
    """(task, psi0, target, V, nsteps, checkpoint_every, basis, describe) of an adjoint workload."""
    if name == "adjoint2d_256":
        from gpe_workloads import ADJOINT2D as W

        grid = W.make_grid("single")
        task = gpe.GPEtask(grid, lambda X, Y, Z: W.trap(grid), device=dev)
        task.Ntotal, task.g = W.Ntotal, W.g
        X, Y = grid.mesh["x"], grid.mesh["y"]
        psi0 = np.asarray(task.groundstate_itp(W.itp_dt, W.itp_eps, np.exp(-(X ** 2 + Y ** 2) / 32).astype(complex)),
                          dtype=np.complex128)
        tgt = gpe.imprint_vortex(grid, psi0, W.g, W.vortex_x0)
        a, basis = W.bumps(grid)
        V = W.trap(grid) + sum(aj * b for aj, b in zip(a, basis))
        cfg = {"workload": W.name, "grid": [W.n, W.n], "box": W.box, "g": W.g, "Ntotal": W.Ntotal, "dt": W.dt,
               "window_steps": W.steps, "checkpoint_every": W.checkpoint_every,
               "potential": "0.5 r^2 + 16 seeded Gaussian bumps", "target": f"vortex imprinted at x0 = {W.vortex_x0}"}
        return task, psi0, tgt, V, W.steps, W.checkpoint_every, basis, cfg
    from gpe_workloads import RING3D as W

    grid, task, phi = ground_state(gpe, W, "single", device=dev)
    psi0 = np.asarray(imprint(gpe, W, grid, task, np.asarray(phi, dtype=np.complex128)))
    tgt = np.asarray(phi, dtype=np.complex128)
    V = np.ascontiguousarray(task.Vtrap)
    cfg = {"workload": "adjoint3d_512", "grid": list(W.n), "box": W.box[0], "trap_lambda": list(W.trap), "g": W.g,
           "Ntotal": W.Ntotal, "dt": W.dt, "window_steps": 500, "checkpoint_every": "auto (sqrt rule)",
           "mem_budget_GB": 60, "start": "vortex ring (0.5 R_TF) on the ITP ground state",
           "target": "the ground state without the ring"}
    return task, psi0, tgt, V, 500, 0, None, cfg


def run_adjoint(args, dist):
    """Gradient workloads: one bench step = one gpe_adjoint_grad call (forward
    window with checkpoints, loss, backward sweep with segment recompute),
    device-timed with CUDA events on the context stream."""
    import ctypes as C

    import gpe_gb300 as gpe
    from gpe_gb300 import _lib as L

    dev = dist.local
    task, psi0, tgt, V, M, K, basis, cfg = adjoint_case(gpe, args.workload, dev)
    P = task.grid.npoints
    budget = 60e9
    precision = "double" if args.adjoint_fp64 else None
    kw = dict(phi0=psi0, V=V, checkpoint_every=K, mem_budget=budget, precision=precision)
    for _ in range(1 if P > 1e7 else args.warmup):
        task.adjoint_grad(tgt, cfg["dt"], M, **kw)
    steps = min(args.steps, 2) if P > 1e7 else args.steps
    task._upload_state(psi0)  # the timed calls run on a device-resident start state
    k0 = task.kernel_launches()
    dist.barrier()
    with ClockSampler(dev) as clk:
        L.check(task._ctx, L.lib.gpe_timer_start(task._ctx))
        for _ in range(steps):
            loss, dV = task.adjoint_grad(tgt, cfg["dt"], M, **kw)
        ms = C.c_double()
        L.check(task._ctx, L.lib.gpe_timer_stop(task._ctx, C.byref(ms)))
    launches = task.kernel_launches() - k0
    # per-kernel durations from one more call with events around every launch
    task.profile(True)
    task.adjoint_grad(tgt, cfg["dt"], M, **kw)
    stats = task.profile_read()
    task.profile(False)
    t_s = dist.reduce(ms.value / 1e3, "max")
    value = dist.reduce(float(P) * M * steps, "sum") / t_s
    hbm, peak_kind = peaks()
    top = max(stats, key=lambda s: s["total_ms"])
    avg_ms = top["total_ms"] / top["launches"]
    achieved = top["bytes_per_launch"] / (avg_ms / 1e3) / 1e9
    line = {
        "metric": ADJ_METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": ms.value / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if precision else "c64 (FP64 dL/dV accumulation)",
        "data": "synthetic (seeded, ITP ground state)", "config": cfg, "loss": loss,
        "grad_norm": float(np.linalg.norm(dV)),
        "roofline": {"bound": "hbm", "kernel": top["name"], "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": None,
                     "algorithmic_bytes_per_launch": top["bytes_per_launch"], "avg_launch_ms": avg_ms,
                     "timing": "CUDA events around every launch on the context stream, in a profiled "
                               "window of the same work right after the timed region"},
        "kernels": stats, "gpu_launches": int(launches), "clocks": clk.summary(),
    }
    if basis is not None:
        line["dloss_da"] = [float(v) for v in task.project_gradient(dV, basis)]
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu and basis is not None:
        from oracle import gpe_oracle as O

        O.set_workers(os.cpu_count() or 1)
        og = O.Grid(cfg["box"], cfg["grid"][0], cfg["box"], cfg["grid"][1])
        n_cpu = 200
        t0 = time.perf_counter()
        O.adjoint_grad(og, V, task.g, psi0, tgt, cfg["dt"], n_cpu)
        tc = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": P * n_cpu / tc, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"FP64 oracle adjoint over {n_cpu} steps of the same grid, {tc:.1f} s"}
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    task.close()


SPIN_METRIC = "spinor split-step grid-pt-steps/s (2 coupled components, complex FP32)"


def spinor_cpu_steps(S, pair, cores: int, blocks: int = 1):
    """`blocks` outer steps of 10 split steps (one n_recalc block each) of the
    FP64 oracle's GPEtaskSpinor.solve_split on the workload grid, timed after
    one untimed block (so the setup, kinetic tables and the applyham before
    the loop, is outside the clock): (grid-pt-steps/s, steps, s).  Built from
    the oracle and the library-free workload tables only."""
    from oracle import gpe_oracle as O

    O.set_workers(cores)
    og = O.Grid(S.box, S.n[0], S.box, S.n[1], S.box, S.n[2])
    ot = O.GPEtaskSpinor(og, S.potentials())
    S.configure(ot)
    ot.init_state = [np.asarray(p, dtype=np.complex128) for p in pair]
    stamps = []

    class Done(Exception):
        pass

    def on_outer(_task):
        stamps.append(time.perf_counter())
        if len(stamps) > blocks:
            raise Done

    ot.user_callback = on_outer
    try:
        ot.solve_split(S.dt, 10, 10 ** 6)
    except Done:
        pass
    t = stamps[-1] - stamps[0]
    return S.npoints * 10 * blocks / t, 10 * blocks, t


def spinor_config(S):
    """The spinor workload's description, identical in both arms."""
    return {"workload": S.name, "grid": list(S.n), "components": 2, "box": S.box, "g": [list(r) for r in S.g],
            "coupling": str(S.coupling), "Ntotal": S.Ntotal, "gamma": S.gamma, "dt": S.dt, "n_recalc": 10,
            "l2": f"inputs larger than L2 (2 states + 2 V = {S.npoints * 24 / 1e6:.0f} MB > 129 MB L2)",
            "points_counted": "grid points (each carries both components)"}


def spinor_start(gpe, dev):
    """The damped workload's ITP ground state (untimed), split into the pair."""
    from gpe_workloads import DAMPED3D as W, SPINOR3D as S

    _, t1, phi = ground_state(gpe, W, "single", device=dev)
    phi = np.asarray(phi, dtype=np.complex128)
    t1.close()
    return S, S.initial_pair(phi)


def run_spinor(args, dist):
    """The two-component workload: one bench step = one outer step (100 split
    steps) of GPEtaskSpinor.solve_split, device-timed with CUDA events."""
    import ctypes as C

    import gpe_gb300 as gpe
    from gpe_gb300 import _lib as L

    dev = dist.local
    S, pair = spinor_start(gpe, dev)
    P = S.npoints
    inner = S.niter_inner
    _, task = S.make_task("single", device=dev)
    task.init_state = pair
    task.solve_split(S.dt, inner, 1)
    psi32_1 = [x.astype(np.complex128) for x in task.current_state]
    mu32 = task.history["mu"][0]
    task.solve_split(S.dt, inner, max(1, args.warmup))
    k0 = task.kernel_launches()
    dist.barrier()
    with ClockSampler(dev) as clk:
        L.check(task._ctx, L.lib.gpe_timer_start(task._ctx))
        task.solve_split(S.dt, inner, int(task.current_iter) + args.steps)
        ms = C.c_double()
        L.check(task._ctx, L.lib.gpe_timer_stop(task._ctx, C.byref(ms)))
    launches = task.kernel_launches() - k0
    t_s = dist.reduce(ms.value / 1e3, "max")
    value = dist.reduce(float(P) * inner * args.steps, "sum") / t_s
    task.profile(True)
    task.solve_split(S.dt, inner, int(task.current_iter) + min(args.steps, 2))
    stats = task.profile_read()
    task.profile(False)
    hbm, peak_kind = peaks()
    top = max(stats, key=lambda s: s["total_ms"])
    avg_ms = top["total_ms"] / top["launches"]
    achieved = top["bytes_per_launch"] / (avg_ms / 1e3) / 1e9
    # FP64 arm on the same start
    _, t64 = S.make_task("double", device=dev)
    t64.init_state = pair
    t64.solve_split(S.dt, inner, 1)
    psi64_1 = t64.current_state
    mu64 = t64.history["mu"][0]
    L.check(t64._ctx, L.lib.gpe_timer_start(t64._ctx))
    t64.solve_split(S.dt, inner, 2)
    ms64 = C.c_double()
    L.check(t64._ctx, L.lib.gpe_timer_stop(t64._ctx, C.byref(ms64)))
    value64 = float(P) * inner / (ms64.value / 1e3)
    t64.close()
    a = np.concatenate([x.ravel() for x in psi32_1])
    b = np.concatenate([x.ravel() for x in psi64_1])
    err_l2 = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    # e2e: both components from and to pinned host buffers through the public API
    host_in = np.ascontiguousarray(np.concatenate([p.ravel() for p in pair]).astype(np.complex64))
    host_out = np.empty_like(host_in)
    e2e_steps = max(1, min(args.steps, 3))
    with gpe.pinned(host_in), gpe.pinned(host_out):
        e2e_t = e2e_abi(task, host_in, host_out, S.dt, inner, e2e_steps)
    e2e_t = dist.reduce(e2e_t, "max")
    e2e_val = dist.reduce(float(P) * inner * e2e_steps, "sum") / e2e_t
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu:
        cores = os.cpu_count() or 1
        cval, n, t = spinor_cpu_steps(S, pair, cores)
        cpu = {"value": cval, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{n} split steps (one block) of the same 256^3 two-component workload in the FP64 "
                         f"oracle (numpy + scipy.fft with {cores} workers), {t:.1f} s, after one untimed block"}
    line = {
        "metric": SPIN_METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms.value / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 (FP64 reductions)",
        "data": "synthetic (ITP ground state of the damped workload split 70/30)",
        "config": spinor_config(S), "step": f"{inner} split steps (1 outer step)",
        "fp64": {"value": value64, "unit": UNIT, "steps": inner, "ratio_fp32_over_fp64": value / dist.world / value64},
        "error": {"fp32_vs_fp64_rel_l2_after_outer_step": err_l2, "mu_rel_after_outer_step": abs(mu32 - mu64) / abs(mu64)},
        "roofline": {"bound": "hbm", "kernel": top["name"], "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": None,
                     "algorithmic_bytes_per_launch": top["bytes_per_launch"], "avg_launch_ms": avg_ms,
                     "timing": "CUDA events around every launch on the context stream, in a profiled "
                               "window of the same work right after the timed region"},
        "kernels": stats,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(host_in.nbytes),
                "d2h_bytes_per_step": int(host_out.nbytes), "steps": e2e_steps},
        "gpu_launches": int(launches), "clocks": clk.summary(),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    task.close()


def run_spinor_reference(args, dist):
    """--impl reference for the spinor workload: the FP64 oracle restatement of
    GPEtaskSpinor.solve_split on the host cores (the start state is the
    seeded Gaussian pair; the timed work does not depend on it)."""
    from gpe_workloads import DAMPED3D as W, SPINOR3D as S

    if dist.rank != 0:
        return
    from oracle import gpe_oracle as O

    cores = os.cpu_count() or 1
    grid = O.Grid(W.box[0], W.n[0], W.box[1], W.n[1], W.box[2], W.n[2])
    pair = S.initial_pair(W.initial_state(grid) * 10.0)
    blocks = max(1, min(args.steps, 2))
    v, n, t = spinor_cpu_steps(S, pair, cores, blocks)
    line = {
        "metric": SPIN_METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": 1, "steps": blocks,
        "warmup": 1, "ms_per_step": 1e3 * t / blocks, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": spinor_config(S), "step": "one block of 10 split steps (n_recalc 10)",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{blocks} x 10 split steps of the 256^3 two-component FP64 oracle after one "
                                   f"untimed block"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_profile_case(precision: str, blocks: int, variant: int = 0, plans: int = 0, workload: str = "damped3d_256"):
    """Small fixed case for ncu captures: a workload's grid and parameters from
    its seeded Gaussian start (no ITP), `blocks` blocks of 10 steps (3D: one
    outer step of 10 per block; 2D: outer steps of the workload's niter_inner,
    the cluster kernel's launch unit).  The FFT plans of 3D grids are fixed
    (no autotuning under the profiler): `plans` = bit mask of the axes (bit 0
    = x) that use the alternative plan.  batch2d_64: the batch's grids from
    their seeded Gaussian starts, `blocks` outer steps of 100."""
    import gpe_gb300 as gpe
    from gpe_workloads import BATCH2D, WORKLOADS

    if workload == "batch2d_64":
        import numpy as np

        tasks = []
        for r in BATCH2D.realisations():
            grid = gpe.grid2d(BATCH2D.box, r["n"], BATCH2D.box, r["n"], precision=precision)
            t = gpe.GPEtask(grid, lambda X, Y, Z, lam=r["lam"]: 0.5 * (X ** 2 + (lam * Y) ** 2))
            t.Ntotal, t.g = BATCH2D.Ntotal, r["g"]
            X, Y = grid.mesh["x"], grid.mesh["y"]
            t.init_state = np.exp(-(X ** 2 + (r["lam"] * Y) ** 2) / 32.0).astype(complex)
            tasks.append(t)
        gpe.solve_split_batch(tasks, BATCH2D.dt, BATCH2D.niter_inner, blocks)
        print(json.dumps({"profile_case": precision, "workload": workload, "outer_steps": blocks,
                          "launches": sum(t.kernel_launches() for t in tasks)}))
        for t in tasks:
            t.close()
        return
    W = WORKLOADS[workload]
    grid, task = W.make_task(precision)
    if W.ndims == 3:
        task.autotune(plans if plans >= 32 else 16 + plans)  # 32 / 48 + mask: paired passes
    task.set_pass_variant(variant)
    task.init_state = W.initial_state(grid) * 30.0
    if W.ndims == 3:
        task.solve_split(W.dt, 10, blocks)
    else:
        task.solve_split(W.dt, W.niter_inner, blocks)
    print(json.dumps({"profile_case": precision, "workload": workload, "blocks": blocks,
                      "launches": task.kernel_launches(), "mu": task.current_mu, "n": task.current_n}))
    task.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile-case", choices=["single", "double"], default=None,
                    help="run the small fixed case used for ncu captures and exit")
    ap.add_argument("--profile-blocks", type=int, default=2)
    ap.add_argument("--profile-workload", default="damped3d_256",
                    choices=["damped3d_256", "ring3d_512", "vortex2d_256", "batch2d_64"],
                    help="profile case: the workload whose grid and parameters it runs")
    ap.add_argument("--profile-plans", type=int, default=0,
                    help="profile case: bit mask of axes (bit 0 = x) on the alternative FFT plan; "
                         "32 / 48 + mask: the paired passes on the alternative / default plan on those axes")
    ap.add_argument("--plans", type=int, default=-1,
                    help="FFT plans of the timed context: -1 the autotuner's choice (default), else a gpe_autotune "
                         "mode (0 default plans, 3 alternative, 4/5 paired on alternative/default, 16/32/48 + axis mask)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--quick", action="store_true", help="FP32 timed region only (no FP64, e2e, CPU legs)")
    ap.add_argument("--pass-variant", type=int, default=0, help="0: direct + L2 prefetch (default), 1: TMA-staged, 2: direct")
    ap.add_argument("--workload", default="damped3d_256",
                    choices=["damped3d_256", "ring3d_512", "vortex2d_256", "batch2d_64", "adjoint2d_256",
                             "adjoint3d_512", "spinor3d_256"],
                    help="damped3d_256 (default, the headline), ring3d_512, vortex2d_256 (L2-resident), "
                         "batch2d_64 (64 uneven grids), adjoint2d_256 / adjoint3d_512 (gradients), "
                         "spinor3d_256 (two coupled components)")
    ap.add_argument("--adjoint-fp64", action="store_true", help="adjoint workloads: FP64 sweep of the FP32 context")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args.profile_case, args.profile_blocks, args.pass_variant, args.profile_plans,
                         args.profile_workload)
        return
    if args.warmup < 3:
        args.warmup = 3
    dist = Dist()
    try:
        if args.impl == "reference":
            if args.workload == "spinor3d_256":
                run_spinor_reference(args, dist)
            else:
                run_reference(args, dist)
        else:
            if args.workload == "spinor3d_256":
                run_spinor(args, dist)
            elif args.workload == "batch2d_64":
                run_batch(args, dist)
            elif args.workload.startswith("adjoint"):
                run_adjoint(args, dist)
            else:
                run_gpu(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
