"""The bench's reference arm (`bench.py --impl reference`) on CPU: the FP64
oracle restatement of solve_split timed on the host cores, printed as one JSON
line with the gb300 arm's metric and unit, a cpu_baseline of kind "port" and
an e2e object without host-device bytes, and the same `config` dict as the
gb300 arm; it never loads libgpe.so (the library path is pointed at a file
that does not exist, so any load would fail the run); workloads without a
reference path print an `unavailable` line and exit 0."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def run_bench(*args):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", GPE_LIB=str(ROOT / "no-such-libgpe.so"))
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", *args], cwd=ROOT,
                       capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def test_reference_arm_json_line():
    d = run_bench("--workload", "vortex2d_256", "--steps", "2", "--warmup", "3")
    assert d["impl"] == "reference"
    assert d["metric"].startswith("split-step grid-pt-steps/s") and d["unit"] == "grid-pt-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["config"]["workload"] == "vortex2d_256" and d["config"]["grid"] == [256, 256]
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "gpe-matlab_gb300"))
    import bench
    from gpe_workloads import VORTEX2D

    assert d["config"] == json.loads(json.dumps(bench.workload_config(VORTEX2D)))
    assert "split steps" in d["step"]
    assert d["ms_per_step"] * d["steps"] < 600e3
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_unavailable_for_the_batch():
    d = run_bench("--workload", "batch2d_64", "--steps", "1", "--warmup", "3")
    assert d["impl"] == "reference" and "unavailable" in d
