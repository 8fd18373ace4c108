"""Build libgpe.so (sm_103a) in-tree with nvcc.

Every translation unit under csrc/ is compiled in parallel, then linked into
``gpe-matlab_gb300/libgpe.so`` (CUDA runtime linked statically, so the
library needs only the driver at run time).  Object files go to
``gpe-matlab_gb300/_build/``.  Rebuilds only what changed (by mtime, headers
included).

    python gpe-matlab_gb300/build_lib.py [--force] [--jobs N] [--verbose]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libgpe.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
           "--expt-relaxed-constexpr", "-I", str(CSRC), "-I", str(INCLUDE)]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgpe")


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


EXTRA: list = []


def _compile(src: Path, force: bool, verbose: bool) -> Path:
    obj = BUILD / (src.stem + ".o")
    if not force and obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, _headers_mtime()):
        return obj
    cmd = [nvcc(), *ARCH, *NVFLAGS, *EXTRA, "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr)
    return obj


def build(force: bool = False, jobs: int | None = None, verbose: bool = False, out: Path | None = None,
          build_dir: Path | None = None, defines: list | None = None) -> Path:
    """Compile and link; `out`/`build_dir`/`defines` (-D macros) select a variant build."""
    global BUILD, LIB, EXTRA
    if out is not None:
        LIB = Path(out)
    if build_dir is not None:
        BUILD = Path(build_dir)
    EXTRA = [f"-D{d}" for d in (defines or [])]
    BUILD.mkdir(parents=True, exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, verbose), srcs))
    if force or not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", str(LIB), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--out", default=None, help="output library path (default: gpe-matlab_gb300/libgpe.so)")
    ap.add_argument("--build-dir", default=None)
    ap.add_argument("-D", dest="defines", action="append", default=[], help="preprocessor define NAME=VALUE")
    a = ap.parse_args()
    p = build(a.force, a.jobs, a.verbose, a.out, a.build_dir, a.defines)
    print(p)
    sys.exit(0)
