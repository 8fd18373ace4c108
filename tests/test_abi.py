"""The C ABI boundary without a GPU: libgpe.so loads, exports exactly what
include/gpe.h declares, the ctypes mirror matches the C struct layouts, and
calls fail cleanly (status + message, no crash) when no GB300 is present."""
import ctypes as C
import json
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "gpe.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"GPE_API\s+(?:const\s+)?\w+(?:\s+\w+)?\s*\**\s*(gpe_\w+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("gpe_create", "gpe_destroy", "gpe_set_potential", "gpe_set_state", "gpe_get_state",
                 "gpe_groundstate_itp", "gpe_solve_split", "gpe_observables", "gpe_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from gpe_gb300 import _lib as L

    names = declared_functions()
    missing = [n for n in names if not hasattr(L.lib, n)]
    assert not missing, missing
    assert set(names) == set(L.PROTOTYPES), "ctypes prototypes must cover the header exactly"
    nm = shutil.which("nm")
    if nm:
        out = subprocess.run([nm, "-D", "--defined-only", str(L.LIB_PATH)], capture_output=True, text=True).stdout
        exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
        gpe_exports = {e for e in exported if e.startswith("gpe_")}
        assert gpe_exports == set(names), gpe_exports ^ set(names)


def test_struct_layouts_match_ctypes(tmp_path):
    from gpe_gb300 import _lib as L

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = tmp_path / "abi_layout"
    subprocess.run([cc, "-std=c99", "-I", str(ROOT / "include"), str(ROOT / "tests" / "abi_layout.c"), "-o",
                    str(exe)], check=True)
    lay = json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    for key, val in lay.items():
        if key == "end":
            continue
        if "." in key:
            s, f = key.split(".")
            assert getattr(getattr(L, s), f).offset == val, key
        else:
            assert C.sizeof(getattr(L, key)) == val, key


def test_abi_version_and_defaults():
    from gpe_gb300 import _lib as L

    assert L.lib.gpe_abi_version() == 1
    p = L.gpe_params()
    L.lib.gpe_default_params(C.byref(p))
    assert (p.n_recalc, p.itp_max_iter, p.itp_min_iter, p.itp_adjust_stepsize) == (10, 5000, 50, 0)
    assert p.g == 0 and p.gamma == 0 and p.Ntotal == 0


def test_invalid_arguments_are_rejected_before_any_device_work():
    from gpe_gb300 import _lib as L

    ctx = C.c_void_p()
    d = L.gpe_grid_desc()
    d.ndims = 4
    assert L.lib.gpe_create(C.byref(d), C.byref(ctx)) == L.GPE_ERR_INVALID
    assert b"ndims" in L.lib.gpe_last_error(None)
    d.ndims = 2
    d.n[0], d.n[1] = 100, 64          # 100 = 2^2 5^2 has no plan
    d.dx[0] = d.dx[1] = 0.1
    d.precision = L.GPE_FP32
    assert L.lib.gpe_create(C.byref(d), C.byref(ctx)) == L.GPE_ERR_UNSUPPORTED
    assert b"no FFT plan" in L.lib.gpe_last_error(None)
    d.n[0] = 64
    d.precision = 7
    assert L.lib.gpe_create(C.byref(d), C.byref(ctx)) == L.GPE_ERR_INVALID
    assert L.lib.gpe_create(None, C.byref(ctx)) == L.GPE_ERR_INVALID
    # null context handles fail cleanly
    assert L.lib.gpe_solve_split(None, None) == L.GPE_ERR_INVALID
    assert L.lib.gpe_kernel_launches(None) == 0


def test_no_gpu_reports_no_device():
    from gpe_gb300 import _lib as L

    if L.lib.gpe_device_available():
        pytest.skip("a GB300 is present")
    ctx = C.c_void_p()
    d = L.gpe_grid_desc()
    d.ndims = 2
    d.n[0] = d.n[1] = 64
    d.dx[0] = d.dx[1] = 0.1
    d.span[0] = d.span[1] = 6.3
    d.precision = L.GPE_FP32
    assert L.lib.gpe_create(C.byref(d), C.byref(ctx)) == L.GPE_ERR_NO_DEVICE
    assert not ctx.value


def test_mex_gateway_compiles_against_the_documented_api():
    """matlab/gpe_mex.cpp cannot be built without MATLAB; this compiles it
    (syntax and types) against declarations of the documented MEX C API and
    include/gpe.h, so a call that no longer matches the C ABI fails here."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    src = ROOT / "gpe-matlab_gb300" / "matlab" / "gpe_mex.cpp"
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-Wall", "-I", str(ROOT / "tests" / "mex_stub"),
                        "-I", str(ROOT / "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_norm_noalloc_refuses_a_misaligned_pointer_before_any_cuda_call():
    """The alignment check of gpe_norm_noalloc runs before any CUDA call, so
    it answers without a GPU: a pointer off the 16-byte boundary of a complex
    double (or the 8-byte one of a complex float) is GPE_ERR_INVALID."""
    from gpe_gb300 import _lib as L

    out = C.c_double(-1.0)
    for addr, prec in ((0x10008, L.GPE_FP64), (0x10004, L.GPE_FP32), (0x10001, L.GPE_FP64)):
        st = L.lib.gpe_norm_noalloc(C.c_void_p(addr), 1024, prec, 1.0, None, C.byref(out))
        assert st == L.GPE_ERR_INVALID
        assert b"aligned" in L.lib.gpe_last_error(None)
    assert out.value == -1.0
