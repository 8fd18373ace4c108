"""ctypes binding of libgpe.so (include/gpe.h).

The library is the product: this module only declares its C ABI.  There is
no fallback: if ``libgpe.so`` is missing or fails to load, importing the
package raises, naming the build command.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("GPE_LIB", _HERE.parent / "libgpe.so"))

GPE_OK, GPE_ERR_INVALID, GPE_ERR_UNSUPPORTED, GPE_ERR_CUDA, GPE_ERR_ALLOC = 0, 1, 2, 3, 4
GPE_ERR_STATE, GPE_ERR_TIMEOUT, GPE_ERR_NONFINITE, GPE_ERR_NO_DEVICE, GPE_ERR_CALLBACK = 5, 6, 7, 8, 9
GPE_ERR_BOUNDS = 10
GPE_FP32, GPE_FP64 = 1, 2

STATUS_NAMES = {0: "GPE_OK", 1: "GPE_ERR_INVALID", 2: "GPE_ERR_UNSUPPORTED", 3: "GPE_ERR_CUDA",
                4: "GPE_ERR_ALLOC", 5: "GPE_ERR_STATE", 6: "GPE_ERR_TIMEOUT", 7: "GPE_ERR_NONFINITE",
                8: "GPE_ERR_NO_DEVICE", 9: "GPE_ERR_CALLBACK", 10: "GPE_ERR_BOUNDS"}


class gpe_grid_desc(C.Structure):
    _fields_ = [("ndims", C.c_int), ("n", C.c_int * 3), ("dx", C.c_double * 3), ("span", C.c_double * 3),
                ("precision", C.c_int), ("device", C.c_int)]


class gpe_params(C.Structure):
    _fields_ = [("g", C.c_double), ("gamma", C.c_double), ("decay_rate", C.c_double), ("Ntotal", C.c_double),
                ("mu_init", C.c_double), ("n_recalc", C.c_int), ("itp_max_iter", C.c_int),
                ("itp_min_iter", C.c_int), ("itp_adjust_stepsize", C.c_int), ("omega", C.c_double)]


class gpe_itp_params(C.Structure):
    _fields_ = [("dt", C.c_double), ("eps", C.c_double), ("want_mu2", C.c_int), ("want_energy", C.c_int),
                ("fp64_polish", C.c_int), ("switch_delta", C.c_double)]


class gpe_itp_result(C.Structure):
    _fields_ = [("iters", C.c_int), ("converged", C.c_int), ("fp32_iters", C.c_int), ("final_dt", C.c_double),
                ("last_delta", C.c_double), ("ms_main", C.c_double), ("ms_fp64", C.c_double)]


VTD_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_double, C.POINTER(C.c_double))
STEP_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double)


class gpe_split_params(C.Structure):
    _fields_ = [("ddt", C.c_double), ("niter_inner", C.c_int), ("niter_outer", C.c_int), ("vtd", VTD_FN),
                ("vtd_user", C.c_void_p), ("on_step", STEP_FN), ("step_user", C.c_void_p)]


class gpe_adjoint_params(C.Structure):
    _fields_ = [("ddt", C.c_double), ("nsteps", C.c_int), ("checkpoint_every", C.c_int),
                ("mem_budget", C.c_double), ("precision", C.c_int)]


class gpe_sgpe_params(C.Structure):
    _fields_ = [("T", C.c_double), ("ecut", C.c_double), ("seed", C.c_ulonglong)]


class gpe_current(C.Structure):
    _fields_ = [("current_iter", C.c_int), ("current_time", C.c_double), ("current_mu", C.c_double),
                ("current_n", C.c_double)]


class gpe_obs(C.Structure):
    _fields_ = [("norm", C.c_double), ("ekin", C.c_double), ("epot", C.c_double), ("eint", C.c_double),
                ("mu_integral", C.c_double), ("energy", C.c_double), ("ecpl", C.c_double)]


class gpe_spinor_params(C.Structure):
    _fields_ = [("g", C.c_double * 4), ("coupling_re", C.c_double), ("coupling_im", C.c_double),
                ("nlincpl", C.c_double)]


class gpe_kernel_stat(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_longlong), ("total_ms", C.c_double),
                ("bytes_per_launch", C.c_double)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)

# name -> (restype, argtypes); exactly the functions include/gpe.h declares.
PROTOTYPES = {
    "gpe_create": (C.c_int, [C.POINTER(gpe_grid_desc), C.POINTER(_P)]),
    "gpe_create_spinor": (C.c_int, [C.POINTER(gpe_grid_desc), C.POINTER(_P)]),
    "gpe_set_omega_field": (C.c_int, [_P, _D, C.c_int]),
    "gpe_set_spinor_params": (C.c_int, [_P, C.POINTER(gpe_spinor_params)]),
    "gpe_get_spinor_params": (C.c_int, [_P, C.POINTER(gpe_spinor_params)]),
    "gpe_destroy": (None, [_P]),
    "gpe_last_error": (C.c_char_p, [_P]),
    "gpe_abi_version": (C.c_int, []),
    "gpe_device_available": (C.c_int, []),
    "gpe_default_params": (None, [C.POINTER(gpe_params)]),
    "gpe_set_params": (C.c_int, [_P, C.POINTER(gpe_params)]),
    "gpe_get_params": (C.c_int, [_P, C.POINTER(gpe_params)]),
    "gpe_get_current": (C.c_int, [_P, C.POINTER(gpe_current)]),
    "gpe_set_current": (C.c_int, [_P, C.POINTER(gpe_current)]),
    "gpe_get_history": (C.c_int, [_P, _D, _D, C.c_int, C.POINTER(C.c_int)]),
    "gpe_get_history_energy": (C.c_int, [_P, _D, C.c_int, C.POINTER(C.c_int)]),
    "gpe_clear_history": (C.c_int, [_P]),
    "gpe_set_potential": (C.c_int, [_P, _D]),
    "gpe_set_potential_f32": (C.c_int, [_P, _F]),
    "gpe_set_state": (C.c_int, [_P, _D]),
    "gpe_set_state_f32": (C.c_int, [_P, _F]),
    "gpe_get_state": (C.c_int, [_P, _D]),
    "gpe_get_state_f32": (C.c_int, [_P, _F]),
    "gpe_set_state_device": (C.c_int, [_P, _P, C.c_int]),
    "gpe_get_state_device": (C.c_int, [_P, _P, C.c_int]),
    "gpe_groundstate_itp": (C.c_int, [_P, C.POINTER(gpe_itp_params), _D, _D, _D, C.c_int,
                                      C.POINTER(gpe_itp_result)]),
    "gpe_groundstate_itp_2comp": (C.c_int, [_P, C.POINTER(gpe_itp_params), C.c_double, C.c_double, C.c_double,
                                            C.c_double, _D, _D, _D, C.c_int, C.POINTER(gpe_itp_result)]),
    "gpe_solve_split": (C.c_int, [_P, C.POINTER(gpe_split_params)]),
    "gpe_solve_split_batch": (C.c_int, [C.POINTER(_P), C.c_int, C.POINTER(gpe_split_params)]),
    "gpe_adjoint_grad": (C.c_int, [_P, C.POINTER(gpe_adjoint_params), _D, _D, _D]),
    "gpe_observables": (C.c_int, [_P, C.POINTER(gpe_obs)]),
    "gpe_detect_core": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _D, C.c_int, C.POINTER(C.c_int), _D, C.c_int,
                                  C.POINTER(C.c_int)]),
    "gpe_groundstate_tf": (C.c_int, [_P, C.c_double, C.c_double, _D, _D]),
    "gpe_synchronize": (C.c_int, [_P]),
    "gpe_timer_start": (C.c_int, [_P]),
    "gpe_timer_stop": (C.c_int, [_P, _D]),
    "gpe_profile_enable": (C.c_int, [_P, C.c_int]),
    "gpe_profile_read": (C.c_int, [_P, C.POINTER(gpe_kernel_stat), C.c_int, C.POINTER(C.c_int)]),
    "gpe_kernel_launches": (C.c_longlong, [_P]),
    "gpe_set_pass_variant": (C.c_int, [_P, C.c_int]),
    "gpe_autotune": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int)]),
    "gpe_selftest_trig": (C.c_int, [_F, _F, _F, C.c_longlong]),
    "gpe_selftest_noise": (C.c_int, [C.c_ulonglong, C.c_ulonglong, C.c_longlong, _F]),
    "gpe_solve_sgpe": (C.c_int, [_P, C.POINTER(gpe_split_params), C.POINTER(gpe_sgpe_params)]),
    "gpe_norm_noalloc": (C.c_int, [_P, C.c_longlong, C.c_int, C.c_double, _P, _D]),
    "gpe_host_register": (C.c_int, [_P, C.c_size_t]),
    "gpe_host_unregister": (C.c_int, [_P]),
}


class GPEError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def _load():
    if not LIB_PATH.exists():
        raise ImportError(
            f"libgpe.so not found at {LIB_PATH}; build it with "
            f"`python gpe-matlab_gb300/build_lib.py` (nvcc, sm_103a)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(ctx, status: int) -> None:
    if status != GPE_OK:
        msg = lib.gpe_last_error(ctx)
        raise GPEError(status, msg.decode() if msg else "")


def dptr(a):
    return a.ctypes.data_as(_D)


def fptr(a):
    return a.ctypes.data_as(_F)
