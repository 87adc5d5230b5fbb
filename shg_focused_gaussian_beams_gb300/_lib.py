"""ctypes binding of the C ABI in include/shg.h (libshg_gb300.so, built in-tree).

The library is required: loading fails loudly when it has not been built; there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# SHG_LIB selects another build of the same C ABI (the check or sanitizer variants of build.py)
LIB_PATH = os.environ.get("SHG_LIB") or os.path.join(HERE, "_build", "libshg_gb300.so")

_i, _f, _d = C.c_int, C.c_float, C.c_double
_pf, _pd, _pi, _vp = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_void_p

SHG_OK = 0
ERRORS = {1: "SHG_ERR_INVALID", 2: "SHG_ERR_UNSUPPORTED", 3: "SHG_ERR_CUDA", 4: "SHG_ERR_NOMEM",
          5: "SHG_ERR_STATE", 6: "SHG_ERR_NONFINITE"}


class ShgError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: {ERRORS.get(code, code)}: {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("nx", _i), ("ny", _i), ("nz", _i), ("lx", _f), ("ly", _f), ("lz", _f), ("lp", _f),
                ("deff", _f), ("lambda_qpm", _f), ("alpha_p", _f), ("alpha_s", _f), ("beta_s", _f),
                ("rho_p", _f), ("rho_s", _f), ("kth", _f), ("htc", _f), ("thermal", _i), ("bc", _i),
                ("sh_seed", _i), ("device", _i), ("crystal", _i)]


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", _i), ("ms", _d), ("bytes", _d)]


class Instance(C.Structure):
    _fields_ = [("nx", _i), ("ny", _i), ("nz", _i), ("lx", _f), ("ly", _f), ("power", _f), ("waist", _f),
                ("temp", _f), ("focal", _f)]


# name -> (restype, argtypes)
SIGNATURES = {
    "shg_config_init": (_i, [C.POINTER(Config)]),
    "shg_index": (_i, [_i, _f, _f, _pf]),
    "shg_create": (_i, [C.POINTER(Config), C.POINTER(_vp)]),
    "shg_destroy": (_i, [_vp]),
    "shg_run": (_i, [_vp, _f, _f, _f, _f, _f, _f, _f, _i, _i]),
    "shg_set_input_pump": (_i, [_vp, _f, _f, _f, _f]),
    "shg_set_input_fields": (_i, [_vp, _pf, _pf]),
    "shg_cwes": (_i, [_vp, _f]),
    "shg_cwes_device": (_i, [_vp, _f, _vp, _vp, _vp, _vp, _vp]),
    "shg_get_fields": (_i, [_vp, _pf, _pf]),
    "shg_get_powers": (_i, [_vp, _pd, _pd, _pd]),
    "shg_efficiency": (_i, [_vp, _pd]),
    "shg_last_error": (C.c_char_p, []),
    "shg_batch_create": (_i, [C.POINTER(Config), C.POINTER(Instance), _i, C.POINTER(_vp)]),
    "shg_batch_destroy": (_i, [_vp]),
    "shg_batch_run": (_i, [_vp, _pd, _vp]),
    "shg_batch_fields": (_i, [_vp, _vp, _vp]),
    "shg_batch_set_instances": (_i, [_vp, C.POINTER(Instance), _i]),
    "shg_batch_field_offsets": (_i, [_vp, C.POINTER(C.c_longlong)]),
    "shg_batch_profile": (_i, [_vp, C.POINTER(KernelStat), _i, _pi]),
    "shg_batch_run_async": (_i, [_vp, _vp]),
    "shg_batch_results": (_i, [_vp, _pd]),
    "shg_batch_launch_count": (_i, [_vp, _pi]),
    "shg_batch_autotune": (_i, [_vp, _vp]),
    "shg_batch_schedule": (_i, [_vp, C.c_char_p, _i]),
    "shg_batch_set_schedule": (_i, [_vp, _i, _i, _i, _i]),
    "shg_batch_set_schedule_split": (_i, [_vp, _i, _i, _i, _i]),
    "shg_batch_timeline": (_i, [_vp, _pd, _i, _pi, _vp]),
    "shg_batch_io_bytes": (_i, [_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "shg_dft2d_device": (_i, [_i, _i, _vp, _vp, _vp]),
    "shg_grad_device": (_i, [_vp, _f, _vp, _vp, _i, _vp, _vp, _pd, _vp]),
    "shg_grad_run": (_i, [_vp, _f, _f, _f, _f, _vp, _i, _vp, _pd, _vp]),
    "shg_set_poling_period": (_i, [_vp, _f]),
    "shg_set_output_dir": (_i, [_vp, C.c_char_p]),
    "shg_get_temperature": (_i, [_vp, _pf]),
    "shg_get_jacobi_counts": (_i, [_vp, _pi]),
    "shg_set_jacobi_rule": (_i, [_vp, C.c_double, _i, _i]),
    "shg_get_jacobi_residual": (_i, [_vp, _pd]),
    "shg_init_temperature": (_i, [C.POINTER(Config), _f, _f, _f, _i, _pf]),
    "shg_heat_sweeps": (_i, [C.POINTER(Config), _pf, _pf, _f, _i, _i]),
    "shg_dk_thermal": (_i, [C.POINTER(Config), _pf, _pf, _pf, _pf]),
    "shg_heat_sweeps_device": (_i, [C.POINTER(Config), _vp, _vp, _vp, _f, _i, _i, _vp]),
    "shg_cwes_noalloc": (_i, [C.POINTER(Config), _f, _vp, _vp, _vp, _vp, _pd, _vp]),
    "shg_thgrad_create": (_i, [C.POINTER(Config), _i, C.POINTER(_vp)]),
    "shg_thgrad_destroy": (None, [_vp]),
    "shg_thgrad_solve_temperature": (_i, [_vp, _i, _f, _f, _f, _f, _f, _f, _f, _pi]),
    "shg_thgrad_set_temperature": (_i, [_vp, _i, _pf, _f, _f, _f]),
    "shg_thgrad_get_temperature": (_i, [_vp, _i, _pf]),
    "shg_thgrad_gaussian_pumps": (_i, [_vp, _vp, _vp]),
    "shg_thgrad_forward": (_i, [_vp, _vp, _vp, _vp, _pd, _pd, _vp]),
    "shg_thgrad_gradient": (_i, [_vp, _vp, _i, _vp, _pd, _pd, _vp]),
    "shg_thgrad_launch_count": (_i, [_vp]),
    "shg_thgrad_device_bytes": (C.c_double, [_vp]),
    "shg_check_status": (_i, [_pi, _pi, C.POINTER(C.c_longlong)]),
    "shg_check_selftest": (_i, [C.c_longlong]),
}

_lib = None


def lib():
    """Load libshg_gb300.so (raises if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build the CUDA library first "
                              "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int, where: str):
    if rc != SHG_OK:
        raise ShgError(rc, where, lib().shg_last_error().decode(errors="replace"))


def default_config(**overrides) -> Config:
    c = Config()
    check(lib().shg_config_init(C.byref(c)), "shg_config_init")
    for k, v in overrides.items():
        setattr(c, k, v)
    return c
