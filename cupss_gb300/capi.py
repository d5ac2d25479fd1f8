"""ctypes binding of the C-ABI declared in include/cupss_gb300.h.

The shared library is the in-tree ``cupss_gb300/libcupss.so`` built by
``cupss_gb300/build.py``.  Loading fails loudly if it is missing: there is no
fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcupss.so")

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_UNSUPPORTED = -3
ERR_STATE = -4
ERR_PARSE = -5
ERR_LIMIT = -6


class Pres(C.Structure):
    """``cupssgb_pres`` == reference ``struct pres`` (inc/cupss/defines.h:31-39)."""
    _fields_ = [("preFactor", C.c_float), ("q2n", C.c_int), ("iqx", C.c_int), ("iqy", C.c_int),
                ("iqz", C.c_int), ("invq", C.c_int)]


class CupssError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("cupss_gb300 error %d: %s" % (code, msg))
        self.code = code


_P = C.c_void_p
_I = C.c_int
_F = C.c_float
_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int)
_PP = C.POINTER(Pres)
_S = C.c_char_p
_LL = C.c_longlong
_ULL = C.c_ulonglong

# cupssgb_callback: void (*)(void* evolver, float* field_pairs, int sx, int sy, int sz)
CALLBACK = C.CFUNCTYPE(None, _P, _P, _I, _I, _I)

# name -> (restype, argtypes)
SIGNATURES = {
    "cupssgb_last_error": (_S, []),
    "cupssgb_version": (_I, []),
    "cupssgb_solver_create": (_I, [_I, _I, _I, _F, _F, _F, _F, C.POINTER(_P)]),
    "cupssgb_solver_destroy": (_I, [_P]),
    "cupssgb_solver_add_field": (_I, [_P, _I]),
    "cupssgb_solver_set_implicit": (_I, [_P, _I, _PP, _I]),
    "cupssgb_solver_update_implicit": (_I, [_P, _I, _PP, _I]),
    "cupssgb_solver_add_term": (_I, [_P, _I, _IP, _I, _PP, _I]),
    "cupssgb_solver_set_term_pres": (_I, [_P, _I, _I, _PP, _I]),
    "cupssgb_solver_set_noise": (_I, [_P, _I, _PP]),
    "cupssgb_solver_set_seed": (_I, [_P, _ULL]),
    "cupssgb_solver_prepare": (_I, [_P]),
    "cupssgb_solver_set_real": (_I, [_P, _I, _FP]),
    "cupssgb_solver_set_real_device": (_I, [_P, _I, _P]),
    "cupssgb_solver_advance": (_I, [_P, _I]),
    "cupssgb_solver_get_real": (_I, [_P, _I, _FP]),
    "cupssgb_solver_get_real_device": (_I, [_P, _I, _P]),
    "cupssgb_solver_get_fourier": (_I, [_P, _I, _FP]),
    "cupssgb_solver_get_fourier_device": (_I, [_P, _I, _P]),
    "cupssgb_solver_synchronize": (_I, [_P]),
    "cupssgb_solver_advance_phase": (_I, [_P, _I]),
    "cupssgb_solver_get_real_pairs_device": (_I, [_P, _I, _P]),
    "cupssgb_solver_get_dealiased_pairs_device": (_I, [_P, _I, _P]),
    "cupssgb_solver_set_fourier_device": (_I, [_P, _I, _P]),
    "cupssgb_solver_set_real_pairs_device": (_I, [_P, _I, _P, _P]),
    "cupssgb_solver_step_count": (_LL, [_P]),
    "cupssgb_solver_launch_count": (_LL, [_P]),
    "cupssgb_solver_device_bytes": (_LL, [_P]),
    "cupssgb_solver_stream": (_P, [_P]),
    "cupssgb_solver_time_advance": (_I, [_P, _I, C.POINTER(C.c_double)]),
    "cupssgb_solver_set_kernel_timing": (_I, [_P, _I]),
    "cupssgb_solver_kernel_report": (_I, [_P, C.c_char_p, _I]),
    "cupssgb_solver_generated_source": (_I, [_P, _I, C.c_char_p, _I]),
    "cupssgb_solver_set_generated_programs": (_I, [_P, _I]),
    "cupssgb_jit_check": (_I, [C.c_char_p, C.c_char_p, _I]),
    "cupssgb_solver_set_members": (_I, [_P, _I]),
    "cupssgb_solver_members": (_I, [_P]),
    "cupssgb_solver_set_member_term_pres": (_I, [_P, _I, _I, _I, _PP, _I]),
    "cupssgb_solver_set_member_implicit": (_I, [_P, _I, _I, _PP, _I]),
    "cupssgb_solver_set_member_noise": (_I, [_P, _I, _I, _PP]),
    "cupssgb_solver_set_member_seed": (_I, [_P, _I, _ULL]),
    "cupssgb_solver_set_member_active": (_I, [_P, _I, _I]),
    "cupssgb_solver_reset_member": (_I, [_P, _I]),
    "cupssgb_solver_member_step": (_LL, [_P, _I]),
    "cupssgb_solver_set_real_member": (_I, [_P, _I, _I, _FP]),
    "cupssgb_solver_set_real_member_device": (_I, [_P, _I, _I, _P]),
    "cupssgb_solver_get_real_member": (_I, [_P, _I, _I, _FP]),
    "cupssgb_solver_get_real_member_device": (_I, [_P, _I, _I, _P]),
    "cupssgb_solver_tune_report": (_I, [_P, C.c_char_p, _I]),
    "cupssgb_solver_estimate_bytes": (_LL, [_P, _I]),
    "cupssgb_solver_query": (_I, [_P]),
    "cupssgb_real_to_fourier_noalloc": (_I, [_P, _P, _I, _I, _I, _P]),
    "cupssgb_host_alloc": (_I, [_LL, C.POINTER(_P)]),
    "cupssgb_host_free": (_I, [_P]),
    "cupssgb_set_device": (_I, [_I]),
    "cupssgb_device_info": (_I, [C.c_char_p, _I]),
    "cupssgb_multi_check": (_I, [C.POINTER(_P), _I, C.c_char_p, _I]),
    "cupssgb_multi_create": (_I, [C.POINTER(_P), _I, C.POINTER(_P)]),
    "cupssgb_multi_destroy": (_I, [_P]),
    "cupssgb_multi_advance": (_I, [_P, _I]),
    "cupssgb_multi_launch_count": (_LL, [_P]),
    "cupssgb_multi_describe": (_I, [_P, C.c_char_p, _I]),
    "cupssgb_multi_choose": (_I, [_P]),
    "cupssgb_solver_set_stream_priority": (_I, [_P, _I]),
    "cupssgb_multi_generated_source": (_I, [C.POINTER(_P), _I, _I, C.c_char_p, _I]),
    "cupssgb_tune_cache_path": (_I, [C.c_char_p, _I]),
    "cupssgb_tune_cache_lookup": (_I, [_S, C.c_char_p, _I]),
    "cupssgb_tune_cache_store": (_I, [_S, _S]),
    "cupssgb_solver_snapshot_real": (_I, [_P, _I, _P, _P]),
    "cupssgb_evolver_flush_output": (_I, [_P]),
    "cupssgb_evolver_create_from_file": (_I, [_P, _S]),
    "cupssgb_evolver_initialize_uniform": (_I, [_P, _S, _F]),
    "cupssgb_evolver_initialize_uniform_noise": (_I, [_P, _S, _F]),
    "cupssgb_evolver_initialize_normal_noise": (_I, [_P, _S, _F, _F]),
    "cupssgb_evolver_initialize_half_system": (_I, [_P, _S, _F, _F, _F, _I]),
    "cupssgb_evolver_initialize_droplet": (_I, [_P, _S, _F, _F, _F, _F, _I, _I, _I]),
    "cupssgb_evolver_add_droplet": (_I, [_P, _S, _F, _F, _F, _I, _I, _I]),
    "cupssgb_evolver_initialize_from_file": (_I, [_P, _S, _S, _I, C.c_char]),
    "cupssgb_evolver_get_host_real": (_I, [_P, _S, _FP]),
    "cupssgb_write_field_csv": (_I, [_S, _S, _FP, _I, _I, _I, _I]),
    "cupssgb_evolver_create": (_I, [_I, _I, _I, _I, _F, _F, _F, _F, _I, C.POINTER(_P)]),
    "cupssgb_evolver_destroy": (_I, [_P]),
    "cupssgb_evolver_create_field": (_I, [_P, _S, _I]),
    "cupssgb_evolver_add_parameter": (_I, [_P, _S, _F]),
    "cupssgb_evolver_add_equation": (_I, [_P, _S]),
    "cupssgb_evolver_add_noise": (_I, [_P, _S, _S]),
    "cupssgb_evolver_update_parameter": (_I, [_P, _S, _F]),
    "cupssgb_evolver_set_output_field": (_I, [_P, _S, _I]),
    "cupssgb_evolver_set_seed": (_I, [_P, _ULL]),
    "cupssgb_evolver_set_real": (_I, [_P, _S, _FP]),
    "cupssgb_evolver_prepare": (_I, [_P]),
    "cupssgb_evolver_advance": (_I, [_P, _I]),
    "cupssgb_evolver_write_out": (_I, [_P]),
    "cupssgb_evolver_get_real": (_I, [_P, _S, _FP]),
    "cupssgb_evolver_get_fourier": (_I, [_P, _S, _FP]),
    "cupssgb_evolver_get_parameter": (_F, [_P, _S]),
    "cupssgb_evolver_current_step": (_I, [_P]),
    "cupssgb_evolver_describe": (_I, [_P, C.c_char_p, _I]),
    "cupssgb_evolver_solver": (_P, [_P]),
    "cupssgb_evolver_set_callback": (_I, [_P, _S, _I, CALLBACK]),
    "cupssgb_ensemble_create": (_I, [C.POINTER(_P)]),
    "cupssgb_ensemble_destroy": (_I, [_P]),
    "cupssgb_ensemble_create_field": (_I, [_P, _S, _I]),
    "cupssgb_ensemble_add_parameter": (_I, [_P, _S, _F]),
    "cupssgb_ensemble_add_equation": (_I, [_P, _S]),
    "cupssgb_ensemble_add_noise": (_I, [_P, _S, _S]),
    "cupssgb_ensemble_add_member": (_I, [_P, _I, _I, _I, _F, _F, _F, _F, _ULL]),
    "cupssgb_ensemble_set_member_parameter": (_I, [_P, _I, _S, _F]),
    "cupssgb_ensemble_prepare": (_I, [_P]),
    "cupssgb_ensemble_set_real": (_I, [_P, _I, _S, _FP]),
    "cupssgb_ensemble_advance": (_I, [_P, _I]),
    "cupssgb_ensemble_get_real": (_I, [_P, _I, _S, _FP]),
    "cupssgb_ensemble_groups": (_I, [_P]),
    "cupssgb_ensemble_device_bytes": (_LL, [_P]),
    "cupssgb_ensemble_launch_count": (_LL, [_P]),
    "cupssgb_ensemble_describe": (_I, [_P, C.c_char_p, _I]),
    "cupssgb_server_create": (_I, [C.c_double, _I, _I, C.POINTER(_P)]),
    "cupssgb_server_destroy": (_I, [_P]),
    "cupssgb_server_add_system": (_I, [_P]),
    "cupssgb_server_create_field": (_I, [_P, _I, _S, _I]),
    "cupssgb_server_add_parameter": (_I, [_P, _I, _S, _F]),
    "cupssgb_server_add_equation": (_I, [_P, _I, _S]),
    "cupssgb_server_add_noise": (_I, [_P, _I, _S, _S]),
    "cupssgb_server_set_output_field": (_I, [_P, _I, _S]),
    "cupssgb_server_submit": (_LL, [_P, _I, _I, _I, _I, _F, _F, _F, _F, _LL, _ULL, _I, C.POINTER(_S), _FP, _I,
                                    C.POINTER(_S), C.POINTER(_FP)]),
    "cupssgb_server_warm": (_I, [_P, _I, _I, _I, _I, _F, _F, _F, _F]),
    "cupssgb_server_wait": (_I, [_P, _LL, C.c_double]),
    "cupssgb_server_result": (_I, [_P, _LL, _FP]),
    "cupssgb_server_times": (_I, [_P, _LL, C.POINTER(C.c_double)]),
    "cupssgb_server_stats": (_I, [_P, C.c_char_p, _I]),
}

_lib = None


def load(path: str | None = None):
    """Loads (once) and returns the C-ABI library with typed entry points."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError("cupss_gb300: %s is missing; run cupss_gb300/build.py (or "
                          "__graft_entry__.build()) first -- there is no fallback" % p)
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(code: int):
    if code < 0:
        raise CupssError(code, load().cupssgb_last_error().decode())
    return code


def fptr(arr):
    import numpy as np
    assert arr.dtype == np.float32 and arr.flags["C_CONTIGUOUS"]
    return arr.ctypes.data_as(_FP)


def pres_array(items):
    n = len(items)
    arr = (Pres * max(n, 1))()
    for i, p in enumerate(items):
        if isinstance(p, Pres):
            arr[i] = p
        else:
            arr[i] = Pres(float(p[0]), *[int(v) for v in p[1:6]])
    return arr, n
