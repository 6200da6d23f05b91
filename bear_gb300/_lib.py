"""ctypes binding of libbeargb300.so (declarations in include/bear_gb300.h).

The library must exist: on a machine with a GPU the product path never falls
back to anything else. ``load()`` raises if the shared object is missing and
cannot be built.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_u8p = C.POINTER(C.c_uint8)
_lib = None
_lock = threading.Lock()

EXPORTS = {
    "bear_last_error": (C.c_char_p, []),
    "bear_model_create": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]),
    "bear_model_add_observation": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int, _dp, _dp, _dp,
                                             _dp, _dp, C.c_int, _dp, _dp, C.c_char_p, C.c_char_p]),
    "bear_model_finalize": (C.c_int, [C.c_void_p]),
    "bear_model_prepare": (C.c_int, [C.c_void_p]),
    "bear_model_observation_setup": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_longlong), C.c_int, _ip]),
    "bear_model_operator_row": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip, C.POINTER(_dp)]),
    "bear_model_info": (C.c_int, [C.c_void_p, _ip, _ip, _ip, _ip]),
    "bear_model_wavenumbers": (C.c_int, [C.c_void_p, _dp]),
    "bear_model_observation_size": (C.c_int, [C.c_void_p, C.c_int, _ip]),
    "bear_model_device_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    "bear_model_destroy": (None, [C.c_void_p]),
    "bear_forward": (C.c_int, [C.c_void_p, _dp, C.c_int, _dp, C.POINTER(_dp), _ip, C.c_void_p]),
    "bear_compute_model": (C.c_int, [C.c_void_p, _dp, C.c_int, _dp, _dp, _ip, C.c_void_p]),
    "bear_loglike": (C.c_int, [C.c_void_p, _dp, C.c_int, _dp, C.c_void_p]),
    "bear_loglike_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "bear_loglike_grad_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p]),
    "bear_model_set_precision": (C.c_int, [C.c_void_p, C.c_int]),
    "bear_model_set_launch": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "bear_model_set_gradient_memory": (C.c_int, [C.c_void_p, C.c_longlong]),
    "bear_model_set_tau_cutoff": (C.c_int, [C.c_void_p, C.c_double]),
    "bear_model_table_sharing": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_size_t)]),
    "bear_model_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                      C.POINTER(C.c_int)]),
    "bear_batch_graph_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                          C.POINTER(C.c_void_p)]),
    "bear_batch_graph_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "bear_batch_graph_destroy": (C.c_int, [C.c_void_p]),
    "bear_loglike_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "bear_model_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "bear_model_stage_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "bear_model_table_info": (C.c_int, [C.c_void_p, _ip, _ip, _ip, C.POINTER(C.c_longlong)]),
    "bear_model_stencil_rows": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_longlong)]),
    "bear_model_set_priors": (C.c_int, [C.c_void_p, C.c_int, _ip, _dp, _dp, _dp, _ip]),
    "bear_contribution_functions": (C.c_int, [C.c_void_p, _dp, C.c_int, _dp, _dp, C.c_void_p]),
    "bear_prior_transform_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "bear_loglike_cube_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p]),
    "bear_batch_graph_create_cube": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.POINTER(C.c_void_p)]),
}


class EngineError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[bear_gb300 error {code}] {msg}")
        self.code = code


def load(build_if_missing: bool = True):
    """Load (building first if needed) and return the engine library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"engine library {path} is missing; run bear_gb300.build.build()")
        lib = C.CDLL(path)
        for name, (res, args) in EXPORTS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int) -> None:
    if rc != 0:
        raise EngineError(rc, _lib.bear_last_error().decode())


def dptr(a):
    """ctypes double* of a contiguous float64 numpy array (or NULL)."""
    if a is None:
        return C.cast(None, _dp)
    return a.ctypes.data_as(_dp)
