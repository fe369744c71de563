"""ctypes binding of the C-ABI (include/integrator2_gb300.h) to the in-tree libi2gb300.so.

The library must exist in the package directory (built by integrator2_gb300.build); there is
no fallback implementation: a missing or unloadable library raises ImportError-style errors.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libi2gb300.so")

I2_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "I/O error",
          5: "call out of order", 6: "unsupported"}

# every symbol declared in include/integrator2_gb300.h with (restype, argtypes)
_vp, _i32, _i64, _d, _cp = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_char_p
_pp = ctypes.POINTER(ctypes.c_void_p)
SIGNATURES = {
    "i2_status_string": (_cp, [ctypes.c_int]),
    "i2_last_error": (_cp, []),
    "i2_version": (_i32, []),
    "i2_mesh_create": (ctypes.c_int, [_pp]),
    "i2_mesh_destroy": (None, [_vp]),
    "i2_mesh_load_file": (ctypes.c_int, [_vp, _cp, _d]),
    "i2_mesh_set_geometry": (ctypes.c_int, [_vp, _vp, _i32, _vp, _i32]),
    "i2_mesh_prepare": (ctypes.c_int, [_vp, _d]),
    "i2_mesh_prepare_device": (ctypes.c_int, [_vp, _d, ctypes.c_int32]),
    "i2_evaluator_run_stats": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int32]),
    "i2_mesh_device_pairs": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp]),
    "i2_mesh_sizes": (ctypes.c_int, [_vp, _vp, _vp]),
    "i2_mesh_pair_count": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "i2_mesh_copy_pairs": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _i64]),
    "i2_mesh_copy_cell_data": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "i2_mesh_copy_geometry": (ctypes.c_int, [_vp, _vp, _vp]),
    "i2_quadrature_builtin": (ctypes.c_int, [_i32, _vp, _vp, _vp]),
    "i2_integrator_create": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _pp]),
    "i2_integrator_destroy": (None, [_vp]),
    "i2_integrator_set_fixed_refinement_level": (ctypes.c_int, [_vp, _i32]),
    "i2_integrator_set_error_control": (ctypes.c_int, [_vp, ctypes.c_int, _d, _i32]),
    "i2_integrator_get_error_control": (ctypes.c_int, [_vp, _vp, _vp]),
    "i2_integrator_set_precision": (ctypes.c_int, [_vp, ctypes.c_int]),
    "i2_integrator_set_potential_rule": (ctypes.c_int, [_vp, _i32, _i32, _i32, _i32]),
    "i2_integrator_set_self_convention": (ctypes.c_int, [_vp, _i32]),
    "i2_integrator_set_potential": (ctypes.c_int, [_vp, _i32]),
    "i2_integrator_set_hard_pair_tolerance": (ctypes.c_int, [_vp, _d]),
    "i2_evaluator_create": (ctypes.c_int, [_vp, _vp, _pp]),
    "i2_evaluator_destroy": (None, [_vp]),
    "i2_evaluator_set_stream": (ctypes.c_int, [_vp, _vp]),
    "i2_evaluator_run_all_pairs": (ctypes.c_int, [_vp, _i32]),
    "i2_evaluator_run_pairs": (ctypes.c_int, [_vp, _vp, _i64, _vp, _i64, _vp, _i64]),
    "i2_evaluator_run_class": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _i64, _i32]),
    "i2_evaluator_run_class_device": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _i64, _vp, _vp, _vp]),
    "i2_evaluator_backward_class": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _i64, _vp, _vp, _vp]),
    "i2_evaluator_synchronize": (ctypes.c_int, [_vp]),
    "i2_evaluator_result_count": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "i2_evaluator_copy_results": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, _i64]),
    "i2_evaluator_output_results": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _cp]),
    "i2_batch_create": (ctypes.c_int, [_vp, _pp]),
    "i2_batch_destroy": (None, [_vp]),
    "i2_batch_set_stream": (ctypes.c_int, [_vp, _vp]),
    "i2_batch_add": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp, _i64, _i32, _vp]),
    "i2_batch_autotune": (ctypes.c_int, [_vp, _vp]),
    "i2_batch_run": (ctypes.c_int, [_vp]),
    "i2_batch_uses_graph": (ctypes.c_int, [_vp, _vp]),
    "i2_batch_result_count": (ctypes.c_int, [_vp, _i32, _vp]),
    "i2_batch_copy_results": (ctypes.c_int, [_vp, _i32, ctypes.c_int, _vp, _i64]),
    "i2_calibrate_pipes": (ctypes.c_int, [_vp]),
    "i2_not_neighbors_noalloc": (ctypes.c_int, [_vp, _i32, _vp, _i32, _vp, _i64, _d, _i32, _vp, _vp, _vp]),
}

_lock = threading.Lock()
_lib = None


class I2Error(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS.get(code, code)}: {msg}")
        self.code = code


def lib():
    """Loads libi2gb300.so (raises if it is absent: there is no CPU fallback)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"{LIB_PATH} is missing; run integrator2_gb300.build.build() first")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def check(code: int, where: str) -> None:
    if code != I2_OK:
        raise I2Error(code, where, lib().i2_last_error().decode())


def call(name: str, *args):
    check(getattr(lib(), name)(*args), name)
