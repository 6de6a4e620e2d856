"""ctypes binding of ``libefs_gb300.so`` (the C ABI in ``include/efs_gb300.h``).

The library is the only compute path: importing this module without the built library raises, and there is
no CPU fallback.  Build it with ``python -c "import __graft_entry__ as g; g.build()"`` (or
``python eulerianfluidsimulation_gb300/build.py``).
"""
import ctypes
import os

from .abi import EfsBatchTuning, EfsParams, EfsQueryMetrics, EfsStats, STATUS_NAMES

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libefs_gb300.so")

_FP = ctypes.POINTER(ctypes.c_float)
_CTX = ctypes.c_void_p

# name -> (restype, argtypes); every declaration of include/efs_gb300.h
SIGNATURES = {
    "efs_params_default": (None, [ctypes.POINTER(EfsParams)]),
    "efs_params_dam": (None, [ctypes.POINTER(EfsParams), ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_float]),
    "efs_abi_version": (ctypes.c_int, []),
    "efs_device_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    "efs_create": (ctypes.c_int, [ctypes.c_int] * 4 + [ctypes.POINTER(EfsParams), ctypes.POINTER(_CTX)]),
    "efs_destroy": (None, [_CTX]),
    "efs_last_error": (ctypes.c_char_p, [_CTX]),
    "efs_set_params": (ctypes.c_int, [_CTX, ctypes.POINTER(EfsParams)]),
    "efs_get_params": (ctypes.c_int, [_CTX, ctypes.POINTER(EfsParams)]),
    "efs_upload_field": (ctypes.c_int, [_CTX, ctypes.c_int, _FP]),
    "efs_download_field": (ctypes.c_int, [_CTX, ctypes.c_int, _FP]),
    "efs_upload_fields": (ctypes.c_int, [_CTX, _FP, _FP, _FP, _FP, _FP]),
    "efs_download_fields": (ctypes.c_int, [_CTX, _FP, _FP, _FP, _FP, _FP, _FP]),
    "efs_download_pressure_fp64": (ctypes.c_int, [_CTX, ctypes.POINTER(ctypes.c_double)]),
    "efs_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(EfsParams), _FP, ctypes.POINTER(_CTX)]),
    "efs_batch_destroy": (None, [_CTX]),
    "efs_batch_last_error": (ctypes.c_char_p, [_CTX]),
    "efs_batch_scene_count": (ctypes.c_int, [_CTX, ctypes.POINTER(ctypes.c_int)]),
    "efs_batch_upload_field": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.c_int, _FP]),
    "efs_batch_download_field": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.c_int, _FP]),
    "efs_batch_stage": (ctypes.c_int, [_CTX, ctypes.c_int]),
    "efs_batch_step": (ctypes.c_int, [_CTX, ctypes.c_int]),
    "efs_batch_synchronize": (ctypes.c_int, [_CTX]),
    "efs_batch_time_steps": (ctypes.c_int, [_CTX, ctypes.c_int, _FP]),
    "efs_batch_stats": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.POINTER(EfsStats)]),
    "efs_batch_kernel_count": (ctypes.c_int, [_CTX, ctypes.POINTER(ctypes.c_int)]),
    "efs_batch_get_tuning": (ctypes.c_int, [_CTX, ctypes.POINTER(EfsBatchTuning)]),
    "efs_batch_set_tuning": (ctypes.c_int, [_CTX, ctypes.POINTER(EfsBatchTuning)]),
    "efs_batch_autotune": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.POINTER(EfsBatchTuning)]),
    "efs_unet_param_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64)]),
    "efs_unet_init": (ctypes.c_int, [_CTX, ctypes.c_uint64, ctypes.c_int]),
    "efs_unet_get_weights": (ctypes.c_int, [_CTX, _FP, ctypes.c_int64]),
    "efs_unet_set_weights": (ctypes.c_int, [_CTX, _FP, ctypes.c_int64]),
    "efs_unet_apply": (ctypes.c_int, [_CTX, _FP, _FP]),
    "efs_unet_loss_grad": (ctypes.c_int, [_CTX, ctypes.c_int, _FP, _FP, _FP, _FP]),
    "efs_unet_add_sample": (ctypes.c_int, [_CTX]),
    "efs_unet_grid": (ctypes.c_int, [_CTX] + [ctypes.POINTER(ctypes.c_int)] * 4),
    "efs_unet_time_forward": (ctypes.c_int, [_CTX, ctypes.c_int, _FP, _FP]),
    "efs_fcg_time_vcycle": (ctypes.c_int, [_CTX, ctypes.c_int, _FP, _FP]),
    "efs_unet_sample_count": (ctypes.c_int, [_CTX, ctypes.POINTER(ctypes.c_int)]),
    "efs_unet_train": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_uint64, _FP]),
    "efs_reset_fields": (ctypes.c_int, [_CTX]),
    "efs_stage": (ctypes.c_int, [_CTX, ctypes.c_int]),
    "efs_step": (ctypes.c_int, [_CTX, ctypes.c_int]),
    "efs_solve": (ctypes.c_int, [_CTX, ctypes.POINTER(EfsStats)]),
    "efs_synchronize": (ctypes.c_int, [_CTX]),
    "efs_get_stats": (ctypes.c_int, [_CTX, ctypes.POINTER(EfsStats)]),
    "efs_total_mass": (ctypes.c_int, [_CTX, ctypes.POINTER(ctypes.c_double)]),
    "efs_step_kernel_count": (ctypes.c_int, [_CTX, ctypes.POINTER(ctypes.c_int)]),
    "efs_solve_timing_arm": (ctypes.c_int, [_CTX, ctypes.c_int]),
    "efs_solve_timing_read": (ctypes.c_int, [_CTX, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                             ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "efs_timer_mark": (ctypes.c_int, [_CTX, ctypes.c_int]),
    "efs_timer_elapsed": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    "efs_solve_noalloc": (ctypes.c_int, [ctypes.c_int] * 4 + [ctypes.POINTER(EfsParams), ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(EfsStats)]),
    "efs_noalloc_last_error": (ctypes.c_char_p, []),
    "efs_scene_dam3d": (ctypes.c_int, [ctypes.c_int] * 5 + [ctypes.c_uint64, _FP, _FP]),
    "efs_scene_dam2d": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _FP, _FP]),
    "efs_scene_batch2d": (ctypes.c_int, [ctypes.c_uint64, ctypes.POINTER(ctypes.c_int), _FP, _FP, ctypes.c_int]),
    "efs_step_host": (ctypes.c_int, [_CTX] + [_FP] * 11),
    "efs_mesh_label": (ctypes.c_int, [_CTX, ctypes.c_int, _FP, ctypes.c_int, _FP, _FP, ctypes.c_float, ctypes.c_float]),
    "efs_mesh_cells": (ctypes.c_int, [_CTX, _FP, ctypes.c_int, _FP, _FP, ctypes.POINTER(ctypes.c_int), ctypes.c_longlong,
                                      ctypes.POINTER(ctypes.c_longlong)]),
    "efs_fill_box": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), _FP]),
    "efs_set_cells": (ctypes.c_int, [_CTX, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_longlong, _FP]),
    "efs_seal_boundary": (ctypes.c_int, [_CTX]),
    "efs_query_box": (ctypes.c_int, [_CTX, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                     ctypes.POINTER(EfsQueryMetrics)]),
}


class EfsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


_lib = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build the CUDA extension first (eulerianfluidsimulation_gb300/build.py)")
        h = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def check(status, ctx=None):
    if status != 0:
        msg = lib().efs_last_error(ctx)
        raise EfsError(status, msg.decode() if msg else "")


def fptr(a):
    return a.ctypes.data_as(_FP) if a is not None else None
