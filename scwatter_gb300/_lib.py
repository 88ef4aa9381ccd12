"""ctypes binding of ``libscwatter_gb300.so`` (the C ABI in ``include/scwatter.h``).

The library is built in-tree by :mod:`scwatter_gb300.build`.  There is no fallback:
if the shared library is missing or fails to load, every product entry point raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_lib = None

SCW_OK = 0
STATUS_NAMES = {0: "SCW_OK", 1: "SCW_ERR_ARG", 2: "SCW_ERR_IO", 3: "SCW_ERR_FORMAT", 4: "SCW_ERR_CUDA",
                5: "SCW_ERR_NOMEM", 6: "SCW_ERR_STATE", 7: "SCW_ERR_NUMERIC", 8: "SCW_ERR_TIMEOUT",
                9: "SCW_ERR_UNSUPPORTED"}


class ScwError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


P = ctypes.c_void_p
I64 = ctypes.c_int64
I32 = ctypes.c_int
F32 = ctypes.c_float
F64 = ctypes.c_double
PP = ctypes.POINTER(ctypes.c_void_p)

# name -> argtypes (restype is always the int status)
_SIGS = {
    "scw_ctx_create": [I32, P, PP],
    "scw_ctx_destroy": [P],
    "scw_ctx_synchronize": [P],
    "scw_ctx_stream": [P, PP],
    "scw_ctx_launch_count": [P, ctypes.POINTER(I64)],
    "scw_ctx_set_timing": [P, I32],
    "scw_ctx_timing_report": [P, ctypes.c_char_p, I64, P, P, I32, ctypes.POINTER(I32)],
    "scw_cw_create": [PP],
    "scw_cw_destroy": [P],
    "scw_cw_load": [ctypes.c_char_p, PP],
    "scw_cw_save": [P, ctypes.c_char_p],
    "scw_cw_set_incident": [P, I64, P],
    "scw_cw_set_layer_count": [P, I64],
    "scw_cw_set_layer": [P, I64, F64, I64, P, I64, P],
    "scw_cw_counts": [P, ctypes.POINTER(I64), ctypes.POINTER(I64)],
    "scw_cw_layer_counts": [P, I64, ctypes.POINTER(F64), ctypes.POINTER(I64), ctypes.POINTER(I64)],
    "scw_cw_get_incident": [P, P],
    "scw_cw_get_layer": [P, I64, P, P],
    "scw_cw_get_plane_index": [P, F64, ctypes.POINTER(I64)],
    "scw_cw_allocate": [P, ctypes.POINTER(I32), ctypes.POINTER(I64)],
    "scw_cw_unpack": [P, P, P, P, P],
    "scw_gpu_initialize": [P, I32, P, P, P, P, I64, PP],
    "scw_gpu_initialize_cw": [P, P, PP],
    "scw_waves_destroy": [P],
    "scw_waves_set_region_rule": [P, I32],
    "scw_waves_info": [P, ctypes.POINTER(I32), ctypes.POINTER(I64)],
    "scw_gpu_cw_evaluate": [P, P, P, P, F32, F32, F32, F32, F32, F32, F32, I32, I32],
    "scw_eval_plane_device": [P, I32, F32, F32, F32, F32, I32, P],
    "scw_eval_volume_device": [P, F32, F32, F32, F32, F32, F32, I32, I32, I32, P],
    "scw_eval_plane_device_static": [P, I32, F32, F32, F32, F32, I32, P],
    "scw_gen_spheres": [P, I32, I32, I32, I32, P, P, P, P],
    "scw_gen_grf": [P, I32, I32, I32, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                    ctypes.c_uint64, P],
    "scw_npy_read": [P, ctypes.c_char_p, P, P],
    "scw_solve": [P, P, I32, I32, I32, P, PP],
    "scw_solution_destroy": [P],
    "scw_solution_info": [P, P, P, P, P],
    "scw_solution_eig_slices": [P, P, P, P],
    "scw_batch_item_eig_slices": [P, I32, P, P, P],
    "scw_solution_eig_info": [P, P, P, P, P, P],
    "scw_solution_get": [P, P, P, P, P],
    "scw_solution_get_modes": [P, I32, P, P],
    "scw_solution_to_sep": [P, PP],
    "scw_solution_to_cw": [P, PP],
    "scw_solution_write_cw": [P, ctypes.c_char_p],
    "scw_sep_save": [P, ctypes.c_char_p],
    "scw_sep_load": [P, ctypes.c_char_p, P],
    "scw_batch_create": [P, P, I32, I32, I32, PP],
    "scw_batch_run": [P],
    "scw_batch_wait": [P, P],
    "scw_batch_get": [P, I32, P, P, P, PP],
    "scw_batch_item_info": [P, I32, P, P, P, P],
    "scw_batch_item_eig": [P, I32, P, P, P, P, P],
    "scw_batch_info": [P, P, P, P, P, P, P, P, P],
    "scw_batch_destroy": [P],
    "scw_layer_problem": [P, P, I32, I32, I32, P, P, P, P, P],
    "scw_mlp_create": [P, I32, I32, I32, ctypes.c_uint64, PP],
    "scw_mlp_destroy": [P],
    "scw_mlp_info": [P, P, P, P, P],
    "scw_mlp_get_params": [P, P],
    "scw_mlp_set_params": [P, P],
    "scw_mlp_forward": [P, P, I32, P],
    "scw_mlp_gradients": [P, P, P, I32, P, P],
    "scw_mlp_train_step": [P, P, P, I32, F32, P],
    "scw_eig_warm": [P, I32, P, I32, P, P, I32, F64, P, P, P, P],
    "scw_view_scalar": [P, P, I64, I32, P],
    "scw_view_minmax": [P, P, I64, P],
    "scw_view_color": [P, P, I64, P, P],
    "scw_layer_solve": [P, I32, P, P, F64, F64, I32, P, P, P],
    "scw_sep_create": [P, I32, I32, I32, I32, P, P, P, PP],
    "scw_sep_destroy": [P],
    "scw_sep_set_exterior": [P, P, P, P, P, P, P],
    "scw_sep_set_slice": [P, I32, P, P, P, P],
    "scw_sep_set_slice_device": [P, I32, P, P, P, P],
    "scw_sep_from_cw": [P, P, PP],
    "scw_sep_info": [P, ctypes.POINTER(I32), ctypes.POINTER(I32), ctypes.POINTER(I32), ctypes.POINTER(I32)],
    "scw_sep_set_region_rule": [P, I32],
    "scw_sep_create_paired": [P, I32, I32, I32, I32, P, P, P, PP],
    "scw_sep_set_slice_paired": [P, I32, P, P, P, P, P],
    "scw_sep_form": [P, ctypes.POINTER(I32)],
    "scw_measure_peaks": [P, P, P, P, P],
    "scw_sep_get_grid": [P, P, P, P],
    "scw_sep_eval_volume_device": [P, F32, F32, F32, F32, F32, F32, I32, I32, I32, P, I32],
    "scw_sep_eval_volume_host": [P, P, F32, F32, F32, F32, F32, F32, I32, I32, I32, P, I32],
    "scw_sep_set_streaming": [P, I64, I64],
    "scw_sep_set_tiles": [P, I32],
    "scw_sep_set_pipeline": [P, I32, I32],
    "scw_sep_eval_slab_device": [P, F32, F32, F32, F32, F32, F32, I32, I32, I32, I32, P, I32],
    "scw_sep_eval_slab_host": [P, P, F32, F32, F32, F32, F32, F32, I32, I32, I32, I32, P, I32],
    "scw_sep_eval_plane_device": [P, I32, F32, F32, F32, F32, I32, P, I32],
    "scw_sep_gpu_cw_evaluate": [P, P, P, P, F32, F32, F32, F32, F32, F32, F32, I32, I32, I32],
    "scw_zgemm": [P, I32, I32, I32, P, P, P, P, P, I32],
    "scw_zgesv": [P, I32, I32, P, P, I32, P],
    "scw_zgeev": [P, I32, P, P, P, I32, P],
    "scw_zgeev_mixed": [P, I32, P, P, P, I32, P, P, P],
    "scw_cgeev": [P, I32, P, P, P, I32, P],
    "scw_set_qr_cluster": [I32],
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the shared library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"scwatter_gb300 native library missing: {path}")
        _build.build()
    L = ctypes.CDLL(path)
    for name, args in _SIGS.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.scw_last_error.restype = ctypes.c_char_p
    L.scw_last_error.argtypes = []
    L.scw_version.restype = ctypes.c_char_p
    _lib = L
    return L


def exported_symbols():
    return list(_SIGS) + ["scw_last_error", "scw_version"]


def check(status: int):
    if status != SCW_OK:
        msg = load().scw_last_error()
        raise ScwError(status, msg.decode() if msg else "")


def call(name: str, *args):
    check(getattr(load(), name)(*args))
