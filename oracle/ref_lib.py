"""ctypes access to the reference-evaluator checkers built by ``oracle/ref_build.py``.

Test infrastructure only.  ``evaluate("reference", ...)`` runs the reference viewer's own
gpu_initialize / gpu_cw_evaluate (gpuEvaluator.cu:15-165, compiled unchanged);
``evaluate("shim", ...)`` runs the same calls through the drop-in shim over the GB300 library.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from oracle import ref_build

_libs = {}


def available() -> bool:
    return os.path.exists(ref_build.LIB_REF) and os.path.exists(ref_build.LIB_SHIM)


def _load(which):
    if which not in _libs:
        path = {"reference": ref_build.LIB_REF, "shim": ref_build.LIB_SHIM}[which]
        L = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
        L.scwref_evaluate.restype = ctypes.c_int
        L.scwref_evaluate.argtypes = ([ctypes.c_int] + [ctypes.c_void_p] * 4 + [ctypes.c_int64] +
                                      [ctypes.c_void_p] * 3 + [ctypes.c_float] * 7 + [ctypes.c_int, ctypes.c_int])
        L.scwref_last_error.restype = ctypes.c_char_p
        _libs[which] = L
    return _libs[which]


def evaluate(which, W, begin, end, z_layers, x_start, y_start, z_start, x, y, z, d, N, device=0):
    """The three planes of gpu_cw_evaluate (xy at z, xz at y, yz at x), each [N, N, 3] complex64,
    from the unpacked globals: W [n, 6] complex (cast to float as cw_unpack does,
    cpuEvaluator.cpp:61-102), begin / end [L+1], z_layers [L]."""
    L = _load(which)
    Wf = np.ascontiguousarray(np.asarray(W).astype(np.complex64)).view(np.float32).reshape(-1, 12)
    b = np.ascontiguousarray(begin, dtype=np.int32)
    e = np.ascontiguousarray(end, dtype=np.int32)
    zl = np.ascontiguousarray(z_layers, dtype=np.float32)
    outs = [np.zeros((N, N, 3), np.complex64) for _ in range(3)]
    ptr = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
    rc = L.scwref_evaluate(len(zl), ptr(zl), ptr(b), ptr(e), ptr(Wf), len(Wf), *[ptr(o) for o in outs],
                           float(x_start), float(y_start), float(z_start), float(x), float(y), float(z), float(d),
                           int(N), int(device))
    if rc != 0:
        raise RuntimeError(f"{which} evaluator: {L.scwref_last_error().decode()}")
    return outs
