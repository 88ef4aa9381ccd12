"""ctypes wrapper and build recipe for the C field-evaluation oracle (``cw_oracle.c``).

TEST INFRASTRUCTURE ONLY: loaded by ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` as the checker / timed CPU baseline.  The product
never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "cw_oracle.c")
_LIB = os.path.join(_HERE, "libcw_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile cw_oracle.c with gcc (no FP contraction, so x86 and aarch64 agree)."""
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
               _SRC, "-o", _LIB, "-lm"]
        subprocess.check_call(cmd)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        f = ctypes.c_float
        L.orc_cpu_eval_plane_f32.argtypes = [ctypes.c_int, P, P, P, P, i64, f, f, f, f, i64, i64, i64, P, ctypes.c_int]
        L.orc_cpu_eval_plane_f32.restype = ctypes.c_int
        L.orc_eval_points_f64.argtypes = [P, P, P, P, i64, P, i64, P, ctypes.c_int]
        L.orc_eval_points_f64.restype = ctypes.c_int
        L.orc_eval_separable_f64.argtypes = [i64, i64, i64, P, P, P, P, P, P, i64, P, ctypes.c_int]
        L.orc_eval_separable_f64.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1)


AXIS_XY, AXIS_YZ, AXIS_XZ = 0, 1, 2


def cpu_eval_plane_f32(axis, W32, begin, end, z_layers32, a_start, b_start, c_fixed, d, N,
                       rows=None, nthreads=1):
    """Reference FP32 CPU evaluator (cpu_cw_evaluate_xy / _yz / _xz).  Returns [N, N, 3] complex64
    (rows outside ``rows`` are left zero)."""
    W32 = np.ascontiguousarray(W32, dtype=np.complex64).view(np.float32)
    begin = np.ascontiguousarray(begin, dtype=np.int64)
    end = np.ascontiguousarray(end, dtype=np.int64)
    zl = np.ascontiguousarray(z_layers32, dtype=np.float32)
    out = np.zeros((N, N, 6), dtype=np.float32)
    r0, r1 = (0, N) if rows is None else rows
    rc = lib().orc_cpu_eval_plane_f32(axis, _ptr(W32), _ptr(begin), _ptr(end), _ptr(zl), len(zl),
                                      np.float32(a_start), np.float32(b_start), np.float32(c_fixed),
                                      np.float32(d), N, r0, r1, _ptr(out), nthreads)
    if rc != 0:
        raise RuntimeError("oracle plane evaluation failed")
    return out.view(np.complex64).reshape(N, N, 3)


def thresholds(z_layers, rule="gpu"):
    """Region thresholds: 'gpu' = (double)(float)z_l - 0.001 (gpuEvaluator.cu:34),
    'cpu' = (float)z_l (cpuEvaluator.cpp:303)."""
    zf = np.asarray(z_layers, dtype=np.float32).astype(np.float64)
    return zf - 0.001 if rule == "gpu" else zf


def eval_points_f64(W, begin, end, thr, pts, nthreads=None):
    """FP64 oracle at float32 points [n, 3]; returns [n, 3] complex128."""
    W = np.ascontiguousarray(W, dtype=np.complex128).view(np.float64)
    begin = np.ascontiguousarray(begin, dtype=np.int64)
    end = np.ascontiguousarray(end, dtype=np.int64)
    thr = np.ascontiguousarray(thr, dtype=np.float64)
    pts = np.ascontiguousarray(pts, dtype=np.float32).reshape(-1, 3)
    out = np.zeros((len(pts), 6), dtype=np.float64)
    rc = lib().orc_eval_points_f64(_ptr(W), _ptr(begin), _ptr(end), _ptr(thr), len(thr), _ptr(pts),
                                   len(pts), _ptr(out), nthreads or default_threads())
    if rc != 0:
        raise RuntimeError("oracle point evaluation failed")
    return out.view(np.complex128).reshape(-1, 3)


def eval_separable_f64(kx, ky, kz, zref, Q, pts, nthreads=None):
    """FP64 oracle of one separable region: Q [3, Ma*Mb, J] complex128."""
    kx = np.ascontiguousarray(kx, dtype=np.float64)
    ky = np.ascontiguousarray(ky, dtype=np.float64)
    kz = np.ascontiguousarray(kz, dtype=np.complex128).view(np.float64)
    zref = np.ascontiguousarray(zref, dtype=np.float64)
    Q = np.ascontiguousarray(Q, dtype=np.complex128)
    J = Q.shape[2]
    Qf = Q.view(np.float64)
    pts = np.ascontiguousarray(pts, dtype=np.float32).reshape(-1, 3)
    out = np.zeros((len(pts), 6), dtype=np.float64)
    rc = lib().orc_eval_separable_f64(len(kx), len(ky), J, _ptr(kx), _ptr(ky), _ptr(kz), _ptr(zref),
                                      _ptr(Qf), _ptr(pts), len(pts), _ptr(out), nthreads or default_threads())
    if rc != 0:
        raise RuntimeError("oracle separable evaluation failed")
    return out.view(np.complex128).reshape(-1, 3)


def plane_points(axis, a_start, b_start, c_fixed, d, N):
    """Float32 coordinates of an N x N plane, computed as the reference kernels do
    (start + d * index, one rounding per operation, no fused multiply-add).
    Returns [N (row), N (col), 3] with rows = second axis (y for xy, z for yz/xz)."""
    idx = np.arange(N, dtype=np.float32)
    a = (np.float32(a_start) + np.float32(d) * idx).astype(np.float32)
    b = (np.float32(b_start) + np.float32(d) * idx).astype(np.float32)
    P = np.empty((N, N, 3), dtype=np.float32)
    if axis == AXIS_XY:
        P[..., 0] = a[None, :]
        P[..., 1] = b[:, None]
        P[..., 2] = np.float32(c_fixed)
    elif axis == AXIS_YZ:
        P[..., 0] = np.float32(c_fixed)
        P[..., 1] = a[None, :]
        P[..., 2] = b[:, None]
    else:
        P[..., 0] = a[None, :]
        P[..., 1] = np.float32(c_fixed)
        P[..., 2] = b[:, None]
    return P
