"""Separable ("GEMM form") evaluator: Python handle of ``scw_sep`` (include/scwatter.h).

Inside slice l every wave of the volume solver is (harmonic p = (a, b), mode j) with
kx = kx_a, ky = ky_b, kz = kz_j, so the field of a z-plane is two small complex GEMMs
(e^{i ky y} . C(z) . e^{i kx x}); the per-slice mode sums C(z) stream the coefficients Q
from HBM once per group of z-planes.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .cw import CoupledWaveStructure
from .evaluator import Context

FP32 = 1        # SIMT FP32 output GEMM
TF32X3 = 2      # tcgen05 kind::tf32, hi/lo split, 3 products
BF16X3 = 3      # tcgen05 kind::f16 (bf16), hi/lo split, 3 products


def _c(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128))
    return a, ctypes.c_void_p(a.ctypes.data)


class SeparableSet:
    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle

    @classmethod
    def create(cls, ctx: Context, kx, ky, z_boundaries, modes_per_half: int) -> "SeparableSet":
        kx = np.ascontiguousarray(kx, dtype=np.float64)
        ky = np.ascontiguousarray(ky, dtype=np.float64)
        zb = np.ascontiguousarray(z_boundaries, dtype=np.float64)
        h = ctypes.c_void_p()
        _lib.call("scw_sep_create", ctx.handle, len(kx), len(ky), len(zb) - 1, int(modes_per_half),
                  kx.ctypes.data_as(ctypes.c_void_p), ky.ctypes.data_as(ctypes.c_void_p),
                  zb.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h))
        return cls(ctx, h)

    @classmethod
    def from_factored(cls, ctx: Context, fs) -> "SeparableSet":
        """From a :class:`scwatter_gb300.synthetic.FactoredSample`-like object."""
        s = cls.create(ctx, fs.kx, fs.ky, fs.z, fs.gamma_dn.shape[1])
        keep = [_c(fs.inc), _c(fs.kz_inc), _c(fs.refl), _c(fs.kz_refl), _c(fs.trans), _c(fs.kz_trans)]
        _lib.call("scw_sep_set_exterior", s.handle, *[p for _, p in keep])
        for l in range(fs.Z):
            kd, pkd = _c(fs.gamma_dn[l] * fs.k)
            ku, pku = _c(fs.gamma_up[l] * fs.k)
            qd = np.ascontiguousarray(fs.Q_dn[l], dtype=np.complex64)
            qu = np.ascontiguousarray(fs.Q_up[l], dtype=np.complex64)
            _lib.call("scw_sep_set_slice_device", s.handle, l, pkd, ctypes.c_void_p(qd.ctypes.data), pku,
                      ctypes.c_void_p(qu.ctypes.data))
            ctx.synchronize()
        return s

    @classmethod
    def from_cw(cls, ctx: Context, cw: CoupledWaveStructure) -> "SeparableSet":
        native = cw._to_native()
        try:
            h = ctypes.c_void_p()
            _lib.call("scw_sep_from_cw", ctx.handle, native, ctypes.byref(h))
        finally:
            _lib.load().scw_cw_destroy(native)
        return cls(ctx, h)

    @classmethod
    def load(cls, ctx: Context, filename: str) -> "SeparableSet":
        """Reads a compact factored coefficient file (.cwf) written by :meth:`save`."""
        h = ctypes.c_void_p()
        _lib.call("scw_sep_load", ctx.handle, str(filename).encode(), ctypes.byref(h))
        return cls(ctx, h)

    def save(self, filename: str) -> None:
        """Writes the set as a compact factored coefficient file (.cwf): per slice Q_check /
        Q_hat in complex64 and the modes' kz, plus the exterior blocks and k grids."""
        _lib.call("scw_sep_save", self.handle, str(filename).encode())

    def info(self):
        v = [ctypes.c_int() for _ in range(4)]
        _lib.call("scw_sep_info", self.handle, *[ctypes.byref(x) for x in v])
        return tuple(x.value for x in v)

    def set_region_rule(self, rule: int):
        _lib.call("scw_sep_set_region_rule", self.handle, int(rule))

    def eval_volume_device(self, x_start, y_start, z_start, dx, dy, dz, Nx, Ny, Nz, dE_ptr: int, method=FP32):
        _lib.call("scw_sep_eval_volume_device", self.handle, x_start, y_start, z_start, dx, dy, dz, int(Nx), int(Ny),
                  int(Nz), ctypes.c_void_p(dE_ptr), int(method))

    def eval_plane_device(self, axis, a_start, b_start, c, d, N, dE_ptr: int, method=FP32):
        _lib.call("scw_sep_eval_plane_device", self.handle, int(axis), a_start, b_start, c, d, int(N),
                  ctypes.c_void_p(dE_ptr), int(method))

    def evaluate_planes_host(self, x_start, y_start, z_start, x, y, z, d, N, method=FP32):
        outs = [np.empty((N, N, 3), dtype=np.complex64) for _ in range(3)]
        _lib.call("scw_sep_gpu_cw_evaluate", self.handle, *[ctypes.c_void_p(o.ctypes.data) for o in outs],
                  x_start, y_start, z_start, x, y, z, d, int(N), int(self.ctx.device), int(method))
        return tuple(outs)

    def close(self):
        if self.handle:
            _lib.load().scw_sep_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
