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


def _host_ptr(a, name):
    """Address of a C-contiguous complex64 host array (numpy) or CPU tensor (torch)."""
    if isinstance(a, np.ndarray):
        if a.dtype != np.complex64 or not a.flags.c_contiguous:
            raise ValueError(f"{name} must be a C-contiguous complex64 array")
        return a.ctypes.data
    if getattr(a, "is_cuda", True) or str(getattr(a, "dtype", "")) != "torch.complex64" or not a.is_contiguous():
        raise ValueError(f"{name} must be a contiguous complex64 host array or CPU tensor")
    return a.data_ptr()


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
    def create_paired(cls, ctx: Context, kx, ky, z_boundaries, modes_per_half: int) -> "SeparableSet":
        """Empty paired set (``scw_sep_create_paired``): per slice one block V and the mode
        amplitudes, Q_dn = V diag(beta_dn), Q_up = diag(1, 1, -1) V diag(beta_up)."""
        kx = np.ascontiguousarray(kx, dtype=np.float64)
        ky = np.ascontiguousarray(ky, dtype=np.float64)
        zb = np.ascontiguousarray(z_boundaries, dtype=np.float64)
        h = ctypes.c_void_p()
        _lib.call("scw_sep_create_paired", ctx.handle, len(kx), len(ky), len(zb) - 1, int(modes_per_half),
                  kx.ctypes.data_as(ctypes.c_void_p), ky.ctypes.data_as(ctypes.c_void_p),
                  zb.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h))
        return cls(ctx, h)

    @classmethod
    def from_paired(cls, ctx: Context, ps, V=None) -> "SeparableSet":
        """From a :class:`scwatter_gb300.synthetic.PairedSample`; ``V`` (host array or device
        tensor, [Z, 3, MF, J] complex64) overrides ``ps.V``."""
        b = ps.base
        V = ps.V if V is None else V
        s = cls.create_paired(ctx, b.kx, b.ky, b.z, ps.beta_dn.shape[1])
        keep = [_c(b.inc), _c(b.kz_inc), _c(b.refl), _c(b.kz_refl), _c(b.trans), _c(b.kz_trans)]
        _lib.call("scw_sep_set_exterior", s.handle, *[p for _, p in keep])
        for l in range(b.Z):
            s.set_slice_paired(l, b.gamma_dn[l] * b.k, b.gamma_up[l] * b.k, V[l], ps.beta_dn[l], ps.beta_up[l])
            ctx.synchronize()
        return s

    def set_slice_paired(self, l, kz_dn, kz_up, V_l, beta_dn, beta_up):
        """Slice l of a paired set: kz and amplitudes [J] complex, V_l [3, MF, J] complex64 (host
        array or device tensor; the copy is asynchronous on the context stream)."""
        kd, pkd = _c(kz_dn)
        ku, pku = _c(kz_up)
        bd, pbd = _c(beta_dn)
        bu, pbu = _c(beta_up)
        if hasattr(V_l, "data_ptr"):
            vptr, keep = V_l.data_ptr(), V_l
        else:
            keep = np.ascontiguousarray(V_l, dtype=np.complex64)
            vptr = keep.ctypes.data
        _lib.call("scw_sep_set_slice_paired", self.handle, int(l), pkd, pku, ctypes.c_void_p(vptr), pbd, pbu)
        if not hasattr(V_l, "data_ptr"):
            self.ctx.synchronize()      # host source: finished before it goes out of scope

    def form(self) -> int:
        """2 for a two-half set, 1 for a paired set."""
        h = ctypes.c_int()
        _lib.call("scw_sep_form", self.handle, ctypes.byref(h))
        return h.value

    def host_block_shape(self):
        """Shape of the amplitude array the host-buffer evaluations take: [Z, 2, 3, MF, J] for a
        two-half set, [Z, 3, MF, J] for a paired set."""
        M0, M1, Z, J = self.info()
        return (Z, 2, 3, M0 * M1, J) if self.form() == 2 else (Z, 3, M0 * M1, J)

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

    def grid(self):
        """(kx [M0], ky [M1], z boundaries [Z + 1]) of the set."""
        M0, M1, Z, _ = self.info()
        kx, ky, zb = np.zeros(M0), np.zeros(M1), np.zeros(Z + 1)
        _lib.call("scw_sep_get_grid", self.handle, *(ctypes.c_void_p(a.ctypes.data) for a in (kx, ky, zb)))
        return kx, ky, zb

    def set_region_rule(self, rule: int):
        _lib.call("scw_sep_set_region_rule", self.handle, int(rule))

    def eval_volume_device(self, x_start, y_start, z_start, dx, dy, dz, Nx, Ny, Nz, dE_ptr: int, method=FP32):
        _lib.call("scw_sep_eval_volume_device", self.handle, x_start, y_start, z_start, dx, dy, dz, int(Nx), int(Ny),
                  int(Nz), ctypes.c_void_p(dE_ptr), int(method))

    def eval_volume_host(self, Q_host, x_start, y_start, z_start, dx, dy, dz, Nx, Ny, Nz, out=None,
                         method=TF32X3):
        """End-to-end volume evaluation from HOST amplitudes (``scw_sep_eval_volume_host``):
        ``Q_host`` (:meth:`host_block_shape`: [Z, 2, 3, MF, J] for a two-half set, [Z, 3, MF, J]
        for a paired set; complex64 numpy array or CPU torch tensor, page-locked for full link
        speed) is uploaded slice by slice while earlier slices are evaluated, and the
        planes come back into ``out`` ([Nz, Ny, Nx, 3] complex64 host array or CPU tensor,
        allocated when None) as they finish.  Returns ``out``."""
        M0, M1, Z, J = self.info()
        shape = self.host_block_shape()
        if tuple(Q_host.shape) != shape:
            raise ValueError(f"Q_host must be {shape}, got {tuple(Q_host.shape)}")
        qptr = _host_ptr(Q_host, "Q_host")
        if out is None:
            out = np.empty((Nz, Ny, Nx, 3), np.complex64)
        if tuple(out.shape) != (Nz, Ny, Nx, 3):
            raise ValueError("out must be [Nz, Ny, Nx, 3]")
        optr = _host_ptr(out, "out")
        _lib.call("scw_sep_eval_volume_host", self.handle, ctypes.c_void_p(qptr), x_start, y_start, z_start, dx, dy,
                  dz, int(Nx), int(Ny), int(Nz), ctypes.c_void_p(optr), int(method))
        return out

    def eval_slab_device(self, x_start, y_start, z_start, dx, dy, dz, Nx, Ny, k_begin, k_end, dE_ptr: int,
                         method=TF32X3):
        """Planes ``k_begin .. k_end-1`` of the volume (same z-values as the whole volume) into
        device memory [k_end - k_begin, Ny, Nx, 3] (``scw_sep_eval_slab_device``)."""
        _lib.call("scw_sep_eval_slab_device", self.handle, x_start, y_start, z_start, dx, dy, dz, int(Nx), int(Ny),
                  int(k_begin), int(k_end), ctypes.c_void_p(dE_ptr), int(method))

    def eval_slab_host(self, Q_host, x_start, y_start, z_start, dx, dy, dz, Nx, Ny, k_begin, k_end, out=None,
                       method=TF32X3):
        """Host-buffer form of :meth:`eval_slab_device` (``scw_sep_eval_slab_host``): only the
        slices the slab's planes lie in are read from ``Q_host`` [Z, 2, 3, MF, J]."""
        if tuple(Q_host.shape) != self.host_block_shape():
            raise ValueError(f"Q_host must be {self.host_block_shape()}, got {tuple(Q_host.shape)}")
        n = int(k_end) - int(k_begin)
        if out is None:
            out = np.empty((n, Ny, Nx, 3), np.complex64)
        if tuple(out.shape) != (n, Ny, Nx, 3):
            raise ValueError("out must be [k_end - k_begin, Ny, Nx, 3]")
        _lib.call("scw_sep_eval_slab_host", self.handle, ctypes.c_void_p(_host_ptr(Q_host, "Q_host")), x_start,
                  y_start, z_start, dx, dy, dz, int(Nx), int(Ny), int(k_begin), int(k_end),
                  ctypes.c_void_p(_host_ptr(out, "out")), int(method))
        return out

    def set_pipeline(self, chunks: int = 0, synth_sm_div: int = 2):
        """Overlapped stages of device slabs (``scw_sep_set_pipeline``); 0 or 1 chunk: one pass."""
        _lib.call("scw_sep_set_pipeline", self.handle, int(chunks), int(synth_sm_div))

    def set_tiles(self, ctr_shape: int = 0):
        """Contraction tile shape (``scw_sep_set_tiles``): 0 = default rows per warp, 1 = half."""
        _lib.call("scw_sep_set_tiles", self.handle, int(ctr_shape))

    def set_streaming(self, chunk_bytes: int = 0, slab_bytes: int = 0):
        """Upload chunk (Q bytes, whole slices) and read-back slab (output bytes, whole planes)
        of :meth:`eval_volume_host`; 0 keeps the defaults (192 MiB, 64 MiB)."""
        _lib.call("scw_sep_set_streaming", self.handle, ctypes.c_int64(chunk_bytes), ctypes.c_int64(slab_bytes))

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
