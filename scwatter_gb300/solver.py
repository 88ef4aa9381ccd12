"""Per-layer coupled-wave solve on the GPU -- the computation of the reference program
``sCWatter`` (sCWatter.cpp:500-956), with its options as keyword arguments:

==============  =====================  ====================================
sCWatter flag   keyword                meaning
==============  =====================  ====================================
--lambda        ``lam``                vacuum wavelength (default 1.0)
--direction     ``direction``          incident direction (default 0 0 1)
--ex/--ey/--ez  ``ex``, ``ey``, ``ez`` incident field (re, im); default ey = (1, 0)
--n             ``n``                  real index of the upper / lower medium
--kappa         ``kappa``              absorbance of the lower medium
--size          ``size``               sample extent x, y, z (default 10 10 2)
--z             ``z``                  sample centre along z
--coef          ``coef``               harmonics along x, y (None: the sample's X, Y)
--external      ``external``           keep only the exterior waves
--npz           ``pz=False``           skip the Ez rows of the modes
--psf           ``psf``                every harmonic carries the incident field
==============  =====================  ====================================

The whole solve runs in the native library on the GPU (FP64); there is no CPU path.
``python -m scwatter_gb300.scwatter`` is the command-line front end.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .cw import CoupledWaveStructure
from .evaluator import Context
from .separable import SeparableSet


class _Params(ctypes.Structure):
    _fields_ = [("lam", ctypes.c_double), ("direction", ctypes.c_double * 3), ("ex", ctypes.c_double * 2),
                ("ey", ctypes.c_double * 2), ("ez", ctypes.c_double * 2), ("n", ctypes.c_double * 2),
                ("kappa", ctypes.c_double), ("size", ctypes.c_double * 3), ("z", ctypes.c_double),
                ("coef", ctypes.c_int * 2), ("external", ctypes.c_int), ("pz", ctypes.c_int), ("psf", ctypes.c_int),
                ("eig_fp64", ctypes.c_int)]


def _params(lam, direction, ex, ey, ez, n, kappa, size, z, coef, external, pz, psf=False, eig_fp64=False) -> _Params:
    p = _Params()
    p.lam = float(lam)
    p.direction[:] = [float(v) for v in direction]
    p.ex[:] = [float(v) for v in ex]
    p.ey[:] = [float(v) for v in ey]
    p.ez[:] = [float(v) for v in ez]
    if len(n) != 2:
        raise ValueError("the volume solver takes exactly two media (upper, lower)")
    p.n[:] = [float(v) for v in n]
    p.kappa = float(kappa[0] if isinstance(kappa, (list, tuple)) else kappa)
    p.size[:] = [float(v) for v in size]
    p.z = float(z)
    if coef is None or len(coef) == 0:
        p.coef[:] = [0, 0]
    elif len(coef) == 1:                     # sCWatter.cpp:598-600: one value = total count
        m = int(np.sqrt(coef[0]))
        p.coef[:] = [m, m]
    else:
        p.coef[:] = [int(coef[0]), int(coef[1])]
    p.external = 1 if external else 0
    p.pz = 1 if pz else 0
    p.psf = 1 if psf else 0
    p.eig_fp64 = 1 if eig_fp64 else 0
    return p


class Solution:
    """Result of one solve (``scw_solution``), resident on the GPU."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle
        M0, M1, Z, k = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _lib.call("scw_solution_info", handle, ctypes.byref(M0), ctypes.byref(M1), ctypes.byref(Z), ctypes.byref(k))
        self.M = (M0.value, M1.value)
        self.MF = M0.value * M1.value
        self.Z = Z.value
        self.k = k.value
        MF = self.MF
        self.gamma = np.zeros((self.Z, 2 * MF), np.complex128)
        self.x = np.zeros(6 * MF, np.complex128)
        self.EF = np.zeros(3 * MF, np.complex128)
        self.z = np.zeros(self.Z + 1)
        _lib.call("scw_solution_get", handle, *(ctypes.c_void_p(a.ctypes.data) for a in
                                                (self.gamma, self.x, self.EF, self.z)))
        mixed, acc, steps, res, checks = (ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double(),
                                          ctypes.c_int())
        _lib.call("scw_solution_eig_info", handle, ctypes.byref(mixed), ctypes.byref(acc), ctypes.byref(steps),
                  ctypes.byref(res), ctypes.byref(checks))
        # eigen-solver record: mixed path on / slices it finished / most steps / largest residual /
        # FP64 residual GEMMs issued
        self.eig = {"mixed": bool(mixed.value), "accepted": acc.value, "fell_back": self.Z - acc.value if mixed.value
                    else self.Z, "max_steps": steps.value, "max_residual": res.value,
                    "residual_checks": checks.value}

    def eig_slices(self):
        """Per-slice record of the mixed eigen-solver: (state, steps, residual) arrays, state 1 =
        refined result accepted, else the fallback's reason code; None when the FP64 solver ran."""
        if not self.eig["mixed"]:
            return None
        st, steps, res = np.zeros(self.Z, np.int32), np.zeros(self.Z, np.int32), np.zeros(self.Z)
        _lib.call("scw_solution_eig_slices", self.handle, *(ctypes.c_void_p(a.ctypes.data) for a in (st, steps, res)))
        return st, steps, res

    def modes(self, l: int):
        """(Q_check, Q_hat) of slice ``l``: [3MF, 2MF] complex128 each."""
        qc = np.zeros((3 * self.MF, 2 * self.MF), np.complex128)
        qh = np.zeros_like(qc)
        _lib.call("scw_solution_get_modes", self.handle, int(l), ctypes.c_void_p(qc.ctypes.data),
                  ctypes.c_void_p(qh.ctypes.data))
        return qc, qh

    def to_cw(self) -> CoupledWaveStructure:
        h = ctypes.c_void_p()
        _lib.call("scw_solution_to_cw", self.handle, ctypes.byref(h))
        try:
            return CoupledWaveStructure._from_native(h)
        finally:
            _lib.load().scw_cw_destroy(h)

    def save(self, filename: str) -> None:
        """Writes the .cw file sCWatter would write (sCWatter.cpp:956), streamed layer by layer."""
        _lib.call("scw_solution_write_cw", self.handle, str(filename).encode())

    def to_sep(self) -> SeparableSet:
        h = ctypes.c_void_p()
        _lib.call("scw_solution_to_sep", self.handle, ctypes.byref(h))
        return SeparableSet(self.ctx, h)

    def close(self):
        if self.handle:
            _lib.load().scw_solution_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve(sample, lam=1.0, direction=(0.0, 0.0, 1.0), ex=(0.0, 0.0), ey=(1.0, 0.0), ez=(0.0, 0.0), n=(1.0, 1.0),
          kappa=0.0, size=(10.0, 10.0, 2.0), z=0.0, coef=None, external=False, pz=True, psf=False,
          ctx: Context | None = None, eig_fp64=False) -> Solution:
    """Solves the sample (``[Z, Y, X]`` or ``[Y, X]`` complex refractive index) on the GPU.
    The sample is a numpy array or a complex128 CUDA tensor (then it never leaves the device).

    ``eig_fp64``: eigen-solve every slice with the FP64 Householder + QR solver instead of the
    default FP32 factorisation refined to FP64 residuals."""
    ctx = ctx or Context(0)
    prm = _params(lam, direction, ex, ey, ez, n, kappa, size, z, coef, external, pz, psf, eig_fp64)
    h = ctypes.c_void_p()
    if hasattr(sample, "data_ptr") and getattr(sample, "is_cuda", False):
        import torch
        vol = sample.contiguous()
        if vol.dtype != torch.complex128:
            raise ValueError("a device sample must be complex128")
        if vol.dim() == 2:
            vol = vol[None]
        Z, Y, X = vol.shape
        torch.cuda.synchronize()
        ptr = ctypes.c_void_p(vol.data_ptr())
    else:
        vol = np.ascontiguousarray(sample, dtype=np.complex128)
        if vol.ndim == 2:
            vol = vol[None]
        if vol.ndim != 3:
            raise ValueError("sample must be [Z, Y, X] or [Y, X]")
        Z, Y, X = vol.shape
        ptr = ctypes.c_void_p(vol.ctypes.data)
    _lib.call("scw_solve", ctx.handle, ptr, Z, Y, X, ctypes.byref(prm), ctypes.byref(h))
    return Solution(ctx, h)
