"""Host-side mirror of ``CoupledWaveStructure<double>`` (CoupledWaveStructure.h:57-147).

Waves are numpy arrays of shape ``[n, 6]`` complex128 (E0x, E0y, E0z, kx, ky, kz), the
record order of the .cw format.  ``save``/``load``/``getPlaneIndex`` go through the
native library (``scw_cw_save`` / ``scw_cw_load`` / ``scw_cw_get_plane_index``).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib


def _as_records(w) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(w, dtype=np.complex128).reshape(-1, 6))
    return a


def planewave(kx, ky, kz, Ex, Ey, Ez) -> np.ndarray:
    """One record built like ``tira::planewave<double>(kx, ky, kz, Ex, Ey, Ez)``."""
    return np.array([[Ex, Ey, Ez, kx, ky, kz]], dtype=np.complex128)


@dataclass
class HomogeneousLayer:
    """CoupledWaveStructure.h:57-62."""
    z: float = 0.0
    Pr: np.ndarray = field(default_factory=lambda: np.zeros((0, 6), np.complex128))
    Pt: np.ndarray = field(default_factory=lambda: np.zeros((0, 6), np.complex128))


class CoupledWaveStructure:
    """CoupledWaveStructure<double> (CoupledWaveStructure.h:64-148)."""

    def __init__(self):
        self.Pi = np.zeros((0, 6), dtype=np.complex128)
        self.Layers: list[HomogeneousLayer] = []

    # -- native handle ----------------------------------------------------------------
    def _to_native(self):
        h = ctypes.c_void_p()
        _lib.call("scw_cw_create", ctypes.byref(h))
        try:
            pi = _as_records(self.Pi)
            _lib.call("scw_cw_set_incident", h, len(pi), pi.ctypes.data_as(ctypes.c_void_p))
            _lib.call("scw_cw_set_layer_count", h, len(self.Layers))
            for l, L in enumerate(self.Layers):
                pr, pt = _as_records(L.Pr), _as_records(L.Pt)
                _lib.call("scw_cw_set_layer", h, l, float(L.z), len(pr), pr.ctypes.data_as(ctypes.c_void_p),
                          len(pt), pt.ctypes.data_as(ctypes.c_void_p))
        except Exception:
            _lib.load().scw_cw_destroy(h)
            raise
        return h

    @classmethod
    def _from_native(cls, h) -> "CoupledWaveStructure":
        out = cls()
        npi, nl = ctypes.c_int64(), ctypes.c_int64()
        _lib.call("scw_cw_counts", h, ctypes.byref(npi), ctypes.byref(nl))
        out.Pi = np.zeros((npi.value, 6), dtype=np.complex128)
        _lib.call("scw_cw_get_incident", h, out.Pi.ctypes.data_as(ctypes.c_void_p))
        for l in range(nl.value):
            z, npr, npt = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int64()
            _lib.call("scw_cw_layer_counts", h, l, ctypes.byref(z), ctypes.byref(npr), ctypes.byref(npt))
            L = HomogeneousLayer(z=z.value, Pr=np.zeros((npr.value, 6), np.complex128),
                                 Pt=np.zeros((npt.value, 6), np.complex128))
            _lib.call("scw_cw_get_layer", h, l, L.Pr.ctypes.data_as(ctypes.c_void_p),
                      L.Pt.ctypes.data_as(ctypes.c_void_p))
            out.Layers.append(L)
        return out

    # -- reference API ----------------------------------------------------------------
    def save(self, filename: str) -> None:
        h = self._to_native()
        try:
            _lib.call("scw_cw_save", h, str(filename).encode())
        finally:
            _lib.load().scw_cw_destroy(h)

    def load(self, filename: str) -> bool:
        """Returns False if the file cannot be opened (CoupledWaveStructure.h:104-105);
        raises ScwError for a truncated or inconsistent file."""
        h = ctypes.c_void_p()
        st = _lib.load().scw_cw_load(str(filename).encode(), ctypes.byref(h))
        if st == 2:  # SCW_ERR_IO
            return False
        _lib.check(st)
        try:
            other = CoupledWaveStructure._from_native(h)
        finally:
            _lib.load().scw_cw_destroy(h)
        self.Pi, self.Layers = other.Pi, other.Layers
        return True

    def getPlaneIndex(self, z: float) -> int:  # noqa: N802 (reference name)
        h = self._to_native()
        try:
            idx = ctypes.c_int64()
            _lib.call("scw_cw_get_plane_index", h, float(z), ctypes.byref(idx))
            return idx.value
        finally:
            _lib.load().scw_cw_destroy(h)

    # -- conveniences -----------------------------------------------------------------
    def total_waves(self) -> int:
        return len(self.Pi) + sum(len(L.Pr) + len(L.Pt) for L in self.Layers)
