"""Host-side mirror of the reference evaluator interface (cpuEvaluator.h / gpuEvaluator.h).

Reference names and meanings are kept:

* module globals ``layers, z_layers, waves_begin, waves_end, W`` (cpuEvaluator.cpp:3-7),
* ``cw_allocate(cw)`` / ``cw_unpack(cw)`` (cpuEvaluator.cpp:34-102),
* ``gpu_initialize()`` (gpuEvaluator.cu:15-26): uploads the globals to the GPU,
* ``gpu_cw_evaluate(E_xy, E_xz, E_yz, x_start, y_start, z_start, x, y, z, d, N, device)``
  (gpuEvaluator.cu:131-165): fills three caller-owned host arrays of N*N*3 complex64.

All compute runs in the native CUDA library; if it is missing or no GPU is present the
calls raise -- there is no CPU fallback.  :class:`Context` and :class:`WaveSet` expose the
device-memory entry points (planes and volumes written straight to GPU buffers).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .cw import CoupledWaveStructure

# cpuEvaluator.cpp:3-7
layers: int = 0
z_layers = np.zeros(0, dtype=np.float32)
waves_begin = np.zeros(0, dtype=np.int32)
waves_end = np.zeros(0, dtype=np.int32)
W = np.zeros((0, 6), dtype=np.complex64)

REGION_RULE_GPU = 0   # z >= z_l - 0.001 (gpuEvaluator.cu:34)
REGION_RULE_CPU = 1   # z >= z_l        (cpuEvaluator.cpp:303)


def _vp(a):
    return ctypes.c_void_p(a.ctypes.data) if isinstance(a, np.ndarray) else ctypes.c_void_p(int(a))


class Context:
    """One CUDA device and one stream (``scw_ctx``)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.device = device
        self.handle = ctypes.c_void_p()
        _lib.call("scw_ctx_create", device, ctypes.c_void_p(stream) if stream else None, ctypes.byref(self.handle))

    def synchronize(self):
        _lib.call("scw_ctx_synchronize", self.handle)

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        _lib.call("scw_ctx_stream", self.handle, ctypes.byref(s))
        return s.value or 0

    @property
    def launches(self) -> int:
        n = ctypes.c_int64()
        _lib.call("scw_ctx_launch_count", self.handle, ctypes.byref(n))
        return n.value

    def set_timing(self, on: bool = True):
        _lib.call("scw_ctx_set_timing", self.handle, 1 if on else 0)

    def timing_report(self) -> dict:
        """{kernel name: (total ms, launches)} since the last report (synchronises)."""
        names = ctypes.create_string_buffer(4096)
        ms = (ctypes.c_double * 64)()
        cnt = (ctypes.c_int64 * 64)()
        n = ctypes.c_int()
        _lib.call("scw_ctx_timing_report", self.handle, names, 4096, ms, cnt, 64, ctypes.byref(n))
        keys = names.value.decode().split("\n")[: n.value]
        return {k: (ms[i], cnt[i]) for i, k in enumerate(keys)}

    def close(self):
        if self.handle:
            _lib.load().scw_ctx_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WaveSet:
    """Device-resident unpacked waves (``scw_waves``)."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle

    @classmethod
    def from_unpacked(cls, ctx: Context, layers_: int, z_layers_, begin, end, W_) -> "WaveSet":
        zl = np.ascontiguousarray(z_layers_, dtype=np.float32)
        b = np.ascontiguousarray(begin, dtype=np.int32)
        e = np.ascontiguousarray(end, dtype=np.int32)
        w = np.ascontiguousarray(W_, dtype=np.complex64).reshape(-1, 6)
        h = ctypes.c_void_p()
        _lib.call("scw_gpu_initialize", ctx.handle, int(layers_), _vp(zl), _vp(b), _vp(e), _vp(w), len(w),
                  ctypes.byref(h))
        return cls(ctx, h)

    @classmethod
    def from_cw(cls, ctx: Context, cw: CoupledWaveStructure) -> "WaveSet":
        native = cw._to_native()
        try:
            h = ctypes.c_void_p()
            _lib.call("scw_gpu_initialize_cw", ctx.handle, native, ctypes.byref(h))
        finally:
            _lib.load().scw_cw_destroy(native)
        return cls(ctx, h)

    def set_region_rule(self, rule: int):
        _lib.call("scw_waves_set_region_rule", self.handle, int(rule))

    def evaluate_planes_host(self, x_start, y_start, z_start, x, y, z, d, N):
        """gpu_cw_evaluate into freshly allocated host arrays; returns (E_xy, E_xz, E_yz) [N, N, 3]."""
        outs = [np.empty((N, N, 3), dtype=np.complex64) for _ in range(3)]
        _lib.call("scw_gpu_cw_evaluate", self.handle, _vp(outs[0]), _vp(outs[1]), _vp(outs[2]),
                  x_start, y_start, z_start, x, y, z, d, int(N), int(self.ctx.device))
        return tuple(outs)

    def eval_plane_device(self, axis: int, a_start, b_start, c, d, N, dE_ptr: int):
        _lib.call("scw_eval_plane_device", self.handle, int(axis), a_start, b_start, c, d, int(N),
                  ctypes.c_void_p(dE_ptr))

    def eval_volume_device(self, x_start, y_start, z_start, dx, dy, dz, Nx, Ny, Nz, dE_ptr: int):
        _lib.call("scw_eval_volume_device", self.handle, x_start, y_start, z_start, dx, dy, dz, int(Nx), int(Ny),
                  int(Nz), ctypes.c_void_p(dE_ptr))

    def close(self):
        if self.handle:
            _lib.load().scw_waves_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------------------------------
# Reference-named functions
# ------------------------------------------------------------------------------------------
_ctx: Context | None = None
_waves: WaveSet | None = None


def cw_allocate(cw: CoupledWaveStructure) -> None:
    """cpuEvaluator.cpp:34-53: sets ``layers``, ``z_layers``, region offsets, sizes ``W``."""
    global layers, z_layers, waves_begin, waves_end, W
    native = cw._to_native()
    try:
        nl, total = ctypes.c_int(), ctypes.c_int64()
        _lib.call("scw_cw_allocate", native, ctypes.byref(nl), ctypes.byref(total))
    finally:
        _lib.load().scw_cw_destroy(native)
    layers = nl.value
    z_layers = np.zeros(layers, dtype=np.float32)
    waves_begin = np.zeros(layers + 1, dtype=np.int32)
    waves_end = np.zeros(layers + 1, dtype=np.int32)
    W = np.zeros((total.value, 6), dtype=np.complex64)


def cw_unpack(cw: CoupledWaveStructure) -> None:
    """cpuEvaluator.cpp:61-102: fills ``W`` (double -> float) and the region offsets."""
    global W
    native = cw._to_native()
    try:
        _lib.call("scw_cw_unpack", native, _vp(W), _vp(waves_begin), _vp(waves_end), _vp(z_layers))
    finally:
        _lib.load().scw_cw_destroy(native)


def gpu_initialize(device: int = 0) -> None:
    """gpuEvaluator.cu:15-26: copies the unpacked globals to the GPU."""
    global _ctx, _waves
    if _ctx is None or _ctx.device != device:
        _ctx = Context(device)
    if _waves is not None:
        _waves.close()
    _waves = WaveSet.from_unpacked(_ctx, layers, z_layers, waves_begin, waves_end, W)


def gpu_cw_evaluate(E_xy: np.ndarray, E_xz: np.ndarray, E_yz: np.ndarray, x_start: float, y_start: float,
                    z_start: float, x: float, y: float, z: float, d: float, N: int, device: int) -> None:
    """gpuEvaluator.cu:131-165: evaluates the xy plane at ``z``, the xz plane at ``y`` and the
    yz plane at ``x`` into the caller's complex64 arrays (N*N*3 each)."""
    if _waves is None:
        raise RuntimeError("gpu_cw_evaluate called before gpu_initialize")
    for a in (E_xy, E_xz, E_yz):
        if not (isinstance(a, np.ndarray) and a.dtype == np.complex64 and a.size == N * N * 3
                and a.flags["C_CONTIGUOUS"]):
            raise ValueError("outputs must be C-contiguous complex64 arrays of N*N*3 elements")
    _lib.call("scw_gpu_cw_evaluate", _waves.handle, _vp(E_xy), _vp(E_xz), _vp(E_yz), x_start, y_start, z_start,
              x, y, z, d, int(N), int(device))
