"""Batched solve + evaluate (``scw_batch``): many samples of uneven harmonic counts, layer
counts and grids, solved in FP64 and evaluated with the separable evaluator, all captured in
one CUDA graph and launched with one call.

    items = [BatchItem(sample, grid=(x0, y0, z0, dx, dy, dz, Nx, Ny, Nz), coef=(8, 12), lam=0.9), ...]
    b = Batch(ctx, items)          # plans, uploads, autotunes, captures
    b.run(); b.wait()
    x, gamma, field = b.result(0)
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field as dfield

import numpy as np

from . import _lib
from .evaluator import Context
from .solver import _Params, _params


class _Item(ctypes.Structure):
    _fields_ = [("sample", ctypes.c_void_p), ("Z", ctypes.c_int), ("Y", ctypes.c_int), ("X", ctypes.c_int),
                ("prm", _Params), ("x0", ctypes.c_float), ("y0", ctypes.c_float), ("z0", ctypes.c_float),
                ("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float), ("Nx", ctypes.c_int),
                ("Ny", ctypes.c_int), ("Nz", ctypes.c_int)]


@dataclass
class BatchItem:
    """One sample with the solve options of :func:`scwatter_gb300.solver.solve` and its
    evaluation grid ``(x0, y0, z0, dx, dy, dz, Nx, Ny, Nz)``."""
    sample: np.ndarray
    grid: tuple
    lam: float = 1.0
    direction: tuple = (0.0, 0.0, 1.0)
    ex: tuple = (0.0, 0.0)
    ey: tuple = (1.0, 0.0)
    ez: tuple = (0.0, 0.0)
    n: tuple = (1.0, 1.0)
    kappa: float = 0.0
    size: tuple = (10.0, 10.0, 2.0)
    z: float = 0.0
    coef: tuple | None = None
    external: bool = False
    pz: bool = True
    psf: bool = False
    extra: dict = dfield(default_factory=dict)


class Batch:
    def __init__(self, ctx: Context, items, lanes: int = 0, method: int = 0):
        self.ctx = ctx
        self.items = list(items)
        self._arrays = []
        arr = (_Item * len(self.items))()
        for i, it in enumerate(self.items):
            vol = np.ascontiguousarray(it.sample, dtype=np.complex128)
            if vol.ndim == 2:
                vol = vol[None]
            self._arrays.append(vol)
            a = arr[i]
            a.sample = vol.ctypes.data
            a.Z, a.Y, a.X = vol.shape
            a.prm = _params(it.lam, it.direction, it.ex, it.ey, it.ez, it.n, it.kappa, it.size, it.z, it.coef,
                            it.external, it.pz, it.psf)
            x0, y0, z0, dx, dy, dz, Nx, Ny, Nz = it.grid
            a.x0, a.y0, a.z0, a.dx, a.dy, a.dz = float(x0), float(y0), float(z0), float(dx), float(dy), float(dz)
            a.Nx, a.Ny, a.Nz = int(Nx), int(Ny), int(Nz)
        self.handle = ctypes.c_void_p()
        _lib.call("scw_batch_create", ctx.handle, arr, len(self.items), int(lanes), int(method),
                  ctypes.byref(self.handle))
        self._arrays = []          # the samples were uploaded during create

    def run(self):
        _lib.call("scw_batch_run", self.handle)

    def wait(self) -> np.ndarray:
        st = np.zeros(len(self.items), np.int32)
        _lib.call("scw_batch_wait", self.handle, ctypes.c_void_p(st.ctypes.data))
        return st

    def item_info(self, i: int):
        M0, M1, Z, pm = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int64()
        _lib.call("scw_batch_item_info", self.handle, int(i), ctypes.byref(M0), ctypes.byref(M1), ctypes.byref(Z),
                  ctypes.byref(pm))
        return M0.value, M1.value, Z.value, pm.value

    def item_eig(self, i: int) -> dict:
        """The mixed eigen-solver's record of item ``i`` after a run (as ``Solution.eig``)."""
        mixed, acc, steps, res, checks = (ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double(),
                                          ctypes.c_int())
        _lib.call("scw_batch_item_eig", self.handle, int(i), ctypes.byref(mixed), ctypes.byref(acc),
                  ctypes.byref(steps), ctypes.byref(res), ctypes.byref(checks))
        Z = self.item_info(i)[2]
        return {"mixed": bool(mixed.value), "accepted": acc.value,
                "fell_back": Z - acc.value if mixed.value else Z, "max_steps": steps.value,
                "max_residual": res.value, "residual_checks": checks.value}

    def item_eig_slices(self, i: int):
        """Per slice of item ``i`` after a run: (state, steps, residual) as ``Solution.eig_slices``
        (state 1 = accepted by the mixed path, else the fallback's reason code)."""
        Z = self.item_info(i)[2]
        st, steps, res = np.zeros(Z, np.int32), np.zeros(Z, np.int32), np.zeros(Z, np.float64)
        _lib.call("scw_batch_item_eig_slices", self.handle, int(i), *(ctypes.c_void_p(a.ctypes.data) for a in (st, steps, res)))
        return st, steps, res

    def result(self, i: int):
        """(x [6MF], gamma [Z, 2MF], field [Nz, Ny, Nx, 3] complex64) of item ``i``."""
        M0, M1, Z, _ = self.item_info(i)
        MF = M0 * M1
        Nx, Ny, Nz = self.items[i].grid[6:9]
        x = np.zeros(6 * MF, np.complex128)
        g = np.zeros((Z, 2 * MF), np.complex128)
        f = np.zeros((Nz, Ny, Nx, 3), np.complex64)
        _lib.call("scw_batch_get", self.handle, int(i), ctypes.c_void_p(x.ctypes.data), ctypes.c_void_p(g.ctypes.data),
                  ctypes.c_void_p(f.ctypes.data), None)
        return x, g, f

    def info(self) -> dict:
        lanes, method, shape, n_tune = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        nodes, kernels = ctypes.c_int64(), ctypes.c_int64()
        tune_ms = ctypes.c_double()
        log = np.zeros(4 * 16, np.float64)
        _lib.call("scw_batch_info", self.handle, ctypes.byref(lanes), ctypes.byref(method), ctypes.byref(shape),
                  ctypes.byref(nodes), ctypes.byref(kernels), ctypes.byref(tune_ms), ctypes.c_void_p(log.ctypes.data),
                  ctypes.byref(n_tune))
        return {"lanes": lanes.value, "method": method.value, "ctr_shape": shape.value, "graph_nodes": nodes.value,
                "kernels": kernels.value, "tune_ms": tune_ms.value,
                "tune_log": [tuple(log[4 * k:4 * k + 4]) for k in range(n_tune.value)]}

    def close(self):
        if self.handle:
            _lib.load().scw_batch_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def uneven_items(count: int, seed: int = 0, m_range=(8, 32), z_range=(4, 64), grid_xy=(64, 256), grid_z=(32, 128),
                 lam_range=(0.5, 1.5), max_angle_deg=30.0, pixels=64):
    """The uneven batched workload: sphere samples ``[Z, pixels, pixels]`` (1 unit per pixel,
    background 1.0, spheres 1.4 + 0.01i), harmonics uniform in ``m_range`` per axis, layers in
    ``z_range``, evaluation grids from ``grid_xy[0]^2 x grid_z[0]`` to ``grid_xy[1]^2 x grid_z[1]``
    over x, y in [-pixels/2, pixels/2] and z in [-Z, Z], wavelengths in ``lam_range`` and
    incidence angles up to ``max_angle_deg`` (azimuth uniform); x-polarised."""
    from . import samples
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        M0, M1 = (int(v) for v in rng.integers(m_range[0], m_range[1] + 1, 2))
        Z = int(rng.integers(z_range[0], z_range[1] + 1))
        Nxy = int(rng.integers(grid_xy[0], grid_xy[1] + 1))
        Nz = int(rng.integers(grid_z[0], grid_z[1] + 1))
        lam = float(rng.uniform(*lam_range))
        th = np.deg2rad(rng.uniform(0.0, max_angle_deg))
        ph = rng.uniform(0.0, 2 * np.pi)
        d = (np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th))
        n_sph = int(rng.integers(2, 7))
        s = samples.spheres((Z, pixels, pixels), n_spheres=n_sph, radius=(4.0, 12.0), seed=seed * 100003 + i)
        h = pixels / 2
        grid = (-h, -h, -float(Z), 2 * h / (Nxy - 1), 2 * h / (Nxy - 1), 2.0 * Z / (Nz - 1), Nxy, Nxy, Nz)
        out.append(BatchItem(sample=s, grid=grid, lam=lam, direction=d, ex=(1, 0), ey=(0, 0),
                             size=(float(pixels), float(pixels), float(Z)), coef=(M0, M1)))
    return out
