"""Seeded synthetic samples (complex refractive-index volumes ``[Z, Y, X]``).

The reference's own sample script (``tilesample.py``) needs scikit-image; these
generators produce inputs with the shapes and value ranges the workloads are quoted on:

* :func:`spheres` -- background index 1.0 with randomly placed spheres of index
  1.4 + 0.01i (radius 4-12 px), the sphere workload at ``[20, 64, 64]`` and
  ``[64, 128, 128]``.
* :func:`gaussian_random_field` -- smoothly varying index (FFT-filtered white noise,
  Gaussian correlation length in px) mapped affinely to ``n in [n_lo, n_hi]`` with an
  absorption ``kappa`` in ``[0, kappa_max]``.
* :func:`slab` -- a homogeneous slab (known-answer tests).

Device versions write the volume straight into GPU memory (a torch complex128 CUDA tensor):
:func:`spheres_device` (the same volume as :func:`spheres` for the same seed),
:func:`grf_device` (the device generator's own counter-based noise stream, see
``scw_gen_grf``) and :func:`npy_to_device` (a .npy volume streamed from the file).
"""
from __future__ import annotations

import numpy as np


def sphere_params(shape, n_spheres=6, radius=(4.0, 12.0), seed=0) -> np.ndarray:
    """[n_spheres, 4] (cz, cy, cx, r) in voxel units, centres uniform in the volume."""
    Z, Y, X = shape
    rng = np.random.default_rng(seed)
    out = np.zeros((n_spheres, 4))
    for s in range(n_spheres):
        out[s, :3] = rng.uniform([0, 0, 0], [Z, Y, X])
        out[s, 3] = rng.uniform(radius[0], radius[1])
    return out


def spheres(shape=(20, 64, 64), n_spheres=6, radius=(4.0, 12.0), n_sphere=1.4 + 0.01j,
            n_background=1.0, seed=0):
    Z, Y, X = shape
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    vol = np.full(shape, n_background, dtype=np.complex128)
    for cz, cy, cx, r in sphere_params(shape, n_spheres, radius, seed):
        m = (zz - cz) ** 2 + (yy - cy) ** 2 + (xx - cx) ** 2 <= r * r
        vol[m] = n_sphere
    return vol


def _c2(v):
    import ctypes
    v = complex(v)
    return (ctypes.c_double * 2)(v.real, v.imag)


def spheres_device(ctx, shape=(20, 64, 64), n_spheres=6, radius=(4.0, 12.0), n_sphere=1.4 + 0.01j,
                   n_background=1.0, seed=0):
    """:func:`spheres` generated on the device (``scw_gen_spheres``): the same volume."""
    import ctypes
    import torch
    from . import _lib
    Z, Y, X = shape
    prm = np.ascontiguousarray(sphere_params(shape, n_spheres, radius, seed))
    out = torch.empty(shape, dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    _lib.call("scw_gen_spheres", ctx.handle, Z, Y, X, n_spheres, ctypes.c_void_p(prm.ctypes.data), _c2(n_background),
              _c2(n_sphere), ctypes.c_void_p(out.data_ptr()))
    return out


def grf_device(ctx, shape=(32, 64, 64), corr_px=8.0, n_range=(1.0, 1.6), kappa_max=0.02, seed=0):
    """Gaussian random field generated on the device (``scw_gen_grf``)."""
    import ctypes
    import torch
    from . import _lib
    Z, Y, X = shape
    out = torch.empty(shape, dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    _lib.call("scw_gen_grf", ctx.handle, Z, Y, X, float(corr_px), float(n_range[0]), float(n_range[1]),
              float(kappa_max), int(seed) & (2 ** 64 - 1), ctypes.c_void_p(out.data_ptr()))
    return out


def npy_shape(path) -> tuple:
    """(Z, Y, X) of a 2-D or 3-D complex128 / float64 .npy volume, from its header alone."""
    import ctypes
    from . import _lib
    d = (ctypes.c_int * 3)()
    _lib.call("scw_npy_read", None, str(path).encode(), d, None)
    return tuple(d)


def npy_to_device(ctx, path):
    """A .npy volume streamed from the file into a complex128 CUDA tensor [Z, Y, X]."""
    import ctypes
    import torch
    from . import _lib
    shape = npy_shape(path)
    out = torch.empty(shape, dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    _lib.call("scw_npy_read", ctx.handle, str(path).encode(), (ctypes.c_int * 3)(), ctypes.c_void_p(out.data_ptr()))
    return out


def gaussian_random_field(shape=(32, 64, 64), corr_px=8.0, n_range=(1.0, 1.6), kappa_max=0.02, seed=0):
    Z, Y, X = shape
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(shape)
    fz = np.fft.fftfreq(Z)[:, None, None]
    fy = np.fft.fftfreq(Y)[None, :, None]
    fx = np.fft.fftfreq(X)[None, None, :]
    # Gaussian kernel exp(-r^2 / (2 l^2)) has transfer exp(-2 pi^2 l^2 f^2)
    H = np.exp(-2.0 * np.pi ** 2 * corr_px ** 2 * (fx ** 2 + fy ** 2 + fz ** 2))
    g = np.real(np.fft.ifftn(np.fft.fftn(noise) * H))
    g = (g - g.min()) / max(g.max() - g.min(), 1e-30)
    n = n_range[0] + (n_range[1] - n_range[0]) * g
    kappa = rng.uniform(0.0, kappa_max)
    return (n + 1j * kappa * g).astype(np.complex128)


def slab(shape=(1, 8, 8), n=1.5 + 0.0j):
    return np.full(shape, n, dtype=np.complex128)
