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
"""
from __future__ import annotations

import numpy as np


def spheres(shape=(20, 64, 64), n_spheres=6, radius=(4.0, 12.0), n_sphere=1.4 + 0.01j,
            n_background=1.0, seed=0):
    Z, Y, X = shape
    rng = np.random.default_rng(seed)
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    vol = np.full(shape, n_background, dtype=np.complex128)
    for _ in range(n_spheres):
        c = rng.uniform([0, 0, 0], [Z, Y, X])
        r = rng.uniform(radius[0], radius[1])
        m = (zz - c[0]) ** 2 + (yy - c[1]) ** 2 + (xx - c[2]) ** 2 <= r * r
        vol[m] = n_sphere
    return vol


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
