"""Homogeneous multilayer solver -- the computation of the reference program sCWatterLayer
(sCWatterLayer.cpp:119-425), with its per-wave 6L x 6L systems solved in a batch on the GPU
(scw_layer_solve, one CTA per incident wave).

    python -m scwatter_gb300.layer --lambda 5 --n 1 1.4 1.4 1.0 --kappa 0.05 --z -5 0 5 --alpha 0 --output a.cw

Options and defaults follow the reference.  A single incident wave (--alpha 0, or one sample)
reproduces the reference exactly.  A focused beam needs incident-wave samplers that come from
tira (SolidAnglePolar / SolidAngleMC), which is not part of the reference sources.  Here the
polar mode places N0 x N1 directions at the midpoints of a (polar angle, azimuth) grid over the
cap between beta and alpha around the direction, and the montecarlo mode draws directions
uniformly over that cap (seeded).  Each amplitude is weighted by the cap's solid angle over the
sample count (the polar weights carry sin(theta)).  These sample sets are this package's own,
not tira's.
"""
from __future__ import annotations

import argparse
import ctypes
import sys

import numpy as np

from . import _lib
from .cw import CoupledWaveStructure, HomogeneousLayer


def _orthogonalize(e, d):
    """FourierWave.h:32-39 (the same as the volume solver's)."""
    e = np.asarray(e, complex)
    e = e / np.sqrt(np.sum(e * e))
    d = np.asarray(d, complex)
    s = np.cross(e, d)
    return np.cross(d, s)


def _wind(w, z):
    w = w.copy()
    w[:3] *= np.exp(-1j * w[5] * z)
    return w


def incident_waves(direction, e, n0, lam, alpha=0.0, beta=0.0, samples=(1, 1), mode="polar", seed=0):
    """Incident plane waves [count, 6] complex (E0 xyz, k xyz)."""
    d = np.asarray(direction, float)
    d = d / np.linalg.norm(d)
    k_vac = 2 * np.pi / lam
    N0, N1 = samples
    if alpha == 0 or N0 * N1 == 1:
        dirs, wts = [d], [1.0]
    else:
        # orthonormal frame around d
        a = np.array([1.0, 0, 0]) if abs(d[0]) < 0.9 else np.array([0, 1.0, 0])
        u = np.cross(d, a)
        u /= np.linalg.norm(u)
        v = np.cross(d, u)
        dirs, wts = [], []
        if mode == "montecarlo":
            rng = np.random.default_rng(seed)
            c0, c1 = np.cos(beta), np.cos(alpha)
            for _ in range(N0 * N1):
                ct = rng.uniform(c1, c0)
                st = np.sqrt(1 - ct * ct)
                ph = rng.uniform(0, 2 * np.pi)
                dirs.append(ct * d + st * (np.cos(ph) * u + np.sin(ph) * v))
                wts.append(1.0 / (N0 * N1))
        else:
            for i in range(N0):
                th = beta + (alpha - beta) * (i + 0.5) / N0
                for j in range(N1):
                    ph = 2 * np.pi * j / N1
                    dirs.append(np.cos(th) * d + np.sin(th) * (np.cos(ph) * u + np.sin(ph) * v))
                    wts.append(np.sin(th))
            wts = list(np.asarray(wts) / np.sum(wts))
    out = []
    for di, wi in zip(dirs, wts):
        E = _orthogonalize(e, di) * wi
        out.append(np.concatenate([E, di * n0 * k_vac]).astype(complex))
    return np.array(out)


def solve_layers(ctx, waves, n, kappa, z, lam, wavemask=(True, True, True)):
    """Returns (x [count, 6L] complex, CoupledWaveStructure) as sCWatterLayer builds it."""
    L = len(n)
    ri = np.array([complex(n[0], 0.0)] + [complex(n[l], kappa[l - 1]) for l in range(1, L)])
    zz = np.ascontiguousarray(np.asarray(z[:L - 1], float))
    W = np.ascontiguousarray(np.asarray(waves, complex).reshape(-1, 6))
    rec = np.ascontiguousarray(W.view(np.float64).reshape(-1, 12))
    count = W.shape[0]
    x = np.zeros((count, 6 * L), complex)
    info = np.zeros(count, np.int32)
    k_vac = 2 * np.pi / lam
    _lib.call("scw_layer_solve", ctx.handle, L, ctypes.c_void_p(ri.ctypes.data), ctypes.c_void_p(zz.ctypes.data),
              float(n[0]), k_vac, count, ctypes.c_void_p(rec.ctypes.data), ctypes.c_void_p(x.ctypes.data),
              ctypes.c_void_p(info.ctypes.data))
    if info.any():
        raise RuntimeError(f"{int(info.sum())} singular layer systems")
    S = CoupledWaveStructure()
    S.Pi = W.copy() if wavemask[0] else np.zeros((0, 6), complex)
    layers = [HomogeneousLayer(z=float(zz[l]), Pr=[], Pt=[]) for l in range(L - 1)]
    for p in range(count):
        kr = W[p, 3:6].real
        s = kr / np.linalg.norm(kr) * n[0]
        sz = np.sqrt(ri ** 2 - s[0] ** 2 - s[1] ** 2)
        for l in range(L - 1):
            r = np.array([x[p, l * 6 + 3], x[p, l * 6 + 4], x[p, l * 6 + 5], s[0] * k_vac, s[1] * k_vac,
                          -sz[l] * k_vac])
            t = np.array([x[p, (l + 1) * 6], x[p, (l + 1) * 6 + 1], x[p, (l + 1) * 6 + 2], s[0] * k_vac,
                          s[1] * k_vac, sz[l + 1] * k_vac])
            if wavemask[1]:
                layers[l].Pr.append(_wind(r, zz[l]))
            if wavemask[2]:
                layers[l].Pt.append(_wind(t, zz[l]))
    for L_ in layers:
        L_.Pr = np.array(L_.Pr, complex).reshape(-1, 6)
        L_.Pt = np.array(L_.Pt, complex).reshape(-1, 6)
    S.Layers = layers
    return x, S


def parser():
    p = argparse.ArgumentParser(prog="scwatterlayer", description="homogeneous multilayer solve on the GPU")
    p.add_argument("--lambda", dest="lam", type=float, default=5.0)
    p.add_argument("--direction", type=float, nargs=3, default=[1.0, 0.0, 1.0])
    p.add_argument("--ex", type=float, nargs=2, default=[1.0, 0.0])
    p.add_argument("--ey", type=float, nargs=2, default=[1.0, 0.0])
    p.add_argument("--ez", type=float, nargs=2, default=[0.0, 0.0])
    p.add_argument("--n", type=float, nargs="+", default=[1.0, 1.4, 1.4, 1.0])
    p.add_argument("--kappa", type=float, nargs="+", default=[0.05])
    p.add_argument("--z", type=float, nargs="+", default=[-5.0, 0.0, 5.0])
    p.add_argument("--output_sample", default="sample.npy")
    p.add_argument("--output", default="a.cw")
    p.add_argument("--alpha", type=float, default=1.0)
    p.add_argument("--beta", type=float, default=0.0)
    p.add_argument("--na", type=float, default=None)
    p.add_argument("--samples", type=int, nargs="+", default=[64, 64])
    p.add_argument("--wavemask", type=int, nargs=3, default=[1, 1, 1])
    p.add_argument("--mode", default="polar", choices=["polar", "montecarlo"])
    p.add_argument("--log", action="store_true")
    p.add_argument("--device", type=int, default=0)
    return p


def main(argv=None) -> int:
    a = parser().parse_args(argv)
    from . import evaluator as ev
    n, kappa, z = list(a.n), list(a.kappa), list(a.z)
    alpha = np.arcsin(a.na / n[0]) if a.na is not None else a.alpha
    L = max(len(n), len(kappa) + 1, len(z) + 1)          # sCWatterLayer.cpp:312-330
    n = n + [n[-1]] * (L - len(n))
    kappa = (kappa + [0.0] * L)[:L - 1]
    while len(z) + 1 < L:
        z.append(z[-1] + 10.0)
    if len(a.samples) == 1:
        N = (a.samples[0], 1) if a.mode == "montecarlo" else (int(np.sqrt(a.samples[0])),) * 2
    else:
        N = (a.samples[0], a.samples[1])
    if alpha == 0:
        N = (1, 1)
    e = [complex(*a.ex), complex(*a.ey), complex(*a.ez)]
    waves = incident_waves(a.direction, e, n[0], a.lam, alpha, a.beta, N, a.mode)
    ctx = ev.Context(a.device)
    _, S = solve_layers(ctx, waves, n, kappa, z, a.lam, [bool(v) for v in a.wavemask])
    if a.output:
        S.save(a.output)
    if a.output_sample and L > 2:
        ri = np.array([complex(n[l], kappa[l - 1]) for l in range(1, L - 1)]).reshape(-1, 1, 1)
        np.save(a.output_sample, ri)
    print(f"layers: {L}, incident waves: {len(waves)} ({N[0]} x {N[1]}, {a.mode})")
    return 0


if __name__ == "__main__":
    sys.exit(main())
