"""Regenerates the golden fixtures in this directory from the FP64 oracle.

    python tests/golden/make_golden.py

Each case: a seeded sphere sample, the solve parameters, the oracle's reflected /
transmitted amplitudes x, incident amplitudes EF, the sorted gamma^2 of every slice, the
.cw file the oracle packs (bytes of the reference's layout), FP64 fields at seeded points,
and the reference-semantics FP32 CPU evaluator's xy plane (cpuEvaluator.cpp:294-407).
The reference itself cannot be built here, so these pin the oracle against regressions and
give the GPU path fixed vectors to match.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle_lib as ol  # noqa: E402
from oracle import solve_oracle as so  # noqa: E402
from scwatter_gb300 import samples  # noqa: E402

CASES = {
    "spheres_2x8x8_c3": dict(shape=(2, 8, 8), coef=(3, 3), seed=11, prm=dict(ex=(1, 0), ey=(0, 0))),
    "oblique_3x10x12_c3x5": dict(shape=(3, 10, 12), coef=(3, 5), seed=12,
                                 prm=dict(lam=0.8, direction=(0.25, -0.1, 1.0), ex=(0.3, 0.1), ey=(1, 0),
                                          n=(1.0, 1.2), kappa=(0.03,), z=0.5)),
}


def points(shape, z0, seed):
    Z, Y, X = shape
    rng = np.random.default_rng(seed)
    n = 96
    return np.stack([rng.uniform(-X / 2, X / 2, n), rng.uniform(-Y / 2, Y / 2, n),
                     rng.uniform(z0 - 1.5 * Z, z0 + 1.5 * Z, n)], 1)


def make(name, c):
    Z, Y, X = c["shape"]
    sample = samples.spheres(c["shape"], n_spheres=2, radius=(2, 4), seed=c["seed"])
    prm = so.SolveParams(size=(float(X), float(Y), float(Z)), coef=c["coef"], **c["prm"])
    r = so.solve(sample, prm)
    cw = so.pack(r, prm)
    pts = points(c["shape"], prm.z, c["seed"])
    W, b, e, zl = so.unpack(cw)
    field = ol.eval_points_f64(W, b, e, ol.thresholds(zl, "cpu"), pts)
    W32, b32, e32, zl32 = so.unpack(cw, np.complex64)
    N = 16
    d = np.float32(X / (N - 1))
    st = np.float32(-X / 2)
    zc = np.float32(prm.z)
    plane = ol.cpu_eval_plane_f32(ol.AXIS_XY, W32, b32, e32, zl32, st, st, zc, d, N)
    g2 = np.stack([np.sort_complex(ev[0::2] ** 2) for ev in r.eigenvalues])
    np.savez(os.path.join(HERE, name + ".npz"), sample=sample, x=r.x, EF=r.EF, gamma2=g2, points=pts, field=field,
             plane_f32=plane, plane_args=np.array([st, st, zc, d, N], np.float64), z=r.z)
    with open(os.path.join(HERE, name + ".cw"), "wb") as f:
        f.write(so.cw_to_bytes(cw))


if __name__ == "__main__":
    ol.build()
    for k, v in CASES.items():
        make(k, v)
        print("wrote", k)
