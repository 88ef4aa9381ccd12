"""Golden fixtures (tests/golden/, made by make_golden.py from the FP64 oracle).

CPU: the oracle reproduces its fixtures (solve amplitudes, gamma^2, .cw bytes, FP64 fields,
reference-semantics FP32 plane).  GPU: the solve and the evaluators match them.
"""
import os

import numpy as np
import pytest

from oracle import oracle_lib as ol
from oracle import solve_oracle as so
from tests._util import rel_l2

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
import importlib.util  # noqa: E402

_spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "make_golden.py"))
mg = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(mg)
NAMES = sorted(mg.CASES)


def _load(name):
    g = dict(np.load(os.path.join(HERE, name + ".npz")))
    with open(os.path.join(HERE, name + ".cw"), "rb") as f:
        g["cw_bytes"] = f.read()
    c = mg.CASES[name]
    Z, Y, X = c["shape"]
    g["prm"] = so.SolveParams(size=(float(X), float(Y), float(Z)), coef=c["coef"], **c["prm"])
    return g


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    g = _load(name)
    r = so.solve(g["sample"], g["prm"])
    assert np.linalg.norm(r.x - g["x"]) / np.linalg.norm(g["x"]) < 1e-12
    np.testing.assert_allclose(r.EF, g["EF"], atol=1e-14)
    cw = so.pack(r, g["prm"])
    b = so.cw_to_bytes(cw)
    assert len(b) == len(g["cw_bytes"])
    back = so.cw_from_bytes(g["cw_bytes"])
    W, bb, e, zl = so.unpack(back)
    f = ol.eval_points_f64(W, bb, e, ol.thresholds(zl, "cpu"), g["points"])
    assert max(rel_l2(f, g["field"])) < 1e-12
    W32, b32, e32, zl32 = so.unpack(back, np.complex64)
    st, st2, zc, d, N = g["plane_args"]
    plane = ol.cpu_eval_plane_f32(ol.AXIS_XY, W32, b32, e32, zl32, np.float32(st), np.float32(st2),
                                  np.float32(zc), np.float32(d), int(N))
    assert np.array_equal(plane, g["plane_f32"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_golden(name):
    from scwatter_gb300 import evaluator as ev
    from scwatter_gb300 import solver
    from scwatter_gb300.cw import CoupledWaveStructure
    g = _load(name)
    p = g["prm"]
    ctx = ev.Context(0)
    s = solver.solve(g["sample"], lam=p.lam, direction=p.direction, ex=p.ex, ey=p.ey, ez=p.ez, n=p.n,
                     kappa=p.kappa, size=p.size, z=p.z, coef=p.coef, ctx=ctx)
    assert np.linalg.norm(s.x - g["x"]) / np.linalg.norm(g["x"]) < 1e-11
    for l in range(s.Z):
        d = np.abs(g["gamma2"][l][:, None] - (s.gamma[l] ** 2)[None, :]).min(axis=1)
        assert d.max() < 1e-11 * np.abs(g["gamma2"][l]).max()
    # the golden .cw through the reference-named evaluator interface
    path = os.path.join(HERE, name + ".cw")
    S = CoupledWaveStructure()
    assert S.load(path)
    ev.cw_allocate(S)
    ev.cw_unpack(S)
    ev.gpu_initialize(0)
    st, st2, zc, d, N = g["plane_args"]
    N = int(N)
    E = [np.zeros(N * N * 3, np.complex64) for _ in range(3)]
    ev.gpu_cw_evaluate(E[0], E[1], E[2], st, st2, st2, 0.0, 0.0, zc, d, N, 0)
    assert max(rel_l2(E[0].reshape(N, N, 3), g["plane_f32"])) < 1e-4   # vs the reference's own FP32 sum
