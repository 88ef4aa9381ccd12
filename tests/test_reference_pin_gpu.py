"""Parity pinned to the reference's own code.

The reference viewer's GPU evaluator (gpuEvaluator.cu:15-165: gpu_initialize, the region
search with the z >= z_l - 0.001 rule, the per-wave exp sum, gpu_cw_evaluate's three planes)
is compiled unchanged by ``oracle/ref_build.py`` and run on the golden .cw structures.  Its
output pins the FP64 oracle (the restatement the other tests use as ground truth) to the
reference, and the drop-in shim ``scwatter_gb300/shim/gpuEvaluator_gb300.cu`` -- the same two
entry points, compiled against the reference's gpuEvaluator.h and run on this library -- must
give the reference's planes.
"""
import os

import numpy as np
import pytest

from oracle import oracle_lib as ol
from oracle import ref_build
from oracle import solve_oracle as so
from tests._util import rel_l2, solved_case

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# FP32 evaluation (the reference's thrust::complex<float> sum, wound to the origin) against FP64
TOL_F32 = 3e-5


def _cases():
    out = []
    for name in sorted(f[:-3] for f in os.listdir(HERE) if f.endswith(".cw")):
        with open(os.path.join(HERE, name + ".cw"), "rb") as f:
            out.append((name, so.cw_from_bytes(f.read())))
    return out


@pytest.fixture(scope="module")
def refmod():
    if not ref_build.sources_present():
        pytest.skip("the reference's gpuEvaluator.cu was not copied into oracle/_ref/src (no reference checkout "
                    "where the checkers were built)")
    ref_build.build()
    from oracle import ref_lib
    return ref_lib


def _views(c):
    zs = np.asarray(c.z, dtype=np.float64)
    ext = 24.0
    N = 40
    d = np.float32(ext / (N - 1))
    st = np.float32(-ext / 2)
    zmid = float(np.float32(0.5 * (zs[0] + zs[-1]) + 0.137))
    return [dict(xs=st, ys=st, zs=st, x=0.31, y=-0.42, z=zmid, d=d, N=N),
            dict(xs=np.float32(-5), ys=np.float32(-4), zs=np.float32(zs[0] - 1.5), x=-1.7, y=2.2,
                 z=float(np.float32(zs[-1] + 0.8)), d=np.float32(0.25), N=33)]


def _oracle(W, b, e, zl, v):
    thr = ol.thresholds(zl, "gpu")
    out = []
    for axis, a0, b0, cc in [(ol.AXIS_XY, v["xs"], v["ys"], v["z"]), (ol.AXIS_XZ, v["xs"], v["zs"], v["y"]),
                             (ol.AXIS_YZ, v["ys"], v["zs"], v["x"])]:
        P = ol.plane_points(axis, a0, b0, np.float32(cc), v["d"], v["N"])
        out.append(ol.eval_points_f64(W, b, e, thr, P.reshape(-1, 3)).reshape(v["N"], v["N"], 3))
    return out


def _structures():
    cases = _cases()
    _, _, _, c = solved_case(shape=(3, 16, 16), coef=(5, 5), seed=1, direction=(0.2, -0.1, 1.0))
    cases.append(("oblique_3x16x16_c5", c))
    return cases


@pytest.mark.parametrize("case", range(3))
def test_oracle_and_shim_match_reference_kernels(refmod, case):
    name, c = _structures()[case]
    W, b, e, zl = so.unpack(c)
    for v in _views(c):
        args = (W, b, e, zl, v["xs"], v["ys"], v["zs"], v["x"], v["y"], v["z"], v["d"], v["N"])
        ref = refmod.evaluate("reference", *args)
        shim = refmod.evaluate("shim", *args)
        orc = _oracle(W, b, e, zl, v)
        for plane, r, s, o in zip(["xy", "xz", "yz"], ref, shim, orc):
            assert np.isfinite(r).all() and np.isfinite(s).all()
            # the FP64 oracle restates the reference's kernels: pinned to their output
            assert max(rel_l2(r, o, floor=0.0)) < TOL_F32, (name, plane, "reference vs oracle", rel_l2(r, o, 0.0))
            # the drop-in shim gives the reference's planes
            assert max(rel_l2(s, r, floor=0.0)) < TOL_F32, (name, plane, "shim vs reference", rel_l2(s, r, 0.0))
            assert max(rel_l2(s, o, floor=0.0)) < TOL_F32, (name, plane, "shim vs oracle", rel_l2(s, o, 0.0))


def test_region_rule_matches_reference_at_boundaries(refmod):
    """Points within 0.001 below a boundary take the lower region in the reference
    (gpuEvaluator.cu:34); the oracle's 'gpu' rule and the shim agree."""
    name, c = _cases()[0]
    W, b, e, zl = so.unpack(c)
    zb = float(np.float32(c.z[1]))
    v = dict(xs=np.float32(-3), ys=np.float32(-3), zs=np.float32(zb - 0.0015), x=0.1, y=0.2, z=zb - 0.0005,
             d=np.float32(0.00025), N=16)
    args = (W, b, e, zl, v["xs"], v["ys"], v["zs"], v["x"], v["y"], v["z"], v["d"], v["N"])
    ref = refmod.evaluate("reference", *args)
    shim = refmod.evaluate("shim", *args)
    orc = _oracle(W, b, e, zl, v)
    for r, s, o in zip(ref, shim, orc):
        assert max(rel_l2(r, o, floor=0.0)) < TOL_F32
        assert max(rel_l2(s, r, floor=0.0)) < TOL_F32
