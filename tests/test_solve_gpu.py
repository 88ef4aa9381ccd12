"""GPU per-layer solve (sCWatter.cpp:569-956) against the FP64 oracle restatement.

The GPU path decomposes the reduced 2MF matrix PQ instead of the 4MF matrix Phi, so mode
order, eigenvector scaling and the up/down labelling of exactly real roots differ from the
reference; everything physical must agree: the reflected / transmitted amplitudes x, the
set of gamma^2 per slice, and the field of the written .cw structure (compared in FP64).
"""
import numpy as np
import pytest

from oracle import oracle_lib as ol
from oracle import solve_oracle as so
from scwatter_gb300 import samples
from tests._util import rel_l2

pytestmark = pytest.mark.gpu

# FP64 solve vs FP64 solve: agreement limited by the conditioning of the mode matrices
TOL_X = 1e-11
TOL_GAMMA2 = 1e-11
TOL_FIELD = 1e-7
# FP32 evaluators (plain and separable) on the solved structure
TOL_EVAL = 2e-5

CASES = {
    "spheres_normal": dict(shape=(3, 16, 16), coef=(5, 5), seed=1, kw=dict(ex=(1, 0), ey=(0, 0))),
    "oblique_absorbing_substrate": dict(shape=(2, 12, 16), coef=(3, 5), seed=2,
                                        kw=dict(lam=0.9, direction=(0.3, 0.1, 1.0), ex=(1, 0), ey=(0, 0.5),
                                                n=(1.0, 1.3), kappa=0.05, z=0.4)),
    "one_slice_even_rows_odd_cols": dict(shape=(1, 10, 9), coef=(3, 3), seed=3, kw=dict()),
    "no_pz_rectangular": dict(shape=(4, 9, 8), coef=(5, 3), seed=4, kw=dict(pz=False, ex=(0.5, 0.2), ey=(1, 0))),
    "psf_default_polarisation": dict(shape=(2, 8, 8), coef=(3, 3), seed=8, kw=dict(psf=True)),
}


def _oracle(sample, coef, kw, external=False):
    Z, Y, X = sample.shape
    kw = dict(kw)
    kappa = kw.pop("kappa", 0.0)
    prm = so.SolveParams(size=(float(X), float(Y), float(Z)), coef=coef, external=external, kappa=(kappa,), **kw)
    r = so.solve(sample, prm)
    return prm, r, so.pack(r, prm)


def _gpu(ctx, sample, coef, kw, external=False):
    from scwatter_gb300 import solver
    Z, Y, X = sample.shape
    return solver.solve(sample, size=(float(X), float(Y), float(Z)), coef=coef, external=external, ctx=ctx, **kw)


@pytest.fixture(scope="module")
def ctx():
    from scwatter_gb300 import evaluator as ev
    return ev.Context(0)


def _points(zmin, zmax, sx, sy, n=400, seed=0):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(-sx, sx, n), rng.uniform(-sy, sy, n), rng.uniform(zmin, zmax, n)], 1)


def _field(cw_like, pts):
    W, b, e, zl = so.unpack(cw_like)
    return ol.eval_points_f64(W, b, e, ol.thresholds(zl, "cpu"), pts)


def _cw_of(S):
    """CoupledWaveStructure -> oracle CW."""
    return so.CW(Pi=S.Pi, z=[L.z for L in S.Layers], Pr=[L.Pr for L in S.Layers], Pt=[L.Pt for L in S.Layers])


@pytest.mark.parametrize("name", list(CASES))
def test_solve_matches_oracle(ctx, name):
    c = CASES[name]
    sample = samples.spheres(c["shape"], n_spheres=2, radius=(2, 4), seed=c["seed"])
    prm, r, cw_ref = _oracle(sample, c["coef"], c["kw"])
    g = _gpu(ctx, sample, c["coef"], c["kw"])
    assert g.M == tuple(r.M) and g.Z == len(r.eigenvalues)
    np.testing.assert_allclose(g.z, r.z, rtol=0, atol=1e-12)
    np.testing.assert_allclose(g.EF, r.EF, rtol=0, atol=1e-12)
    assert np.linalg.norm(g.x - r.x) / np.linalg.norm(r.x) < TOL_X
    for l in range(g.Z):
        ref2 = np.sort_complex(np.round(r.eigenvalues[l][0::2] ** 2, 12))
        got2 = g.gamma[l] ** 2
        # nearest match of every reference gamma^2 among the GPU's
        d = np.abs(ref2[:, None] - got2[None, :]).min(axis=1)
        assert d.max() / np.abs(ref2).max() < TOL_GAMMA2, (l, d.max())
        assert np.all(g.gamma[l].imag >= 0)
    # the written structure: same wave counts, same field (FP64 evaluation of both)
    S = g.to_cw()
    assert len(S.Pi) == len(cw_ref.Pi) and len(S.Layers) == len(cw_ref.z)
    for L, zr, pr, pt in zip(S.Layers, cw_ref.z, cw_ref.Pr, cw_ref.Pt):
        assert L.z == pytest.approx(zr, abs=1e-12) and len(L.Pr) == len(pr) and len(L.Pt) == len(pt)
    Z, Y, X = sample.shape
    zc = c["kw"].get("z", 0.0)
    pts = _points(zc - 1.5 * Z, zc + 1.5 * Z, X / 2, Y / 2, seed=c["seed"])
    fr = _field(cw_ref, pts)
    fg = _field(_cw_of(S), pts)
    assert max(rel_l2(fg, fr)) < TOL_FIELD


def test_external_mode(ctx):
    sample = samples.spheres((3, 12, 12), n_spheres=2, radius=(2, 4), seed=5)
    kw = dict(ex=(1, 0), ey=(0, 0))
    _, r, cw_ref = _oracle(sample, (3, 3), kw, external=True)
    g = _gpu(ctx, sample, (3, 3), kw, external=True)
    assert np.linalg.norm(g.x - r.x) / np.linalg.norm(r.x) < TOL_X
    S = g.to_cw()
    for L, zr, pr, pt in zip(S.Layers, cw_ref.z, cw_ref.Pr, cw_ref.Pt):
        assert L.z == zr and len(L.Pr) == len(pr) and len(L.Pt) == len(pt)
    pts = _points(-5, 5, 6, 6)
    assert max(rel_l2(_field(_cw_of(S), pts), _field(cw_ref, pts))) < TOL_FIELD


def test_solve_to_evaluators(ctx):
    """solve -> separable set and solve -> .cw -> plain evaluator give the same planes."""
    from scwatter_gb300 import evaluator as ev
    from scwatter_gb300 import separable as sp
    sample = samples.spheres((3, 16, 16), n_spheres=2, radius=(2, 4), seed=6)
    kw = dict(ex=(1, 0), ey=(0, 0))
    g = _gpu(ctx, sample, (5, 5), kw)
    S = g.to_cw()
    ws = ev.WaveSet.from_cw(ctx, S)
    sep = g.to_sep()
    N = 40
    d = np.float32(20.0 / (N - 1))
    args = (np.float32(-10), np.float32(-10), np.float32(-10), 0.3, -0.2, 0.1, d, N)
    plain = ws.evaluate_planes_host(*args)
    ref = [None] * 3
    W, b, e, zl = so.unpack(_cw_of(S))
    thr = ol.thresholds(zl, "gpu")
    for i, (axis, a0, b0, cc) in enumerate([(ol.AXIS_XY, args[0], args[1], args[5]),
                                            (ol.AXIS_XZ, args[0], args[2], args[4]),
                                            (ol.AXIS_YZ, args[1], args[2], args[3])]):
        P = ol.plane_points(axis, a0, b0, cc, d, N)
        ref[i] = ol.eval_points_f64(W, b, e, thr, P.reshape(-1, 3)).reshape(N, N, 3)
    for method in (sp.FP32, sp.TF32X3):
        got = sep.evaluate_planes_host(*args, method=method)
        for gg, rr in zip(got, ref):
            assert max(rel_l2(gg, rr)) < TOL_EVAL
    for pp, rr in zip(plain, ref):
        assert max(rel_l2(pp, rr)) < TOL_EVAL


def test_save_roundtrip(ctx, tmp_path):
    from scwatter_gb300.cw import CoupledWaveStructure
    sample = samples.spheres((2, 8, 8), n_spheres=1, radius=(2, 3), seed=7)
    g = _gpu(ctx, sample, (3, 3), dict())
    p = tmp_path / "c.cw"
    g.save(str(p))
    S = CoupledWaveStructure()
    assert S.load(str(p))
    T = g.to_cw()
    np.testing.assert_array_equal(S.Pi, T.Pi)
    for a, b in zip(S.Layers, T.Layers):
        np.testing.assert_array_equal(a.Pr, b.Pr)
        np.testing.assert_array_equal(a.Pt, b.Pt)


def test_command_line(tmp_path):
    """python -m scwatter_gb300.scwatter writes the structure the oracle packs."""
    from scwatter_gb300 import scwatter
    from scwatter_gb300.cw import CoupledWaveStructure
    sample = samples.spheres((2, 8, 8), n_spheres=1, radius=(2, 3), seed=9)
    np.save(tmp_path / "s.npy", sample)
    out = tmp_path / "c.cw"
    rc = scwatter.main(["--sample", str(tmp_path / "s.npy"), "--size", "8", "8", "2", "--coef", "3", "3",
                        "--ex", "1", "0", "--ey", "0", "0", "--direction", "0.2", "-0.1", "1", "--output", str(out)])
    assert rc == 0
    S = CoupledWaveStructure()
    assert S.load(str(out))
    prm = so.SolveParams(size=(8.0, 8.0, 2.0), coef=(3, 3), ex=(1, 0), ey=(0, 0), direction=(0.2, -0.1, 1.0))
    cw_ref = so.pack(so.solve(sample, prm), prm)
    pts = _points(-3, 3, 4, 4)
    assert max(rel_l2(_field(_cw_of(S), pts), _field(cw_ref, pts))) < TOL_FIELD
