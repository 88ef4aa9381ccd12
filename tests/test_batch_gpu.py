"""Batched solve + evaluate (one CUDA graph) against the single-sample path and the oracle."""
import numpy as np
import pytest

from oracle import oracle_lib as ol
from oracle import solve_oracle as so
from scwatter_gb300 import samples
from tests._util import rel_l2

pytestmark = pytest.mark.gpu

TOL_X = 1e-11
TOL_EVAL = {1: 2e-5, 2: 2e-5, 3: 1e-4}


@pytest.fixture(scope="module")
def ctx():
    from scwatter_gb300 import evaluator as ev
    return ev.Context(0)


def _items():
    from scwatter_gb300.batch import BatchItem
    rng = np.random.default_rng(3)
    out = []
    shapes = [(1, 8, 8), (3, 12, 10), (2, 16, 16), (4, 9, 12), (2, 10, 10)]
    coefs = [(3, 3), (5, 3), (4, 6), (3, 5), (1, 5)]
    for i, (shape, coef) in enumerate(zip(shapes, coefs)):
        Z, Y, X = shape
        s = samples.spheres(shape, n_spheres=2, radius=(2, 4), seed=20 + i)
        th = np.deg2rad(rng.uniform(0, 30))
        d = (np.sin(th), 0.0, np.cos(th))
        Nx, Ny, Nz = 12 + 3 * i, 10 + i, 5 + i
        grid = (-X / 2, -Y / 2, -1.5 * Z, X / (Nx - 1), Y / (Ny - 1), 3.0 * Z / (Nz - 1), Nx, Ny, Nz)
        out.append(BatchItem(sample=s, grid=grid, lam=float(rng.uniform(0.8, 1.2)), direction=d, ex=(1, 0),
                             ey=(0, 0), size=(float(X), float(Y), float(Z)), coef=coef,
                             external=(i == 4)))
    return out


def _grid_points(grid):
    x0, y0, z0, dx, dy, dz, Nx, Ny, Nz = grid
    f = np.float32
    xs = (f(x0) + f(dx) * np.arange(Nx, dtype=np.float32)).astype(np.float32)
    ys = (f(y0) + f(dy) * np.arange(Ny, dtype=np.float32)).astype(np.float32)
    zs = (f(z0) + f(dz) * np.arange(Nz, dtype=np.float32)).astype(np.float32)
    Zg, Yg, Xg = np.meshgrid(zs, ys, xs, indexing="ij")
    return np.stack([Xg, Yg, Zg], -1).reshape(-1, 3).astype(np.float64)


def _oracle(it):
    Z, Y, X = it.sample.shape
    prm = so.SolveParams(lam=it.lam, direction=it.direction, ex=it.ex, ey=it.ey, size=it.size, coef=it.coef,
                         external=it.external)
    r = so.solve(it.sample, prm)
    return r, so.pack(r, prm)


@pytest.mark.parametrize("lanes,method", [(1, 2), (3, 2), (2, 3), (2, 1)])
def test_batch_matches_oracle(ctx, lanes, method):
    from scwatter_gb300.batch import Batch
    items = _items()
    b = Batch(ctx, items, lanes=lanes, method=method)
    info = b.info()
    assert info["lanes"] == lanes and info["method"] == method and info["graph_nodes"] > 0
    for rep in range(2):                      # the graph relaunches with the same results
        b.run()
        st = b.wait()
        assert (st == 0).all()
        for i, it in enumerate(items):
            x, g, f = b.result(i)
            e = b.item_eig(i)                 # the mixed eigen-solver finished every slice itself
            assert e["mixed"] and e["fell_back"] == 0 and e["max_residual"] <= 1e-12
            st_s, steps_s, res_s = b.item_eig_slices(i)
            assert (st_s == 1).all() and res_s.max() == e["max_residual"] and steps_s.max() == e["max_steps"]
            r, cw = _oracle(it)
            assert np.linalg.norm(x - r.x) / np.linalg.norm(r.x) < TOL_X
            W, bb, e, zl = so.unpack(cw)
            ref = ol.eval_points_f64(W, bb, e, ol.thresholds(zl, "gpu"), _grid_points(it.grid))
            assert max(rel_l2(f.reshape(-1, 3), ref)) < TOL_EVAL[method], (i, rep)


def test_batch_autotune(ctx):
    from scwatter_gb300.batch import Batch
    items = _items()
    b = Batch(ctx, items)
    info = b.info()
    assert info["lanes"] >= 1 and info["method"] in (1, 2, 3) and len(info["tune_log"]) >= 5
    assert info["ctr_shape"] in (0, 1)
    # the tile-shape candidates were timed on evaluation-only graphs, both shapes
    assert {int(e[2]) for e in info["tune_log"]} == {0, 1}
    b.run()
    assert (b.wait() == 0).all()
    for i, it in enumerate(items):
        x, g, f = b.result(i)
        r, cw = _oracle(it)
        assert np.linalg.norm(x - r.x) / np.linalg.norm(r.x) < TOL_X
        W, bb, e, zl = so.unpack(cw)
        ref = ol.eval_points_f64(W, bb, e, ol.thresholds(zl, "gpu"), _grid_points(it.grid))
        assert max(rel_l2(f.reshape(-1, 3), ref)) < TOL_EVAL[info["method"]]


def test_uneven_generator_shapes():
    from scwatter_gb300.batch import uneven_items
    items = uneven_items(6, seed=1, m_range=(3, 6), z_range=(1, 4), grid_xy=(8, 16), grid_z=(4, 8), pixels=16)
    assert len(items) == 6
    for it in items:
        assert 1 <= it.sample.shape[0] <= 4 and 3 <= it.coef[0] <= 6 and 8 <= it.grid[6] <= 16
