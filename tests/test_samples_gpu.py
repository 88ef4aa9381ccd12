"""Device sample generators and the .npy device reader against the host generators, the oracle
restatement and numpy; a solve from a device sample against the same solve from host memory."""
import numpy as np
import pytest

from oracle import sample_oracle as smo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from scwatter_gb300 import evaluator as ev
    return ev.Context(0)


def test_spheres_device_equals_host(ctx):
    from scwatter_gb300 import samples
    for shape, seed in [((20, 64, 64), 0), ((5, 17, 33), 3)]:
        d = samples.spheres_device(ctx, shape, seed=seed).cpu().numpy()
        assert np.array_equal(d, samples.spheres(shape, seed=seed))


def test_grf_device_matches_oracle(ctx):
    from scwatter_gb300 import samples
    for shape, corr, seed in [((4, 24, 20), 3.0, 5), ((2, 16, 16), 8.0, 2 ** 63 + 7)]:
        d = samples.grf_device(ctx, shape, corr_px=corr, seed=seed).cpu().numpy()
        ref = smo.grf(shape, corr_px=corr, seed=seed)
        assert np.abs(d - ref).max() < 1e-12


def test_npy_to_device(ctx, tmp_path):
    from scwatter_gb300 import samples
    rng = np.random.default_rng(0)
    for arr in [rng.standard_normal((3, 5, 7)) + 1j * rng.standard_normal((3, 5, 7)),
                rng.standard_normal((6, 9)),
                np.asfortranarray(rng.standard_normal((6, 9)) + 1j)]:
        p = tmp_path / "v.npy"
        np.save(p, arr)
        d = samples.npy_to_device(ctx, p).cpu().numpy()
        want = np.asarray(arr, np.complex128).reshape(d.shape)
        assert np.array_equal(d, want)


def test_solve_from_device_sample(ctx):
    from scwatter_gb300 import samples, solver
    kw = dict(lam=1.0, size=(24.0, 24.0, 3.0), coef=(6, 6), direction=(0.1, 0.0, 1.0), ctx=ctx)
    host = solver.solve(samples.spheres((3, 24, 24), n_spheres=3, radius=(3.0, 6.0), seed=1), **kw)
    dev = solver.solve(samples.spheres_device(ctx, (3, 24, 24), n_spheres=3, radius=(3.0, 6.0), seed=1), **kw)
    assert np.array_equal(host.x, dev.x)
