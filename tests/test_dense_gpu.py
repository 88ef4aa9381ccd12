"""FP64 complex dense kernels (GPU replacements of the reference's MKL wrappers,
third_Lapack.h:38-87) vs numpy/LAPACK."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from scwatter_gb300 import evaluator as ev
    return ev.Context(0)


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex128)).cuda()


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _rand(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("M,N,K,batch", [(5, 7, 3, 1), (130, 70, 200, 3), (64, 64, 64, 2)])
def test_zgemm(ctx, M, N, K, batch):
    from scwatter_gb300 import _lib
    import torch
    rng = np.random.default_rng(0)
    A, B, C = _rand(rng, batch, M, K), _rand(rng, batch, K, N), _rand(rng, batch, M, N)
    dA, dB, dC = _dev(A), _dev(B), _dev(C)
    torch.cuda.synchronize()
    al = (ctypes.c_double * 2)(0.5, -1.25)
    be = (ctypes.c_double * 2)(2.0, 0.5)
    _lib.call("scw_zgemm", ctx.handle, M, N, K, al, _p(dA), _p(dB), be, _p(dC), batch)
    ctx.synchronize()
    ref = (0.5 - 1.25j) * (A @ B) + (2.0 + 0.5j) * C
    assert np.abs(dC.cpu().numpy() - ref).max() < 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("n,nrhs,batch", [(1, 1, 1), (37, 3, 2), (200, 5, 3), (97, 64, 1)])
def test_zgesv(ctx, n, nrhs, batch):
    from scwatter_gb300 import _lib
    import torch
    rng = np.random.default_rng(1)
    A, B = _rand(rng, batch, n, n), _rand(rng, batch, n, nrhs)
    dA, dB = _dev(A), _dev(B)
    torch.cuda.synchronize()
    _lib.call("scw_zgesv", ctx.handle, n, nrhs, _p(dA), _p(dB), batch, None)
    X = dB.cpu().numpy()
    for b in range(batch):
        r = np.linalg.norm(A[b] @ X[b] - B[b]) / (np.linalg.norm(A[b]) * np.linalg.norm(X[b]))
        assert r < 1e-13


def test_zgesv_singular_reported(ctx):
    from scwatter_gb300 import _lib
    import torch
    A = np.zeros((1, 4, 4), complex)
    A[0, :3, :3] = np.eye(3)
    dA, dB = _dev(A), _dev(np.ones((1, 4, 1), complex))
    torch.cuda.synchronize()
    info = (ctypes.c_int * 1)()
    st = _lib.load().scw_zgesv(ctx.handle, 4, 1, _p(dA), _p(dB), 1, info)
    assert st == 7 and info[0] == 4


def _check_eig(A, w, V):
    n = A.shape[0]
    res = np.linalg.norm(A @ V - V * w[None, :]) / (np.linalg.norm(A) * np.linalg.norm(V))
    assert res < 1e-12, res
    ref = np.linalg.eigvals(A)
    # every reference eigenvalue has a match
    d = np.abs(ref[:, None] - w[None, :]).min(axis=1)
    assert d.max() < 1e-9 * max(1.0, np.abs(ref).max())
    # independent eigenvectors
    s = np.linalg.svd(V / np.linalg.norm(V, axis=0), compute_uv=False)
    assert s[-1] / s[0] > 1e-9


@pytest.mark.parametrize("n,batch", [(2, 1), (17, 2), (96, 3), (300, 1)])
def test_zgeev_random(ctx, n, batch):
    from scwatter_gb300 import _lib
    import torch
    rng = np.random.default_rng(2)
    A = _rand(rng, batch, n, n)
    dA = _dev(A)
    dW = torch.zeros((batch, n), dtype=torch.complex128, device="cuda")
    dV = torch.zeros((batch, n, n), dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    _lib.call("scw_zgeev", ctx.handle, n, _p(dA), _p(dW), _p(dV), batch, None)
    W, V = dW.cpu().numpy(), dV.cpu().numpy()
    for b in range(batch):
        _check_eig(A[b], W[b], V[b])


def test_zgeev_degenerate(ctx):
    """Repeated eigenvalues of a diagonalizable matrix (as in homogeneous slices)."""
    from scwatter_gb300 import _lib
    import torch
    rng = np.random.default_rng(3)
    n = 40
    lam = np.repeat(rng.standard_normal(10) + 0.3j * rng.standard_normal(10), 4)
    S = _rand(rng, n, n) + 4 * np.eye(n)
    A = (S * lam[None, :]) @ np.linalg.inv(S)
    dA = _dev(A[None])
    dW = torch.zeros((1, n), dtype=torch.complex128, device="cuda")
    dV = torch.zeros((1, n, n), dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    _lib.call("scw_zgeev", ctx.handle, n, _p(dA), _p(dW), _p(dV), 1, None)
    W, V = dW.cpu().numpy()[0], dV.cpu().numpy()[0]
    res = np.linalg.norm(A @ V - V * W[None, :]) / (np.linalg.norm(A) * np.linalg.norm(V))
    assert res < 1e-10
    s = np.linalg.svd(V / np.linalg.norm(V, axis=0), compute_uv=False)
    assert s[-1] / s[0] > 1e-8


def test_zgeev_diagonal_with_rounding_couplings(ctx):
    """A homogeneous slice's PQ: diagonal with repeated eigenvalues and 1e-18 couplings
    between equal entries.  The QR iteration must deflate them instead of cycling."""
    from scwatter_gb300 import _lib
    import torch
    rng = np.random.default_rng(5)
    n = 30
    lam = np.repeat(rng.uniform(0.9, 1.0, 6), 5).astype(np.complex128)
    A = np.diag(lam)
    for i in range(0, n - 1, 2):
        if lam[i] == lam[i + 1]:
            A[i, i + 1] = A[i + 1, i] = 4.3e-18
    dA = _dev(A[None])
    dW = torch.zeros((1, n), dtype=torch.complex128, device="cuda")
    dV = torch.zeros((1, n, n), dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    _lib.call("scw_zgeev", ctx.handle, n, _p(dA), _p(dW), _p(dV), 1, None)
    W, V = dW.cpu().numpy()[0], dV.cpu().numpy()[0]
    res = np.linalg.norm(A @ V - V * W[None, :]) / (np.linalg.norm(A) * np.linalg.norm(V))
    assert res < 1e-14
    assert np.linalg.cond(V / np.linalg.norm(V, axis=0)) < 10
    np.testing.assert_allclose(np.sort(W.real), np.sort(lam.real), atol=1e-15)
