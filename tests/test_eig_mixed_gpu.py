"""Mixed-precision eigen-solver (FP32 Householder + QR, FP64 Newton refinement, FP64 QR
fallback) against LAPACK (numpy): the GPU replacement of the reference's MKL_eigensolve
(third_Lapack.h:38-47) on the reduced layer matrices."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from scwatter_gb300 import evaluator as ev
    return ev.Context(0)


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _mixed(ctx, A):
    """Runs scw_zgeev_mixed on the batch A [B, n, n]; returns (W, V, accepted, steps, residual)."""
    import torch
    from scwatter_gb300 import _lib
    B, n, _ = A.shape
    dA = torch.from_numpy(np.ascontiguousarray(A, dtype=np.complex128)).cuda()
    dW = torch.zeros((B, n), dtype=torch.complex128, device="cuda")
    dV = torch.zeros((B, n, n), dtype=torch.complex128, device="cuda")
    acc = np.zeros(B, np.int32)
    steps = np.zeros(B, np.int32)
    res = np.zeros(B, np.float64)
    torch.cuda.synchronize()
    _lib.call("scw_zgeev_mixed", ctx.handle, n, _p(dA), _p(dW), _p(dV), B, ctypes.c_void_p(acc.ctypes.data),
              ctypes.c_void_p(steps.ctypes.data), ctypes.c_void_p(res.ctypes.data))
    return dW.cpu().numpy(), dV.cpu().numpy(), acc, steps, res


def _check(A, W, V, tol=1e-12):
    """Relative column residuals, eigenvalues as a set against LAPACK, a nonsingular basis."""
    for b in range(A.shape[0]):
        nA = np.linalg.norm(A[b], 1)
        r = np.linalg.norm(A[b] @ V[b] - V[b] * W[b][None, :], axis=0) / (nA * np.linalg.norm(V[b], axis=0))
        assert r.max() < tol, (b, r.max())
        ref = np.linalg.eigvals(A[b])
        d = np.abs(W[b][:, None] - ref[None, :]).min(axis=1)
        assert d.max() < 1e-10 * nA
        assert np.linalg.cond(V[b]) < 1e8


def test_random_matrices(ctx):
    rng = np.random.default_rng(7)
    A = rng.standard_normal((3, 96, 96)) + 1j * rng.standard_normal((3, 96, 96))
    W, V, acc, steps, res = _mixed(ctx, A)
    _check(A, W, V)
    assert (acc == 1).all() and (res <= 1e-12).all()


def test_layer_matrices(ctx):
    """Reduced matrices PQ of sphere slices, a homogeneous slab (eigenvalues of multiplicity up
    to 16 at normal incidence) and a centred cylinder (dense clusters): all accepted, and the
    FP64 QR reference agrees."""
    from scwatter_gb300 import samples
    from scwatter_gb300.warmstart import layer_problems, plain_eig
    vol = samples.spheres((6, 48, 48), seed=2)
    y, x = np.mgrid[:48, :48]
    cyl = np.where((x - 24) ** 2 + (y - 24) ** 2 < 64, 1.4 + 0.01j, 1.0 + 0j)
    vol[0] = 1.4 + 0.01j
    vol[1] = cyl
    lp = layer_problems(ctx, vol, lam=1.0, size=(48.0, 48.0, 6.0), coef=(12, 12))
    A = lp.PQ.cpu().numpy()
    W, V, acc, steps, res = _mixed(ctx, A)
    _check(A, W, V)
    assert (acc == 1).sum() >= 5                 # the cylinder slice may take the FP64 solver
    W64, V64 = plain_eig(ctx, lp.PQ)
    for b in range(A.shape[0]):
        d = np.abs(W[b][:, None] - W64[b].cpu().numpy()[None, :]).min(axis=1)
        assert d.max() < 1e-11 * np.linalg.norm(A[b], 1)


def test_fallback_on_defective_matrix(ctx):
    """A Jordan block cannot be refined to a residual basis: that matrix goes through the FP64
    QR solver (accepted != 1: the reason code) while its neighbour in the batch is refined."""
    rng = np.random.default_rng(3)
    n = 48
    J = np.diag(np.full(n, 0.5 + 0.1j)) + np.diag(np.ones(n - 1), 1)
    G = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = np.stack([J, G])
    W, V, acc, steps, res = _mixed(ctx, A)
    assert acc[1] == 1 and acc[0] in (2, 3, 4, 5, 6)
    _check(A[1:], W[1:], V[1:])
    assert np.abs(W[0] - (0.5 + 0.1j)).max() < 1e-1          # the FP64 QR's (perturbed) eigenvalues


def test_solve_matches_fp64_eigen_solver(ctx):
    """The whole coupled-wave solve with the mixed eigen-solver against the FP64 QR path."""
    from scwatter_gb300 import samples, solver
    vol = samples.spheres((8, 32, 32), seed=4)
    kw = dict(lam=1.0, size=(32.0, 32.0, 8.0), coef=(10, 10), direction=(0.2, 0.1, 1.0), ctx=ctx)
    g = solver.solve(vol, **kw)
    f = solver.solve(vol, eig_fp64=True, **kw)
    assert g.eig["mixed"] and g.eig["accepted"] == 8 and g.eig["max_residual"] <= 1e-12
    assert not f.eig["mixed"]
    assert np.linalg.norm(g.x - f.x) < 1e-11 * np.linalg.norm(f.x)


def test_wide_hessenberg_path(ctx):
    """Matrices of order >= 128 take the Hessenberg reduction spread over the GPU (3 launches per
    column): random and layer-like (nearly diagonal, clustered) matrices in one batch, refined to
    FP64 residuals, eigenvalues equal to LAPACK's."""
    rng = np.random.default_rng(11)
    n = 200
    A = rng.standard_normal((3, n, n)) + 1j * rng.standard_normal((3, n, n))
    d = np.repeat(np.linspace(0.5, 1.5, n // 8), 8)             # multiplicity-8 diagonal with couplings
    A[2] = np.diag(d + 0.01j) + 1e-3 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    W, V, acc, steps, res = _mixed(ctx, A)
    _check(A, W, V)
    assert (acc == 1).all()


def test_wide_fp32_stage_matches_lapack(ctx):
    """scw_cgeev at n = 256 (wide Hessenberg + FP32 QR): FP32 eigenvalues against LAPACK's."""
    import torch
    from scwatter_gb300 import _lib
    rng = np.random.default_rng(5)
    n, B = 256, 2
    A = (rng.standard_normal((B, n, n)) + 1j * rng.standard_normal((B, n, n))).astype(np.complex64)
    dA = torch.from_numpy(A.copy()).cuda()
    dW = torch.zeros((B, n), dtype=torch.complex64, device="cuda")
    dV = torch.zeros((B, n, n), dtype=torch.complex64, device="cuda")
    st = np.zeros(B, np.int32)
    torch.cuda.synchronize()
    _lib.call("scw_cgeev", ctx.handle, n, _p(dA), _p(dW), _p(dV), B, ctypes.c_void_p(st.ctypes.data))
    W, V = dW.cpu().numpy(), dV.cpu().numpy()
    assert (st == 0).all()
    for b in range(B):
        A64 = A[b].astype(np.complex128)
        ref = np.linalg.eigvals(A64)
        nA = np.linalg.norm(A64, 1)
        assert np.abs(W[b][:, None] - ref[None, :]).min(axis=1).max() < 1e-4 * nA
        r = np.linalg.norm(A64 @ V[b] - V[b] * W[b][None, :], axis=0) / (nA * np.linalg.norm(V[b], axis=0))
        assert r.max() < 1e-5
