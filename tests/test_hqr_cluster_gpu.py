"""QR sweeps on thread-block clusters against one CTA per matrix.

``scw_set_qr_cluster`` selects how many CTAs share each matrix's QR sweeps in the single-call
eigen-solvers (scw_zgeev, scw_cgeev, and through them scw_zgeev_mixed and scw_solve).  Rank 0 of a
cluster makes the decisions and chases each window; every CTA applies the window's rotations to
its share of the stripes.  Each element sees the same sequence of rotations in every setting, but
the cluster kernel is compiled separately from the one-CTA kernel and its multiply-adds may be
fused differently, so the results agree to rounding, not bit for bit (at n = 96 the second CTA
of a pair has no stripe to update, and the results still differ in the last bits).  The tests
require, for FP64 and FP32, cluster sizes 2, 4 and 8 and the per-call choice: the one-CTA
residual bound, the one-CTA eigenvalues as a set, and the mixed solver's FP64 fallback likewise.
"""
import ctypes
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.fixture(scope="module")
def ctx():
    from scwatter_gb300 import evaluator as ev
    return ev.Context(0)


def _matrices(B, n, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((B, n, n)) + 1j * rng.standard_normal((B, n, n))) / np.sqrt(n)


def _eig(ctx, fn, A, ctas):
    """fn ('scw_zgeev' or 'scw_cgeev') on the batch A with scw_set_qr_cluster(ctas); returns
    (W, V, status, seconds)."""
    import torch
    from scwatter_gb300 import _lib
    dt = torch.complex128 if fn == "scw_zgeev" else torch.complex64
    B, n, _ = A.shape
    dA = torch.from_numpy(np.ascontiguousarray(A)).to(dt).cuda()
    dW = torch.zeros((B, n), dtype=dt, device="cuda")
    dV = torch.zeros((B, n, n), dtype=dt, device="cuda")
    st = np.zeros(B, np.int32)
    torch.cuda.synchronize()
    _lib.call("scw_set_qr_cluster", int(ctas))
    try:
        t0 = time.perf_counter()
        _lib.call(fn, ctx.handle, n, _p(dA), _p(dW), _p(dV), B, ctypes.c_void_p(st.ctypes.data))
        t = time.perf_counter() - t0
    finally:
        _lib.call("scw_set_qr_cluster", 0)
    return dW.cpu().numpy(), dV.cpu().numpy(), st, t


def _set_dist(W1, W2):
    """max over matrices and eigenvalues of W1 of the distance to the nearest of W2, relative to
    the largest |eigenvalue|."""
    d = 0.0
    for a, b in zip(W1, W2):
        a = a.astype(np.complex128)
        b = b.astype(np.complex128)
        d = max(d, float(np.abs(a[:, None] - b[None, :]).min(axis=1).max() / np.abs(a).max()))
    return d


def _residual(A, W, V):
    r = 0.0
    for b in range(A.shape[0]):
        Ab = A[b].astype(np.complex128)
        Vb = V[b].astype(np.complex128)
        R = Ab @ Vb - Vb * W[b][None, :].astype(np.complex128)
        r = max(r, float((np.linalg.norm(R, axis=0) / (np.linalg.norm(Ab, 1) * np.linalg.norm(Vb, axis=0))).max()))
    return r


@pytest.mark.parametrize("fn,n,B", [("scw_zgeev", 96, 3), ("scw_zgeev", 300, 2), ("scw_cgeev", 300, 3),
                                    ("scw_cgeev", 700, 2)])
def test_cluster_sizes_agree(ctx, fn, n, B):
    A = _matrices(B, n, seed=n + B)
    fp64 = fn == "scw_zgeev"
    tol_res, tol_eig = (1e-12, 1e-9) if fp64 else (2e-4, 1e-2)
    W1, V1, s1, _ = _eig(ctx, fn, A, 1)
    assert not s1.any()
    assert _residual(A, W1, V1) < tol_res
    for k in (2, 4, 8, 0):
        Wk, Vk, sk, _ = _eig(ctx, fn, A, k)
        assert not sk.any(), (fn, n, k)
        assert _residual(A, Wk, Vk) < tol_res, (fn, n, k)
        assert _set_dist(W1, Wk) < tol_eig, (fn, n, k)


def test_cluster_setting_rejects_out_of_range():
    from scwatter_gb300 import _lib
    for bad in (-1, 9):
        with pytest.raises(_lib.ScwError):
            _lib.call("scw_set_qr_cluster", bad)


def test_mixed_solver_fallback_on_clusters(ctx):
    """scw_zgeev_mixed's FP64 QR fallback (only the matrices it does not accept, counted on the
    host) on clusters agrees with the one-CTA result."""
    import torch
    from scwatter_gb300 import _lib
    n = 200
    A = _matrices(3, n, seed=11)
    # a normal matrix with one eigenvalue 80 times over: a cluster above the refinement's 64
    # eigenvalues, so the FP64 QR solves it; the random ones are accepted
    rng = np.random.default_rng(7)
    S, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    lam = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    lam[:80] = 0.3 - 0.2j
    A[1] = (S * lam[None, :]) @ S.conj().T
    out = []
    for k in (1, 0):
        dA = torch.from_numpy(A).cuda()
        dW = torch.zeros((3, n), dtype=torch.complex128, device="cuda")
        dV = torch.zeros((3, n, n), dtype=torch.complex128, device="cuda")
        acc = np.zeros(3, np.int32)
        torch.cuda.synchronize()
        _lib.call("scw_set_qr_cluster", k)
        try:
            _lib.call("scw_zgeev_mixed", ctx.handle, n, _p(dA), _p(dW), _p(dV), 3, ctypes.c_void_p(acc.ctypes.data),
                      None, None)
        finally:
            _lib.call("scw_set_qr_cluster", 0)
        out.append((dW.cpu().numpy(), dV.cpu().numpy(), acc.copy()))
    (W1, V1, a1), (W0, V0, a0) = out
    assert a0[0] == 1 and a0[2] == 1 and a0[1] != 1, a0
    assert np.array_equal(a1, a0)
    assert _residual(A, W1, V1) < 1e-12
    assert _residual(A, W0, V0) < 1e-12
    assert _set_dist(W1, W0) < 1e-9


def test_fp64_qr_time_one_cta_vs_clusters(ctx):
    """Two n = 800 FP64 matrices: the QR sweeps on one CTA each against clusters (printed)."""
    A = _matrices(2, 800, seed=3)
    W1, V1, _, t1 = _eig(ctx, "scw_zgeev", A, 1)
    W0, V0, _, t0 = _eig(ctx, "scw_zgeev", A, 0)
    print(f"scw_zgeev n=800 x2: one CTA per matrix {t1:.3f} s, clusters {t0:.3f} s ({t1 / t0:.2f}x)")
    assert _residual(A, W0, V0) < 1e-12
    assert _set_dist(W1, W0) < 1e-9
