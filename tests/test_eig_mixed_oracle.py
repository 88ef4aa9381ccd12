"""The mixed-precision eigen-solver's method, restated on the CPU (oracle/eig_mixed_oracle.py),
on reduced layer matrices of the workloads: FP32 eigenpairs refined to FP64 residuals, the
eigenvalues matching FP64 LAPACK, and a defective matrix refused."""
import numpy as np
import pytest
import scipy.linalg

from oracle import eig_mixed_oracle as emo
from oracle import solve_oracle as so
from scwatter_gb300 import samples


def _pq(vol, coef, lam=1.0, size=None, direction=(0.0, 0.0, 1.0)):
    """Reduced matrices P Q (Phi = [[0, P], [Q, 0]], FourierWave.h:336-397) of every slice."""
    slices, shape = so.reformat(vol)
    Z, Y, X = shape
    size = size or (float(X), float(Y))
    k = 2 * so.PI_REF / lam
    M0, M1 = coef
    p, q = so.series(M0), so.series(M1)
    d = np.asarray(direction, float)
    d = d / np.linalg.norm(d)
    up = 2 * so.PI_REF * p / size[0] + d[0] * k
    wq = 2 * so.PI_REF * q / size[1] + d[1] * k
    MF = M0 * M1
    out = []
    for i in range(Z):
        Phi, _ = so.build_phi(slices[i], (M0, M1), up, wq, k, p, q)
        out.append(Phi[:2 * MF, 2 * MF:] @ Phi[2 * MF:, :2 * MF])
    return out


def _eig32(A):
    """Eigenpairs from LAPACK's single-precision cgeev.  (numpy.linalg.eig on complex64 input
    computes in double precision and rounds the result, which is not an FP32 start.)"""
    lam32, X32 = scipy.linalg.eig(A.astype(np.complex64), check_finite=False)
    assert lam32.dtype == np.complex64 and X32.dtype == np.complex64
    return lam32, X32


def _check(A, tol_eig=1e-11):
    lam32, X32 = _eig32(A)
    ok, lam, X, hist = emo.refine(A, lam32, X32)
    assert ok, hist
    assert hist[0] > 1e-9 and hist[-1] <= 1e-12          # from FP32 quality to FP64 quality
    ref = np.linalg.eigvals(A)
    nA = np.linalg.norm(A, 1)
    assert np.abs(lam[:, None] - ref[None, :]).min(axis=1).max() < tol_eig * nA
    assert np.linalg.cond(X) < 1e6
    return len(hist) - 1


def test_sphere_layers():
    vol = samples.spheres((3, 32, 32), n_spheres=3, radius=(4.0, 9.0), seed=1)
    for A in _pq(vol, (8, 8), direction=(0.1, 0.05, 1.0)):
        assert _check(A) <= 10


def test_homogeneous_layer_with_degenerate_eigenvalues():
    # normal incidence on a square grid: every eigenvalue of PQ is (kx^2 + ky^2 - eps) with
    # multiplicity up to 16 (x / y blocks and the grid's symmetries)
    A = _pq(np.full((1, 16, 16), 1.4 + 0.01j), (8, 8))[0]
    _check(A)


def test_grf_layer():
    vol = samples.gaussian_random_field((2, 32, 32), corr_px=6.0, seed=4)
    for A in _pq(vol, (8, 8), direction=(0.2, 0.1, 1.0)):
        _check(A)


def test_jordan_block_is_refused():
    n = 24
    J = np.diag(np.full(n, 0.5 + 0.1j)) + np.diag(np.ones(n - 1), 1)
    lam32, X32 = _eig32(J)
    ok, lam, X, hist = emo.refine(J, lam32, X32)
    assert not ok
