"""CPU restatement of the mixed-precision eigen-solver (test infrastructure only).

``refine`` follows scwatter_gb300/csrc/eig_mixed.cu in FP64 numpy, starting from FP32
eigenpairs (LAPACK cgeev through numpy stands in for the FP32 Householder + QR stage):

* clusters: connected components of |lambda_i - lambda_j| < tau_rel ||A||_1 (cluster_kernel);
* per step: R = A X - X diag(lambda) in FP64, max relative column residual
  ||r_i|| / (||A||_1 ||x_i||) as the gate (resid_kernel, gate_kernel); E = X^-1 R with X and R
  rounded to FP32; singletons lambda_i += E_ii; each cluster's block diag(lambda_S) + E_SS
  solved by a complex Schur decomposition with pairs closer than deg_rel ||A||_1 left uncoupled
  (cluster_eig_kernel); F_ij = E_ij / (lambda_j - lambda_i) between clusters (f_kernel);
  X += X F with an FP32 product (xupdate_kernel); cluster columns rotated by their block's
  eigenvectors (rotate_kernel);
* stop at tol; from step ``steps`` on accept at tol_accept; after the last step (``steps``, or
  ``steps_large`` for matrices of order >= ``large_n``) the FP64 solver.

The reference solves the same eigenproblems with LAPACKE_zgeev (third_Lapack.h:38-47); the
tests compare the refined eigenvalues with numpy's FP64 LAPACK ones.
"""
import numpy as np
import scipy.linalg


def clusters(lam, tau):
    """Labels: the smallest index of each connected component of |lam_i - lam_j| < tau."""
    n = len(lam)
    lab = np.arange(n)
    near = np.abs(lam[:, None] - lam[None, :]) < tau
    for _ in range(64):
        new = np.array([lab[near[i]].min() for i in range(n)])
        new = new[new]
        if (new == lab).all():
            return lab
        lab = new
    return None


def cluster_eig(M, deg):
    """Eigenvalues and eigenvectors of a small cluster block: Schur form, then the triangular
    eigenvectors with pairs closer than deg left uncoupled (the unitary Schur basis kept)."""
    T, U = scipy.linalg.schur(M, output="complex")
    k = T.shape[0]
    Y = np.eye(k, dtype=complex)
    for j in range(k):
        for i in range(j - 1, -1, -1):
            d = T[i, i] - T[j, j]
            Y[i, j] = 0.0 if abs(d) <= deg else -(T[i, i + 1:j + 1] @ Y[i + 1:j + 1, j]) / d
    return np.diag(T).copy(), U @ Y


def refine(A, lam32, X32, steps=10, tau_rel=1e-5, deg_rel=1e-12, tol=1e-14, tol_accept=1e-12, max_cluster=64,
           steps_large=16, large_n=1600):
    """Returns (accepted, lam, X, residual per check).  Matrices of order >= large_n refine for up
    to steps_large steps; from step ``steps`` on a slice is accepted at tol_accept (eig_mixed.cu)."""
    A = np.asarray(A, np.complex128)
    nA = np.linalg.norm(A, 1)
    lam = np.asarray(lam32).astype(np.complex128)
    X = np.asarray(X32).astype(np.complex128)
    lab = clusters(lam, tau_rel * nA)
    if lab is None:
        return False, lam, X, []
    sizes = np.bincount(lab, minlength=len(lam))
    if sizes.max() > max_cluster:
        return False, lam, X, []
    groups = [np.where(lab == c)[0] for c in np.unique(lab) if sizes[c] > 1]
    same = lab[:, None] == lab[None, :]
    single = sizes[lab] == 1
    hist = []
    last = max(steps, steps_large) if A.shape[0] >= large_n else steps
    for s in range(last + 1):
        R = A @ X - X * lam[None, :]
        res = (np.linalg.norm(R, axis=0) / np.linalg.norm(X, axis=0)).max() / nA
        hist.append(res)
        if res <= (tol_accept if s >= steps else tol):
            return True, lam, X, hist
        if s == last:
            return False, lam, X, hist
        X32s = X.astype(np.complex64)
        # E = X^-1 R by LAPACK's single-precision LU (cgesv).  numpy.linalg.solve would compute
        # in double precision for complex64 input and round, which is not what the GPU does.
        try:                                   # a singular eigenvector matrix: lu_check_kernel's refusal
            E = scipy.linalg.solve(X32s, R.astype(np.complex64), check_finite=False).astype(np.complex128)
        except (np.linalg.LinAlgError, scipy.linalg.LinAlgError):
            return False, lam, X, hist
        lam = lam + np.where(single, np.diag(E), 0)
        Ys = []
        for g in groups:
            d, Y = cluster_eig(np.diag(lam[g]) + E[np.ix_(g, g)], deg_rel * nA)
            lam[g] = d
            Ys.append(Y)
        den = lam[None, :] - lam[:, None]
        F = np.where(same, 0, E / np.where(same | (den == 0), 1, den))
        X = X + (X32s @ F.astype(np.complex64)).astype(np.complex128)
        for g, Y in zip(groups, Ys):
            X[:, g] = X[:, g] @ Y
    return False, lam, X, hist
