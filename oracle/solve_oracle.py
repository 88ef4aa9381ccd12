"""FP64 CPU oracle for scwatter's per-layer coupled-wave solve.

TEST INFRASTRUCTURE ONLY.  This module is the checker that the GPU solve and the
``.cw`` writer are compared against.  Only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.
The product (``scwatter_gb300``) never calls into it.

It restates, in numpy/scipy double precision, the solve of the reference program
``sCWatter`` (STIM-Lab/scwatter):

* ``FourierWave.h:18``        ``PI = 3.141592653`` (truncated on purpose: used for k and the k-grids)
* ``FourierWave.h:32-39``     ``orthogonalize``
* ``FourierWave.h:82-145``    ``fftShift2d`` (including its parity quirk for even rows / odd columns)
* ``FourierWave.h:152-195``   ``fftw_fft2`` (forward DFT / (N1 N2), shift, centred M1 x M0 crop)
* ``FourierWave.h:283-301``   ``volume::reformat`` (slice i = column-major Y x X map of C-order data)
* ``FourierWave.h:319-334``   ``UpWq_Cal`` (k-grids, principal complex sqrt for Sz)
* ``FourierWave.h:336-397``   ``volume::phi`` (dense 4MF x 4MF coupled-wave matrix, wrapped harmonic differences)
* ``third_Lapack.h:38-87``    zgeev('N','V') / zgesv / zgemm  -> scipy LAPACK (zgeev) and numpy (zgesv, matmul)
* ``sCWatter.cpp:157-163``    ``InitLayer_z``
* ``sCWatter.cpp:172-225``    ``sorter`` / ``Eigen_Sort`` (even slots: largest Im first, odd slots: smallest Im first)
* ``sCWatter.cpp:230-332``    ``EigenDecompositionD`` (Gd / Gc, cascade Gc_static)
* ``sCWatter.cpp:334-390``    ``MatTransfer`` (f1, f2, f3)
* ``sCWatter.cpp:393-461``    ``SetGaussianConstraints``, ``SetBoundaryConditions``
* ``sCWatter.cpp:464-488``    ``mat2waves``
* ``sCWatter.cpp:569-956``    ``main``: direction / polarisation set-up, M clamping, incident FFT,
                              zgesv, beta, Q_check / Q_hat, Ez from the magnetic field, packing

Parity status: the reference ships no golden vectors, fixtures or tests, and it cannot
be built here (tira, Eigen, FFTW, MKL, Boost and glm are absent).  So this oracle is
pinned by physics known answers instead (Fresnel coefficients, a homogeneous slab
against an independent transfer-matrix solution, tangential-field continuity across
every boundary, energy balance) -- "parity unpinned" with respect to reference
outputs.

Assumption about the absent third-party type ``tira::planewave<double>``: its raw
bytes are ``E0.xyz`` then ``k.xyz`` (complex, re/im interleaved), as the layout
comment in ``CoupledWaveStructure.h:7-55`` states, the constructor
``planewave(kx, ky, kz, Ex, Ey, Ez)`` stores k and E0 unchanged, and
``wind(0, 0, -z)`` multiplies E0 by ``exp(-i kz z)`` (the only sign under which the
reference's own boundary printout in ``sCWatterLayer.cpp:524-527`` is continuous).
"""
from __future__ import annotations

import functools
import math
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg

PI_REF = 3.141592653          # FourierWave.h:18
DBL_EPS = np.finfo(np.float64).eps


# --------------------------------------------------------------------------------------
# FourierWave.h helpers
# --------------------------------------------------------------------------------------
def _cross(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1],
                     a[2] * b[0] - a[0] * b[2],
                     a[0] * b[1] - a[1] * b[0]], dtype=np.complex128)


def orthogonalize(E, d):
    """FourierWave.h:32-39.  |E| is the complex sqrt of sum(E_i^2) (not the Hermitian norm)."""
    E = np.asarray(E, dtype=np.complex128)
    mag = np.sqrt(E[0] ** 2 + E[1] ** 2 + E[2] ** 2)
    E = E / mag
    dc = np.asarray(d, dtype=np.complex128)
    s = _cross(E, dc)
    return _cross(dc, s)


def fft_shift_2d(mat):
    """FourierWave.h:82-145.  Matches numpy.fft.fftshift except when rows are even and
    columns odd, where the reference builds a non-permutation column index (reproduced)."""
    m, n = mat.shape
    if m % 2 == 1:
        p, q = m // 2, n // 2
    else:
        p, q = (m + 1) // 2, (n + 1) // 2
    indx = np.empty(m, dtype=np.int64)
    indy = np.empty(n, dtype=np.int64)
    if m % 2 == 1:
        for i in range(m):
            indx[i] = (m - p) + i if i < m - p - 1 else i - (m - p - 1)
    else:
        for i in range(m):
            indx[i] = p + i if i < m - p else i - (m - p)
    if n % 2 == 1:
        for i in range(n):
            indy[i] = (n - q) + i if i < n - q - 1 else i - (n - q - 1)
    else:
        for i in range(n):
            indy[i] = q + i if i < n - q else i - (n - q)
    return mat[np.ix_(indx, indy)]


def fft2_crop(A, M1, M2):
    """FourierWave.h:152-195: forward 2-D DFT scaled by 1/(N1 N2), fftShift2d, centred crop."""
    N1, N2 = A.shape
    B = np.fft.fft2(np.asarray(A, dtype=np.complex128)) / N1 / N2
    S = fft_shift_2d(B)
    r0 = N1 // 2 - M1 // 2
    c0 = N2 // 2 - M2 // 2
    return S[r0:r0 + M1, c0:c0 + M2].copy()


def reformat(sample):
    """FourierWave.h:283-301.  Slice i is an Eigen column-major (Y x X) map of the C-order
    slice data: S[r, c] = flat[r + c*Y]."""
    sample = np.asarray(sample, dtype=np.complex128)
    if sample.ndim == 2:
        sample = sample[None]
    Z, Y, X = sample.shape
    return [sample[i].reshape(-1).reshape(X, Y).T.copy() for i in range(Z)], (Z, Y, X)


def series(M):
    """Eigen setLinSpaced(M, -(M/2), (M-1)/2) with C++ integer division."""
    lo, hi = -float(M // 2), float((M - 1) // 2)
    if M == 1:
        return np.array([hi])
    step = (hi - lo) / (M - 1)
    return lo + np.arange(M) * step


# --------------------------------------------------------------------------------------
# Solve
# --------------------------------------------------------------------------------------
@dataclass
class SolveParams:
    lam: float = 1.0
    direction: tuple = (0.0, 0.0, 1.0)
    ex: tuple = (0.0, 0.0)
    ey: tuple = (1.0, 0.0)
    ez: tuple = (0.0, 0.0)
    n: tuple = (1.0, 1.0)
    kappa: tuple = (0.0,)
    size: tuple = (10.0, 10.0, 2.0)
    z: float = 0.0
    coef: tuple | None = None
    external: bool = False
    pz: bool = True          # False == the reference's --npz flag
    psf: bool = False        # the reference's --psf flag (sCWatter.cpp:665-669)


@dataclass
class SolveResult:
    M: tuple
    MF: int
    k: float
    z: np.ndarray                      # ZL boundary coordinates
    dir: np.ndarray                    # normalised direction * n0
    Sx: np.ndarray
    Sy: np.ndarray
    Sz0: np.ndarray
    Sz1: np.ndarray
    EF: np.ndarray                     # 3MF incident Fourier amplitudes
    x: np.ndarray                      # 6MF boundary solution (R xyz, T xyz)
    eigenvalues: list                  # sorted, per slice (4MF)
    eigenvectors: list                 # sorted, per slice (4MF x 4MF)
    Q_check: list = field(default_factory=list)   # per slice, 3MF x 2MF (downward, ref at top)
    Q_hat: list = field(default_factory=list)     # per slice, 3MF x 2MF (upward, ref at bottom)
    NIf: list = field(default_factory=list)
    Phi: list = field(default_factory=list)
    beta: list = field(default_factory=list)
    warnings: list = field(default_factory=list)


def clamp_coef(coef, shape, size, lam, dirn, n):
    """sCWatter.cpp:594-645 (M selection and clamping, including its warnings)."""
    Z, Y, X = shape
    warns = []
    if coef is None or len(coef) == 0:
        M0, M1 = X, Y
    elif len(coef) == 1:
        M0 = M1 = int(math.sqrt(coef[0]))
    else:
        M0, M1 = int(coef[0]), int(coef[1])
    if (float(M0 // 2) / size[0] * lam + dirn[0]) ** 2 + (float(M1 // 2) / size[1] * lam + dirn[1]) ** 2 >= n[0] ** 2:
        warns.append("cutting off invalid waves with imaginary sz")
        if M0 != 1 and M1 != 1:
            if (float(M0 // 2) / size[0] * lam + dirn[0]) > 0.71 * n[0]:
                M0 = int(0.707 * n[0] * 2 * size[0] / lam) - 1
            if (float(M1 // 2) / size[1] * lam + dirn[1]) > 0.71 * n[0]:
                M1 = int(0.707 * n[1] * 2 * size[1] / lam) - 1
        if M0 == 1:
            if (float(M1 // 2) / size[1] * lam + abs(dirn[1])) >= n[0]:
                M1 = int(n[1] * 2 * size[1] / lam - 1e-10)
                if M1 % 2 == 0:
                    M1 -= 1
        if M1 == 1:
            if (float(M0 // 2) / size[1] * lam + abs(dirn[0])) >= n[0]:
                M0 = int(n[0] * 2 * size[0] / lam - 1e-10)
                if M0 % 2 == 0:
                    M0 -= 1
    if M0 > X:
        M0 = X
    if M1 > Y:
        M1 = Y
    return (M0, M1), warns


def _sorter_cmp(a, b):
    """sCWatter.cpp:172-179 (epsilon tie-break on the imaginary, then the real part)."""
    if abs(a.imag - b.imag) > DBL_EPS:
        return -1 if a.imag < b.imag else (1 if a.imag > b.imag else 0)
    if abs(a.real - b.real) > DBL_EPS:
        return -1 if a.real < b.real else (1 if a.real > b.real else 0)
    return -1 if a.imag < b.imag else (1 if a.imag > b.imag else 0)


def eigen_sort(evl, evt):
    """sCWatter.cpp:185-225: slot 2i <- i-th largest Im, slot 2i+1 <- i-th smallest Im."""
    n = len(evl)
    order = sorted(range(n), key=functools.cmp_to_key(lambda i, j: _sorter_cmp(evl[i], evl[j])))
    perm = np.empty(n, dtype=np.int64)
    for i in range(n // 2):
        perm[2 * i] = order[n - 1 - i]
        perm[2 * i + 1] = order[i]
    return evl[perm].copy(), evt[:, perm].copy()


def build_phi(S, M, up, wq, k, p_series, q_series):
    """FourierWave.h:336-397 for one slice S (Y x X, column-major view).  Returns Phi, Nif."""
    M0, M1 = M
    MF = M0 * M1
    Nf = fft2_crop(S ** 2, M1, M0)
    Nif = fft2_crop((1.0 / S) ** 2, M1, M0)
    qi_s = q_series.astype(np.int64)
    pi_s = p_series.astype(np.int64)
    # wrapped differences (C++ % on the integer series values, then +M/2, mod M)
    dq = (np.fmod(qi_s[:, None], M1) - np.fmod(qi_s[None, :], M1) + M1) % M1
    dp = (np.fmod(pi_s[:, None], M0) - np.fmod(pi_s[None, :], M0) + M0) % M0
    R = (dq + M1 // 2) % M1                         # [qi, qj]
    C = (dp + M0 // 2) % M0                         # [pi, pj]
    # harmonic index m = q*M0 + p
    Rm = np.repeat(np.repeat(R, M0, axis=0), M0, axis=1)   # [(qi,pi), (qj,pj)] -> R[qi,qj]
    Cm = np.tile(C, (M1, M1))                               # -> C[pi,pj]
    A0 = Nf[Rm, Cm]
    NI = Nif[Rm, Cm]
    up_m = np.tile(up, M1).astype(np.complex128)          # up[p] for m = q*M0+p
    wq_m = np.repeat(wq, M0).astype(np.complex128)        # wq[q]
    A1 = up_m[None, :] * NI
    A2 = wq_m[None, :] * NI
    k_inv = 1.0 / k ** 2
    Phi = np.zeros((4 * MF, 4 * MF), dtype=np.complex128)
    upc = up_m[:, None]
    wqc = wq_m[:, None]
    Phi[0:MF, 2 * MF:3 * MF] = upc * k_inv * A2
    Phi[0:MF, 3 * MF:4 * MF] = -upc * k_inv * A1
    Phi[MF:2 * MF, 2 * MF:3 * MF] = wqc * k_inv * A2
    Phi[MF:2 * MF, 3 * MF:4 * MF] = -wqc * k_inv * A1
    Phi[2 * MF:3 * MF, MF:2 * MF] = -A0
    Phi[3 * MF:4 * MF, 0:MF] = A0
    ar = np.arange(MF)
    Phi[ar, 3 * MF + ar] += 1
    Phi[MF + ar, 2 * MF + ar] += -1
    Phi[2 * MF + ar, ar] += -up_m * wq_m * k_inv
    Phi[2 * MF + ar, MF + ar] += up_m * up_m * k_inv
    Phi[3 * MF + ar, ar] += -wq_m * wq_m * k_inv
    Phi[3 * MF + ar, MF + ar] += up_m * wq_m * k_inv
    return Phi, Nif


def solve(sample, prm: SolveParams, keep_phi: bool = False) -> SolveResult:
    """Restatement of ``sCWatter`` ``main`` (sCWatter.cpp:569-885) up to the packing."""
    slices, shape = reformat(sample)
    Z, Y, X = shape
    n = list(prm.n)
    L = len(n)
    if L != 2:
        raise ValueError("the volume solver takes exactly two media (upper, lower)")
    dvec = np.asarray(prm.direction, dtype=np.float64)
    dvec = dvec / np.linalg.norm(dvec)
    e = np.array([complex(*prm.ex), complex(*prm.ey), complex(*prm.ez)])
    e = orthogonalize(e, dvec)
    dirn = dvec * n[0]
    k = 2 * PI_REF / prm.lam
    ni = [complex(n[0], 0.0), complex(n[1], prm.kappa[0])]
    ZL = Z + 1
    size = list(prm.size)
    zb = np.empty(ZL)
    zb[0] = prm.z - size[2] / 2.0
    for i in range(1, ZL):
        zb[i] = zb[i - 1] + size[2] / Z
    M, warns = clamp_coef(prm.coef, shape, size, prm.lam, dirn, n)
    M0, M1 = M
    MF = M0 * M1

    # UpWq_Cal (FourierWave.h:319-334)
    p_series = series(M0)
    q_series = series(M1)
    up = 2 * PI_REF * p_series / size[0] + dirn[0] * k
    wq = 2 * PI_REF * q_series / size[1] + dirn[1] * k
    Sxv = (up / k).astype(np.complex128)
    Syv = (wq / k).astype(np.complex128)
    meshS0 = np.tile(Sxv[None, :], (M1, 1))
    meshS1 = np.tile(Syv[:, None], (1, M0))
    Sz0m = np.sqrt(ni[0] ** 2 - meshS0 ** 2 - meshS1 ** 2)
    Sz1m = np.sqrt(ni[1] ** 2 - meshS0 ** 2 - meshS1 ** 2)
    # sCWatter.cpp:677-680: column-major flattening of the M1 x M0 meshes
    Sx = meshS0.flatten(order="F")
    Sy = meshS1.flatten(order="F")
    Sz0 = Sz0m.flatten(order="F")
    Sz1 = Sz1m.flatten(order="F")

    # incident field (sCWatter.cpp:656-674)
    EF = np.concatenate([fft2_crop(e[c] * np.ones((Y, X)), M1, M0).flatten(order="F") for c in range(3)])
    if prm.psf:     # sCWatter.cpp:665-669: every harmonic carries E0
        EF = np.concatenate([np.full(MF, e[c]) for c in range(3)])

    # CalculateD + EigenDecompositionD
    evals, evecs, NIfs, Phis = [], [], [], []
    for i in range(Z):
        Phi, Nif = build_phi(slices[i], M, up, wq, k, p_series, q_series)
        NIfs.append(Nif)
        if keep_phi:
            Phis.append(Phi)
        w, V = scipy.linalg.eig(Phi, left=False, right=True, overwrite_a=True, check_finite=False)
        w, V = eigen_sort(w, V)
        evals.append(w)
        evecs.append(V)

    GD, GC = [], []
    Gd_static = Gc_static = None
    for i in range(Z):
        lamv = evals[i]
        if Z == 1:
            dz = zb[ZL - 1] - zb[0]
        else:
            dz = zb[i + 1] - zb[i]
        Ci = np.exp(1j * k * lamv * dz)
        Di = np.exp(1j * k * lamv * (-dz)) if Z == 1 else np.exp(1j * k * lamv * (zb[i] - zb[i + 1]))
        odd = (np.arange(4 * MF) % 2) == 1
        Gd = evecs[i] * np.where(odd, Di, 1.0)[None, :]
        Gc = evecs[i] * np.where(odd, 1.0, Ci)[None, :]
        if not prm.external:
            GD.append(Gd)
            GC.append(Gc)
        if i == 0:
            Gd_static, Gc_static = Gd, Gc
        else:
            tmp = np.linalg.solve(Gd, np.eye(4 * MF))
            Gc_static = (Gc @ tmp) @ Gc_static

    # MatTransfer (sCWatter.cpp:334-390)
    I = np.eye(MF)
    phase = np.exp(1j * k * zb[0] * Sz0)
    f1 = np.zeros((4 * MF, 3 * MF), dtype=np.complex128)
    f2 = np.zeros_like(f1)
    f3 = np.zeros_like(f1)
    f1[0:MF, 0:MF] = np.diag(phase)
    f1[MF:2 * MF, MF:2 * MF] = np.diag(phase)
    f1[2 * MF:3 * MF, MF:2 * MF] = -np.diag(phase * Sz0)
    f1[2 * MF:3 * MF, 2 * MF:3 * MF] = np.diag(phase * Sy)
    f1[3 * MF:4 * MF, 0:MF] = np.diag(phase * Sz0)
    f1[3 * MF:4 * MF, 2 * MF:3 * MF] = -np.diag(phase * Sx)
    f2[0:MF, 0:MF] = I
    f2[MF:2 * MF, MF:2 * MF] = I
    f2[2 * MF:3 * MF, MF:2 * MF] = np.diag(Sz0)
    f2[2 * MF:3 * MF, 2 * MF:3 * MF] = np.diag(Sy)
    f2[3 * MF:4 * MF, 0:MF] = -np.diag(Sz0)
    f2[3 * MF:4 * MF, 2 * MF:3 * MF] = -np.diag(Sx)
    f3[0:MF, 0:MF] = -I
    f3[MF:2 * MF, MF:2 * MF] = -I
    f3[2 * MF:3 * MF, MF:2 * MF] = np.diag(Sz1)
    f3[2 * MF:3 * MF, 2 * MF:3 * MF] = -np.diag(Sy)
    f3[3 * MF:4 * MF, 0:MF] = -np.diag(Sz1)
    f3[3 * MF:4 * MF, 2 * MF:3 * MF] = np.diag(Sx)

    # InitMatrices + SetGaussianConstraints + SetBoundaryConditions (sCWatter.cpp:143-146, 393-461)
    A = np.zeros((6 * MF, 6 * MF), dtype=np.complex128)
    b = np.zeros(6 * MF, dtype=np.complex128)
    ar = np.arange(MF)
    A[ar, ar] = Sx
    A[ar, MF + ar] = Sy
    A[ar, 2 * MF + ar] = -Sz0
    A[MF + ar, 3 * MF + ar] = Sx
    A[MF + ar, 4 * MF + ar] = Sy
    A[MF + ar, 5 * MF + ar] = Sz1
    Gc_inv = np.linalg.solve(Gc_static, np.eye(4 * MF))
    A[2 * MF:6 * MF, 0:3 * MF] = f2
    A[2 * MF:6 * MF, 3 * MF:6 * MF] = (Gd_static @ Gc_inv) @ f3
    b[2 * MF:6 * MF] = -(f1 @ EF)
    x = np.linalg.solve(A, b)                     # MKL_linearsolve (sCWatter.cpp:722)

    res = SolveResult(M=M, MF=MF, k=k, z=zb, dir=dirn, Sx=Sx, Sy=Sy, Sz0=Sz0, Sz1=Sz1,
                      EF=EF, x=x, eigenvalues=evals, eigenvectors=evecs, NIf=NIfs,
                      Phi=Phis, warnings=warns)
    if prm.external:
        return res

    # beta (sCWatter.cpp:743-777)
    betas = []
    beta = None
    for i in range(Z):
        if i == 0:
            tmp = np.linalg.solve(GD[0], np.eye(4 * MF))
            beta = (tmp @ f1) @ EF + (tmp @ f2) @ x[0:3 * MF]
        else:
            tmp = np.linalg.solve(GD[i], np.eye(4 * MF))
            beta = (tmp @ GC[i - 1]) @ beta
        betas.append(beta)
    res.beta = betas

    # Q_check / Q_hat and Ez from H (sCWatter.cpp:781-885)
    WQ = 2.0 * q_series * math.pi / size[1]
    UP = 2.0 * p_series * math.pi / size[0]
    up_pz = np.tile(UP + dirn[0] * k, M1)            # indexed by m = q*M0 + p
    wq_pz = np.repeat(WQ + dirn[1] * k, M0)
    qi = np.repeat(np.arange(M1), M0)
    pi = np.tile(np.arange(M0), M1)
    for i in range(Z):
        V = evecs[i]
        Q1 = V[:, 0::2] * betas[i][0::2][None, :]
        Q2 = V[:, 1::2] * betas[i][1::2][None, :]
        Qc = np.zeros((3 * MF, 2 * MF), dtype=np.complex128)
        Qh = np.zeros((3 * MF, 2 * MF), dtype=np.complex128)
        Qc[0:2 * MF] = Q1[0:2 * MF]
        Qh[0:2 * MF] = Q2[0:2 * MF]
        if prm.pz:
            I1, J1 = Q1[2 * MF:3 * MF], Q1[3 * MF:4 * MF]
            I2, J2 = Q2[2 * MF:3 * MF], Q2[3 * MF:4 * MF]
            indR = (qi[:, None] - qi[None, :] + M1) % M1
            indC = (pi[:, None] - pi[None, :] + M0) % M0
            lin = ((indR + M1 // 2) % M1) * M0 + (indC + M0 // 2) % M0
            Kn = NIfs[i].flatten(order="F")[lin]                      # NIf[i](linear index)
            Qc[2 * MF:3 * MF] = (-1.0 / k) * (Kn @ (up_pz[:, None] * J1 - wq_pz[:, None] * I1))
            Qh[2 * MF:3 * MF] = (-1.0 / k) * (Kn @ (up_pz[:, None] * J2 - wq_pz[:, None] * I2))
        res.Q_check.append(Qc)
        res.Q_hat.append(Qh)
    return res


# --------------------------------------------------------------------------------------
# Packing into the .cw structure (sCWatter.cpp:890-956, 464-488)
# --------------------------------------------------------------------------------------
@dataclass
class CW:
    """In-memory CoupledWaveStructure<double> (CoupledWaveStructure.h:57-71).
    Each wave is a row [E0x, E0y, E0z, kx, ky, kz] of complex128."""
    Pi: np.ndarray
    z: list
    Pr: list
    Pt: list


def _wind(waves, zl):
    """tira::planewave::wind(0, 0, -z): E0 <- E0 * exp(-i kz z)."""
    out = waves.copy()
    out[:, 0:3] *= np.exp(-1j * out[:, 5] * zl)[:, None]
    return out


def pack(res: SolveResult, prm: SolveParams) -> CW:
    M0, M1 = res.M
    MF = res.MF
    k = res.k
    n_in = list(prm.n)
    Z = len(res.eigenvalues)
    ZL = Z + 1
    x = res.x
    Pi = np.zeros((MF, 6), dtype=np.complex128)
    Pr = [[] for _ in range(ZL)]
    Pt = [[] for _ in range(ZL)]
    zs = [0.0] * ZL
    for kk in range(M1):
        for j in range(M0):
            p = kk * M0 + j
            kx, ky = res.Sx[p] * k, res.Sy[p] * k
            Pi[p] = [res.EF[p], res.EF[MF + p], res.EF[2 * MF + p], kx, ky, res.Sz0[p] * k]
            r = np.array([[x[p], x[MF + p], x[2 * MF + p], kx, ky, -res.Sz0[p] * k * n_in[0]]])
            t = np.array([[x[3 * MF + p], x[4 * MF + p], x[5 * MF + p], kx, ky, res.Sz1[p] * k * n_in[1]]])
            for l in range(ZL):
                if l == 0:
                    zs[l] = res.z[l]
                    Pr[l].append(_wind(r, res.z[l]))
                    if not prm.external:
                        Qc = res.Q_check[l]
                        w = np.stack([Qc[p], Qc[MF + p], Qc[2 * MF + p],
                                      np.full(2 * MF, kx), np.full(2 * MF, ky),
                                      res.eigenvalues[l][0::2] * k], axis=1)
                        Pt[l].append(_wind(w, res.z[l]))
                elif l == ZL - 1:
                    zs[l] = res.z[l]
                    Pt[l].append(_wind(t, res.z[l]))
                    if not prm.external:
                        Qh = res.Q_hat[l - 1]
                        w = np.stack([Qh[p], Qh[MF + p], Qh[2 * MF + p],
                                      np.full(2 * MF, kx), np.full(2 * MF, ky),
                                      res.eigenvalues[l - 1][1::2] * k], axis=1)
                        Pr[l].append(_wind(w, res.z[l]))
                else:
                    if not prm.external:
                        Qh = res.Q_hat[l - 1]
                        w = np.stack([Qh[p], Qh[MF + p], Qh[2 * MF + p],
                                      np.full(2 * MF, kx), np.full(2 * MF, ky),
                                      res.eigenvalues[l - 1][1::2] * k], axis=1)
                        Pr[l].append(_wind(w, res.z[l]))
                        Qc = res.Q_check[l]
                        w = np.stack([Qc[p], Qc[MF + p], Qc[2 * MF + p],
                                      np.full(2 * MF, kx), np.full(2 * MF, ky),
                                      res.eigenvalues[l][0::2] * k], axis=1)
                        Pt[l].append(_wind(w, res.z[l]))
                        zs[l] = res.z[l]
    cat = lambda lst: np.concatenate(lst, axis=0) if lst else np.zeros((0, 6), dtype=np.complex128)
    return CW(Pi=Pi, z=zs, Pr=[cat(v) for v in Pr], Pt=[cat(v) for v in Pt])


# --------------------------------------------------------------------------------------
# .cw bytes (CoupledWaveStructure.h:72-134), double precision records of 12 doubles
# --------------------------------------------------------------------------------------
def cw_to_bytes(cw: CW) -> bytes:
    def rec(w):
        w = np.ascontiguousarray(w, dtype=np.complex128)
        return w.view(np.float64).tobytes()
    out = [np.uint64(8).tobytes(), np.uint64(len(cw.Pi)).tobytes(), rec(cw.Pi),
           np.uint64(len(cw.z)).tobytes()]
    for l in range(len(cw.z)):
        out.append(np.float64(cw.z[l]).tobytes())
        out.append(np.uint64(len(cw.Pr[l])).tobytes())
        out.append(rec(cw.Pr[l]))
        out.append(np.uint64(len(cw.Pt[l])).tobytes())
        out.append(rec(cw.Pt[l]))
    return b"".join(out)


def cw_from_bytes(buf: bytes) -> CW:
    off = 0

    def u64():
        nonlocal off
        v = int(np.frombuffer(buf, dtype=np.uint64, count=1, offset=off)[0])
        off += 8
        return v

    def f64():
        nonlocal off
        v = float(np.frombuffer(buf, dtype=np.float64, count=1, offset=off)[0])
        off += 8
        return v

    def waves(n):
        nonlocal off
        a = np.frombuffer(buf, dtype=np.float64, count=12 * n, offset=off).reshape(n, 12)
        off += 96 * n
        return a.view(np.complex128).reshape(n, 6).copy()

    u64()                       # precision (ignored, CoupledWaveStructure.h:107-108)
    Pi = waves(u64())
    nl = u64()
    zs, Pr, Pt = [], [], []
    for _ in range(nl):
        zs.append(f64())
        Pr.append(waves(u64()))
        Pt.append(waves(u64()))
    return CW(Pi=Pi, z=zs, Pr=Pr, Pt=Pt)


# --------------------------------------------------------------------------------------
# cw_allocate / cw_unpack (cpuEvaluator.cpp:34-102)
# --------------------------------------------------------------------------------------
def unpack(cw: CW, dtype=np.complex128):
    """Returns (W [n, 6], waves_begin [L+1], waves_end [L+1], z_layers [L])."""
    layers = len(cw.z)
    begin = [0]
    end = []
    total = len(cw.Pi)
    for l in range(layers):
        total += len(cw.Pr[l])
        end.append(total)
        begin.append(total)
        total += len(cw.Pt[l])
    end.append(total)
    parts = [cw.Pi]
    for l in range(layers):
        parts.append(cw.Pr[l])
        parts.append(cw.Pt[l])
    W = np.concatenate(parts, axis=0).astype(dtype)
    return W, np.array(begin, dtype=np.int64), np.array(end, dtype=np.int64), np.array(cw.z, dtype=np.float64)
