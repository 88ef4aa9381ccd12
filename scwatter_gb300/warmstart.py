"""Learned eigen warm start for the per-layer eigen-solve.

A small network (3 fully connected layers, ReLU, FP32; its own CUDA forward, backward and
Adam kernels in csrc/mlp.cu) maps a layer's Fourier coefficients (the crops of n^2 and
n^-2) to that layer's eigenvalues lambda = gamma^2 of the reduced matrix PQ,
sorted by descending real part.  It predicts the correction to the homogeneous-medium spectrum
lambda0 = <n^2> - (up^2 + wq^2) / k^2 (every harmonic twice, one per polarisation) sorted the same
way, the guess used without it.  The predicted eigenvalues are the shifts of the warm eigen-solver, each task
starting from the plane-wave mode of its slot in the sorted homogeneous spectrum
(scw_eig_warm: Rayleigh-quotient iteration per eigenpair on the Hessenberg form, accepted only
when every residual ||A v - lambda v|| and the mode count pass; otherwise the layer is
solved by the plain eigen-solver).

Training data are eigenpairs from the plain solver (scw_zgeev on the same matrices).
Device buffers are torch tensors; all compute runs in the native library.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from .evaluator import Context
from .solver import _params

PI_REF = 3.141592653


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@dataclass
class LayerProblems:
    """Per-slice Fourier crops (host, [Z, 2, MF] complex: n^2 then n^-2) and the reduced
    matrices PQ (device, torch [Z, n, n] complex128) of one sample, with the homogeneous-medium
    spectrum (host [Z, n], sorted by descending real part) and the plane-wave mode of each of its
    entries (host [Z, n] ints: row of PQ, Ex rows then Ey rows)."""
    coef: np.ndarray
    PQ: object
    M0: int
    M1: int
    baseline: np.ndarray
    modes: np.ndarray

def layer_problems(ctx: Context, sample, lam=1.0, direction=(0.0, 0.0, 1.0), ex=(1.0, 0.0), ey=(0.0, 0.0),
                   ez=(0.0, 0.0), n=(1.0, 1.0), kappa=0.0, size=(10.0, 10.0, 2.0), z=0.0, coef=None) -> LayerProblems:
    import torch
    vol = np.ascontiguousarray(sample, dtype=np.complex128)
    if vol.ndim == 2:
        vol = vol[None]
    Z, Y, X = vol.shape
    prm = _params(lam, direction, ex, ey, ez, n, kappa, size, z, coef, False, True)
    M0, M1 = ctypes.c_int(), ctypes.c_int()
    _lib.call("scw_layer_problem", ctx.handle, ctypes.c_void_p(vol.ctypes.data), Z, Y, X, ctypes.byref(prm),
              ctypes.byref(M0), ctypes.byref(M1), None, None)
    MF = M0.value * M1.value
    nn = 2 * MF
    dcoef = torch.zeros((Z, 2, MF), dtype=torch.complex128, device="cuda")
    dPQ = torch.zeros((Z, nn, nn), dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    _lib.call("scw_layer_problem", ctx.handle, ctypes.c_void_p(vol.ctypes.data), Z, Y, X, ctypes.byref(prm),
              None, None, _p(dcoef), _p(dPQ))
    # baseline: homogeneous layer of the slice's mean n^2 (the DFT's DC bin)
    d = np.asarray(direction, float)
    d = d / np.linalg.norm(d) * n[0]
    k = 2 * PI_REF / lam
    up = 2 * PI_REF * (np.arange(M0.value) - M0.value // 2) / size[0] + d[0] * k
    wq = 2 * PI_REF * (np.arange(M1.value) - M1.value // 2) / size[1] + d[1] * k
    kt2 = (np.add.outer(wq ** 2, up ** 2).ravel() / k ** 2)          # harmonic m = q M0 + p
    n2 = np.mean(vol.astype(np.complex128) ** 2, axis=(1, 2))
    base = n2[:, None] - np.concatenate([kt2, kt2])[None, :]
    order = np.stack([np.lexsort((-b.imag, -b.real)) for b in base]).astype(np.int32)
    base = np.take_along_axis(base, order, axis=1)                   # descending real part
    return LayerProblems(coef=dcoef.cpu().numpy(), PQ=dPQ, M0=M0.value, M1=M1.value, baseline=base, modes=order)


def plain_eig(ctx: Context, PQ):
    """Eigenpairs of every matrix of the device batch by the plain eigen-solver (copy kept)."""
    import torch
    A = PQ.clone()
    Z, n, _ = A.shape
    W = torch.zeros((Z, n), dtype=torch.complex128, device="cuda")
    V = torch.zeros((Z, n, n), dtype=torch.complex128, device="cuda")
    torch.cuda.synchronize()
    _lib.call("scw_zgeev", ctx.handle, n, _p(A), _p(W), _p(V), Z, None)
    return W, V


def mixed_eig(ctx: Context, PQ):
    """Eigenpairs of every matrix of the device batch by the mixed-precision solver
    (scw_zgeev_mixed: FP32 factorisation, FP64 Newton refinement, FP64 QR for matrices it does not
    accept; copy kept).  Returns (W, V, accepted) with accepted[z] = 1 where the refined result
    was kept."""
    import torch
    A = PQ.clone()
    Z, n, _ = A.shape
    W = torch.zeros((Z, n), dtype=torch.complex128, device="cuda")
    V = torch.zeros((Z, n, n), dtype=torch.complex128, device="cuda")
    acc = np.zeros(Z, np.int32)
    torch.cuda.synchronize()
    _lib.call("scw_zgeev_mixed", ctx.handle, n, _p(A), _p(W), _p(V), Z, ctypes.c_void_p(acc.ctypes.data), None,
              None)
    return W, V, acc


def warm_eig(ctx: Context, PQ, shifts, modes=None, max_it=12, tol=1e-11):
    """scw_eig_warm on the device batch PQ with device shifts [Z, n] complex128 and optional
    proposed modes [Z, n] (host ints: the start vector of each eigenpair)."""
    import torch
    Z, n, _ = PQ.shape
    W = torch.zeros((Z, n), dtype=torch.complex128, device="cuda")
    V = torch.zeros((Z, n, n), dtype=torch.complex128, device="cuda")
    acc = np.zeros(Z, np.int32)
    stats = np.zeros(5, np.float64)
    sh = shifts.contiguous()
    md = torch.from_numpy(np.ascontiguousarray(modes, dtype=np.int32)).cuda() if modes is not None else None
    torch.cuda.synchronize()
    _lib.call("scw_eig_warm", ctx.handle, n, _p(PQ), Z, _p(sh), _p(md) if md is not None else None, int(max_it),
              float(tol), _p(W), _p(V),
              ctypes.c_void_p(acc.ctypes.data), ctypes.c_void_p(stats.ctypes.data))
    return W, V, acc, {"mean_iterations": stats[0], "max_residual": stats[1], "accepted": int(stats[2]),
                       "fell_back": int(stats[3]), "repaired": int(stats[4])}


def sorted_desc(lam):
    """Eigenvalues sorted by descending real part (ties by imaginary part), per row."""
    lam = np.asarray(lam)
    return -np.sort_complex(-lam)


def features(coef):
    """[Z, 2, MF] complex crops -> [Z, 4 MF] float (Re, Im of n^2 then n^-2)."""
    c = np.asarray(coef).reshape(coef.shape[0], -1)
    return np.concatenate([c.real, c.imag], axis=1).astype(np.float32)


def _ri(z):
    return np.stack([z.real, z.imag], axis=-1).reshape(z.shape[0], -1)


class MLP:
    """scw_mlp: W3 relu(W2 relu(W1 x + b1) + b2) + b3 with device inputs (torch float32)."""

    def __init__(self, ctx: Context, n_in, width, n_out, seed=0):
        self.ctx = ctx
        self.shape = (n_in, width, n_out)
        self.handle = ctypes.c_void_p()
        _lib.call("scw_mlp_create", ctx.handle, n_in, width, n_out, ctypes.c_uint64(seed), ctypes.byref(self.handle))
        n = ctypes.c_int64()
        _lib.call("scw_mlp_info", self.handle, None, None, None, ctypes.byref(n))
        self.n_params = n.value

    def forward(self, X):
        import torch
        Y = torch.empty((X.shape[0], self.shape[2]), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        _lib.call("scw_mlp_forward", self.handle, _p(X), X.shape[0], _p(Y))
        self.ctx.synchronize()
        return Y

    def train_step(self, X, T, lr):
        import torch
        torch.cuda.synchronize()
        loss = ctypes.c_double()
        _lib.call("scw_mlp_train_step", self.handle, _p(X), _p(T), X.shape[0], ctypes.c_float(lr), ctypes.byref(loss))
        return loss.value

    def gradients(self, X, T):
        import torch
        g = np.zeros(self.n_params, np.float32)
        loss = ctypes.c_double()
        torch.cuda.synchronize()
        _lib.call("scw_mlp_gradients", self.handle, _p(X), _p(T), X.shape[0], ctypes.c_void_p(g.ctypes.data),
                  ctypes.byref(loss))
        return loss.value, g

    def params(self):
        p = np.zeros(self.n_params, np.float32)
        _lib.call("scw_mlp_get_params", self.handle, ctypes.c_void_p(p.ctypes.data))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _lib.call("scw_mlp_set_params", self.handle, ctypes.c_void_p(p.ctypes.data))

    def close(self):
        if self.handle:
            _lib.load().scw_mlp_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WarmStart:
    """Network + feature / target standardisation; predicts eigenvalue shifts of layers."""

    def __init__(self, ctx: Context, MF: int, width=512, seed=0):
        self.ctx = ctx
        self.MF = MF
        self.net = MLP(ctx, 4 * MF, width, 4 * MF, seed)
        self.fx = None
        self.ft = None

    def fit(self, coef, eigs, baseline, epochs=400, lr=1e-3, batch=256, seed=0, log=None):
        """coef [L, 2, MF] complex, eigs / baseline [L, 2MF] complex (both sorted by
        descending real part).  Returns the training loss history (per epoch, mean)."""
        import torch
        Xh = features(coef)
        Th = _ri(np.asarray(eigs) - np.asarray(baseline)).astype(np.float32)
        self.fx = (Xh.mean(0), Xh.std(0) + 1e-6)
        self.ft = (Th.mean(0), Th.std(0) + 1e-6)
        X = torch.from_numpy((Xh - self.fx[0]) / self.fx[1]).cuda()
        T = torch.from_numpy((Th - self.ft[0]) / self.ft[1]).cuda()
        rng = np.random.default_rng(seed)
        L = X.shape[0]
        hist = []
        for ep in range(epochs):
            perm = torch.from_numpy(rng.permutation(L)).cuda()
            tot = 0.0
            nb = 0
            for s in range(0, L, batch):
                idx = perm[s:s + batch]
                tot += self.net.train_step(X[idx].contiguous(), T[idx].contiguous(), lr)
                nb += 1
            hist.append(tot / nb)
            if log and (ep % 50 == 0 or ep == epochs - 1):
                log(f"epoch {ep} loss {hist[-1]:.4e}")
        return hist

    def predict(self, coef, baseline):
        """Predicted eigenvalues [L, 2MF] complex (host), in the baseline's sorted slots."""
        import torch
        Xh = (features(coef) - self.fx[0]) / self.fx[1]
        Y = self.net.forward(torch.from_numpy(Xh.astype(np.float32)).cuda()).cpu().numpy()
        d = Y * self.ft[1] + self.ft[0]
        corr = d[:, 0::2] + 1j * d[:, 1::2]
        return np.asarray(baseline) + corr
