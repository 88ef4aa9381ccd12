"""FP64 checks of the evaluators on SOLVED coefficient sets (test and benchmark infrastructure).

The reference's evaluator sums E0 exp(i k.r) over the waves of a point's region
(gpuEvaluator.cu:28-68, cpuEvaluator.cpp:294-407), and the waves of region l + 1 (the interior
of slice l) are the 2MF downward modes of slice l referenced at z_l and the 2MF upward modes
referenced at z_{l+1}, each for every harmonic p = (a, b) with kx = kx_a, ky = ky_b
(sCWatter.cpp:890-956, wound to the origin with wind(0, 0, -z)).

* :func:`region_waves` restates that packing for one region from the solve's FP64 mode
  amplitudes (Q_check / Q_hat, [3MF, 2MF]) and roots gamma, giving the wave records the FP64
  oracle evaluator ``oracle_lib.eval_points_f64`` sums term by term;
* :func:`eval_points_sep_f64` is the same FP64 sum grouped by harmonic (first over the modes,
  then over the harmonics), for many points at once; it is checked against the term-by-term
  oracle on a subset wherever it is used.
"""
from __future__ import annotations

import numpy as np


def region_waves(Qc, Qh, gamma, kx, ky, k, z_lo, z_hi):
    """[4 MF^2, 6] complex128 records (E0 x y z, k x y z) of the interior region of one slice,
    E0 wound to the origin in FP64: downward modes (Q_check, kz = gamma k, referenced at z_lo)
    then upward modes (Q_hat, kz = -gamma k, referenced at z_hi), harmonic p = a M1 + b."""
    M0, M1 = len(kx), len(ky)
    MF = M0 * M1
    Qc = np.asarray(Qc).reshape(3, MF, -1)
    Qh = np.asarray(Qh).reshape(3, MF, -1)
    KX = np.repeat(np.asarray(kx, np.float64), M1)
    KY = np.tile(np.asarray(ky, np.float64), M0)
    out = []
    for Q, kz, zr in [(Qc, gamma * k, z_lo), (Qh, -gamma * k, z_hi)]:
        J = Q.shape[2]
        w = np.empty((MF, J, 6), np.complex128)
        w[..., 0:3] = np.transpose(Q, (1, 2, 0)) * np.exp(-1j * kz * zr)[None, :, None]
        w[..., 3] = KX[:, None]
        w[..., 4] = KY[:, None]
        w[..., 5] = kz[None, :]
        out.append(w.reshape(-1, 6))
    return np.concatenate(out)


def eval_points_sep_f64(Qc, Qh, gamma, kx, ky, k, z_lo, z_hi, pts):
    """FP64 field [n, 3] at float32 points [n, 3] (all inside the slice) from the slice's modes:
    C(p; z) = sum_j Qc(p, j) e^{i gamma_j k (z - z_lo)} + Qh(p, j) e^{-i gamma_j k (z - z_hi)},
    E = sum_p C(p; z) e^{i (kx_a x + ky_b y)}, evaluated once per distinct z."""
    M0, M1 = len(kx), len(ky)
    MF = M0 * M1
    Qc = np.asarray(Qc, np.complex128).reshape(3 * MF, -1)
    Qh = np.asarray(Qh, np.complex128).reshape(3 * MF, -1)
    pts = np.asarray(pts, np.float32).astype(np.float64).reshape(-1, 3)
    KX = np.repeat(np.asarray(kx, np.float64), M1)
    KY = np.tile(np.asarray(ky, np.float64), M0)
    out = np.zeros((len(pts), 3), np.complex128)
    for z in np.unique(pts[:, 2]):
        sel = np.nonzero(pts[:, 2] == z)[0]
        C = (Qc @ np.exp(1j * gamma * k * (z - z_lo)) + Qh @ np.exp(-1j * gamma * k * (z - z_hi))).reshape(3, MF)
        ph = np.exp(1j * (np.outer(pts[sel, 0], KX) + np.outer(pts[sel, 1], KY)))      # [n, MF]
        out[sel] = ph @ C.T
    return out
