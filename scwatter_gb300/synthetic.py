"""Seeded synthetic coefficient sets with the structure and value ranges of a solved sample.

Used by the benchmark and the large-size tests, where running the full FP64 solve for
every configuration would take hours: the evaluator's cost depends only on the
wave counts and the region structure, not on the values.

The structure follows the solver's output (sCWatter.cpp:890-956):
  * incident and reflected blocks of MF waves each (region 0), transmitted MF waves
    (last region);
  * inside slice l, for every harmonic p = (a, b) of the M0 x M1 grid, 2MF downward
    modes referenced at the slice top and 2MF upward modes referenced at its bottom,
    with kx = kx_a, ky = ky_b (real, on the separable grid) and kz = gamma_j k.
Values: gamma_j has Re in [1.0, 1.4] (sign by direction) and |Im| <= 0.02 with the
decaying sign; amplitudes are complex normal scaled by 1/(2 MF).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

PI_REF = 3.141592653


@dataclass
class FactoredSample:
    """Separable (factored) coefficients of one sample.

    kx [M0], ky [M1] (real), k (vacuum wavenumber), z [Z+1] boundaries,
    gamma_dn / gamma_up [Z, 2MF] (complex), Q_dn / Q_up [Z, 3, MF, 2MF] complex
    (rows p = a*M1 + b, i.e. harmonic (kx_a, ky_b)), plus the exterior blocks
    inc / refl / trans [3, MF] and their kz (complex, [MF]).
    """
    M0: int
    M1: int
    k: float
    kx: np.ndarray
    ky: np.ndarray
    z: np.ndarray
    gamma_dn: np.ndarray
    gamma_up: np.ndarray
    Q_dn: np.ndarray
    Q_up: np.ndarray
    inc: np.ndarray
    refl: np.ndarray
    trans: np.ndarray
    kz_inc: np.ndarray
    kz_refl: np.ndarray
    kz_trans: np.ndarray

    @property
    def MF(self):
        return self.M0 * self.M1

    @property
    def Z(self):
        return len(self.z) - 1


def make_factored(M0=20, M1=20, Z=20, size=(64.0, 64.0, 20.0), lam=1.0, z_center=0.0, seed=0,
                  dtype=np.complex128) -> FactoredSample:
    rng = np.random.default_rng(seed)
    k = 2 * PI_REF / lam
    MF = M0 * M1
    p = np.arange(M0) - M0 // 2
    q = np.arange(M1) - M1 // 2
    kx = 2 * PI_REF * p / size[0]
    ky = 2 * PI_REF * q / size[1]
    z = z_center - size[2] / 2 + np.arange(Z + 1) * (size[2] / Z)
    J = 2 * MF
    re = rng.uniform(1.0, 1.4, size=(Z, J))
    im = rng.uniform(0.0, 0.02, size=(Z, J))
    gamma_dn = (re + 1j * im).astype(np.complex128)
    gamma_up = (-re + 1j * -im).astype(np.complex128)
    scale = 1.0 / (2 * MF)
    shp = (Z, 3, MF, J)
    Q_dn = (rng.standard_normal(shp) + 1j * rng.standard_normal(shp)).astype(dtype) * scale
    Q_up = (rng.standard_normal(shp) + 1j * rng.standard_normal(shp)).astype(dtype) * (0.3 * scale)
    sz = np.sqrt((1.0 + 0j) - (np.repeat(kx, M1) / k) ** 2 - (np.tile(ky, M0) / k) ** 2)
    inc = np.zeros((3, MF), np.complex128)
    inc[0, (M0 // 2) * M1 + M1 // 2] = 1.0
    refl = (rng.standard_normal((3, MF)) + 1j * rng.standard_normal((3, MF))) * 0.05
    trans = (rng.standard_normal((3, MF)) + 1j * rng.standard_normal((3, MF))) * 0.5
    return FactoredSample(M0, M1, k, kx, ky, z, gamma_dn, gamma_up, Q_dn, Q_up, inc, refl, trans,
                          sz * k, -sz * k, sz * k)


def to_cw_arrays(fs: FactoredSample):
    """Expands a factored sample into .cw wave blocks wound to the origin exactly as the
    solver writes them: returns (Pi [MF,6], z list, Pr list, Pt list) of complex128."""
    MF, Z, k = fs.MF, fs.Z, fs.k
    KX = np.repeat(fs.kx, fs.M1).astype(np.complex128)
    KY = np.tile(fs.ky, fs.M0).astype(np.complex128)

    def block(E, kz, zl):      # E [3, MF], kz [MF]
        w = np.stack([E[0], E[1], E[2], KX, KY, kz], axis=1)
        w[:, 0:3] *= np.exp(-1j * kz * zl)[:, None]
        return w

    def modes(Q, gamma, zl):   # Q [3, MF, J], gamma [J]: per p, J waves
        J = Q.shape[2]
        w = np.empty((MF, J, 6), np.complex128)
        w[..., 0] = Q[0]
        w[..., 1] = Q[1]
        w[..., 2] = Q[2]
        w[..., 3] = KX[:, None]
        w[..., 4] = KY[:, None]
        w[..., 5] = (gamma * k)[None, :]
        w[..., 0:3] *= np.exp(-1j * gamma * k * zl)[None, :, None]
        return w.reshape(MF * J, 6)

    Pi = np.stack([fs.inc[0], fs.inc[1], fs.inc[2], KX, KY, fs.kz_inc], axis=1)
    zs, Pr, Pt = [], [], []
    for l in range(Z + 1):
        zl = float(fs.z[l])
        zs.append(zl)
        pr = [block(fs.refl, fs.kz_refl, zl)] if l == 0 else [modes(fs.Q_up[l - 1], fs.gamma_up[l - 1], zl)]
        pt = [block(fs.trans, fs.kz_trans, zl)] if l == Z else [modes(fs.Q_dn[l], fs.gamma_dn[l], zl)]
        Pr.append(np.concatenate(pr))
        Pt.append(np.concatenate(pt))
    return Pi, zs, Pr, Pt


def to_structure(fs: FactoredSample):
    from .cw import CoupledWaveStructure, HomogeneousLayer
    Pi, zs, Pr, Pt = to_cw_arrays(fs)
    S = CoupledWaveStructure()
    S.Pi = Pi
    S.Layers = [HomogeneousLayer(z=zs[l], Pr=Pr[l], Pt=Pt[l]) for l in range(len(zs))]
    return S


def device_factored(M0, M1, Z, size, lam=1.0, z_center=0.0, seed=0, device="cuda"):
    """Same structure and value ranges as :func:`make_factored`, with the large Q blocks
    drawn on the GPU (torch, seeded) as complex64 [Z, 3, MF, 2MF] tensors; everything else
    on the host in float64/complex128.  Returns (fs, Q_dn, Q_up) with fs.Q_dn / fs.Q_up None."""
    import torch
    rng = np.random.default_rng(seed)
    k = 2 * PI_REF / lam
    MF = M0 * M1
    J = 2 * MF
    p = np.arange(M0) - M0 // 2
    q = np.arange(M1) - M1 // 2
    kx = 2 * PI_REF * p / size[0]
    ky = 2 * PI_REF * q / size[1]
    z = z_center - size[2] / 2 + np.arange(Z + 1) * (size[2] / Z)
    re = rng.uniform(1.0, 1.4, size=(Z, J))
    im = rng.uniform(0.0, 0.02, size=(Z, J))
    gamma_dn = (re + 1j * im).astype(np.complex128)
    gamma_up = (-re - 1j * im).astype(np.complex128)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    scale = 1.0 / (2 * MF)
    Q_dn = torch.randn((Z, 3, MF, J), dtype=torch.complex64, device=device, generator=g) * scale
    Q_up = torch.randn((Z, 3, MF, J), dtype=torch.complex64, device=device, generator=g) * (0.3 * scale)
    sz = np.sqrt((1.0 + 0j) - (np.repeat(kx, M1) / k) ** 2 - (np.tile(ky, M0) / k) ** 2)
    inc = np.zeros((3, MF), np.complex128)
    inc[0, (M0 // 2) * M1 + M1 // 2] = 1.0
    refl = (rng.standard_normal((3, MF)) + 1j * rng.standard_normal((3, MF))) * 0.05
    trans = (rng.standard_normal((3, MF)) + 1j * rng.standard_normal((3, MF))) * 0.5
    fs = FactoredSample(M0, M1, k, kx, ky, z, gamma_dn, gamma_up, None, None, inc, refl, trans,
                        sz * k, -sz * k, sz * k)
    return fs, Q_dn, Q_up


@dataclass
class PairedSample:
    """Paired form of a factored sample (the solver's mode structure): per slice one block
    V [Z, 3, MF, J] and amplitudes beta_dn, beta_up [Z, J], with Q_dn = V diag(beta_dn) and
    Q_up = diag(1, 1, -1) V diag(beta_up); gamma_up = -gamma_dn.  Exterior blocks as in
    :class:`FactoredSample`."""
    base: FactoredSample          # k grids, z, gamma, exterior blocks (its Q_dn / Q_up unused)
    V: np.ndarray
    beta_dn: np.ndarray
    beta_up: np.ndarray

    def to_factored(self) -> FactoredSample:
        """The same coefficients as a two-half :class:`FactoredSample` (for the FP64 oracle)."""
        import dataclasses
        s = np.array([1.0, 1.0, -1.0])[None, :, None, None]
        V = self.V.astype(np.complex128)
        return dataclasses.replace(self.base, Q_dn=V * self.beta_dn[:, None, None, :],
                                   Q_up=s * V * self.beta_up[:, None, None, :])


def _paired_meta(M0, M1, Z, size, lam, z_center, rng):
    k = 2 * PI_REF / lam
    MF = M0 * M1
    J = 2 * MF
    p = np.arange(M0) - M0 // 2
    q = np.arange(M1) - M1 // 2
    kx = 2 * PI_REF * p / size[0]
    ky = 2 * PI_REF * q / size[1]
    z = z_center - size[2] / 2 + np.arange(Z + 1) * (size[2] / Z)
    re = rng.uniform(1.0, 1.4, size=(Z, J))
    im = rng.uniform(0.0, 0.02, size=(Z, J))
    gamma_dn = (re + 1j * im).astype(np.complex128)
    # eigenvector columns normalised to 1 (entries ~ 1/sqrt(3 MF)); amplitudes ~ 1/sqrt(2 MF)
    bd = (rng.standard_normal((Z, J)) + 1j * rng.standard_normal((Z, J))) / np.sqrt(2 * J)
    bu = 0.3 * (rng.standard_normal((Z, J)) + 1j * rng.standard_normal((Z, J))) / np.sqrt(2 * J)
    sz = np.sqrt((1.0 + 0j) - (np.repeat(kx, M1) / k) ** 2 - (np.tile(ky, M0) / k) ** 2)
    inc = np.zeros((3, MF), np.complex128)
    inc[0, (M0 // 2) * M1 + M1 // 2] = 1.0
    refl = (rng.standard_normal((3, MF)) + 1j * rng.standard_normal((3, MF))) * 0.05
    trans = (rng.standard_normal((3, MF)) + 1j * rng.standard_normal((3, MF))) * 0.5
    base = FactoredSample(M0, M1, k, kx, ky, z, gamma_dn, -gamma_dn, None, None, inc, refl, trans,
                          sz * k, -sz * k, sz * k)
    return base, bd, bu


def make_paired(M0=20, M1=20, Z=20, size=(64.0, 64.0, 20.0), lam=1.0, z_center=0.0, seed=0) -> PairedSample:
    """Seeded paired sample on the host (V complex64)."""
    rng = np.random.default_rng(seed)
    base, bd, bu = _paired_meta(M0, M1, Z, size, lam, z_center, rng)
    MF, J = M0 * M1, 2 * M0 * M1
    shp = (Z, 3, MF, J)
    V = ((rng.standard_normal(shp) + 1j * rng.standard_normal(shp)) / np.sqrt(6 * MF)).astype(np.complex64)
    return PairedSample(base, V, bd, bu)


def device_paired(M0, M1, Z, size, lam=1.0, z_center=0.0, seed=0, device="cuda"):
    """Paired sample with the large block V drawn on the GPU (torch, seeded) as a complex64
    [Z, 3, MF, 2MF] tensor.  Returns (PairedSample with V None, V)."""
    import torch
    rng = np.random.default_rng(seed)
    base, bd, bu = _paired_meta(M0, M1, Z, size, lam, z_center, rng)
    MF = M0 * M1
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    V = torch.randn((Z, 3, MF, 2 * MF), dtype=torch.complex64, device=device, generator=g) / float(np.sqrt(3 * MF))
    return PairedSample(base, None, bd, bu), V
