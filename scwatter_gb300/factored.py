"""Compact factored coefficient files (.cwf) on the host, without a GPU.

The .cwf file holds the separable coefficient set the GEMM-form evaluator reads (written and
read on the device by ``scw_sep_save`` / ``scw_sep_load``):

    char[8]    "SCWSEP01"
    int32      M0, M1, Z, J (modes per half), rule (region rule), 0
    float64    kx[M0], ky[M1], z_boundaries[Z + 1]
    complex128 exterior[12 MF]   inc[3][MF], refl[3][MF], trans[3][MF], kz_inc, kz_refl, kz_trans
    complex128 kz[Z][2][Jp]      (Jp = J rounded up to even; entries J..Jp-1 are zero)
    complex64  Q[Z][2][3][MF][Jp]

A paired set (the solver's own output, ``scw_sep_create_paired``) is written as "SCWSEP02": the
same blocks up to kz, then complex128 beta[Z][2][Jp] and complex64 V[Z][3][MF][Jp] with
Q_dn = V diag(beta_dn), Q_up = diag(1, 1, -1) V diag(beta_up).  :func:`read_cwf` reads both and
returns the two-half blocks.

Row p = a M1 + b of an MF block is harmonic (kx[a], ky[b]).  Every amplitude is referenced to
its own plane: E0 exp(i kz z_ref), where the .cw record stores E0 wound to z = 0
(sCWatter.cpp:469-482).  :func:`factor_cw` builds the set from a volume-solver ``.cw``
structure (the host restatement of ``scw_sep_from_cw``), :func:`to_cw` rebuilds the wave
lists from it, and :func:`read_cwf` / :func:`write_cwf` move it to and from a file.  These are
format tools: evaluation runs on the GPU (``SeparableSet``).
"""
from __future__ import annotations

import argparse
import sys
from dataclasses import dataclass

import numpy as np

from .cw import CoupledWaveStructure, HomogeneousLayer

MAGIC = b"SCWSEP01"
MAGIC_PAIRED = b"SCWSEP02"


@dataclass
class FactoredSet:
    M0: int
    M1: int
    Z: int
    J: int
    rule: int
    kx: np.ndarray          # [M0] float64
    ky: np.ndarray          # [M1] float64
    zb: np.ndarray          # [Z + 1] float64
    ext: np.ndarray         # [12 MF] complex128
    kz: np.ndarray          # [Z, 2, Jp] complex128
    Q: np.ndarray           # [Z, 2, 3, MF, Jp] complex64

    @property
    def MF(self) -> int:
        return self.M0 * self.M1

    @property
    def Jp(self) -> int:
        return self.J + (self.J & 1)

    def exterior(self, block: str) -> tuple:
        """(amplitudes [3, MF], kz [MF]) of ``"inc"``, ``"refl"`` or ``"trans"``."""
        MF = self.MF
        i = {"inc": 0, "refl": 1, "trans": 2}[block]
        return self.ext[3 * MF * i:3 * MF * (i + 1)].reshape(3, MF), self.ext[9 * MF + MF * i:9 * MF + MF * (i + 1)]


def file_size(M0, M1, Z, J, paired=False) -> int:
    MF, Jp = M0 * M1, J + (J & 1)
    head = 8 + 24 + 8 * (M0 + M1 + Z + 1) + 16 * 12 * MF + 16 * Z * 2 * Jp
    if paired:
        return head + 16 * Z * 2 * Jp + (8 * Z * 3 * MF * Jp if J else 0)
    return head + (8 * Z * 2 * 3 * MF * Jp if J else 0)


def write_cwf(path, fs: FactoredSet) -> None:
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(np.array([fs.M0, fs.M1, fs.Z, fs.J, fs.rule, 0], dtype="<i4").tobytes())
        for a in (fs.kx, fs.ky, fs.zb):
            f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(fs.ext, dtype="<c16").tobytes())
        f.write(np.ascontiguousarray(fs.kz, dtype="<c16").tobytes())
        if fs.J and fs.Z:
            f.write(np.ascontiguousarray(fs.Q, dtype="<c8").tobytes())


def read_cwf(path) -> FactoredSet:
    data = open(path, "rb").read()
    if len(data) < 32 or data[:8] not in (MAGIC, MAGIC_PAIRED):
        raise ValueError(f"not a factored coefficient file: {path}")
    paired = data[:8] == MAGIC_PAIRED
    M0, M1, Z, J, rule, _ = (int(v) for v in np.frombuffer(data, "<i4", 6, 8))
    if M0 <= 0 or M1 <= 0 or Z < 0 or J < 0 or len(data) != file_size(M0, M1, Z, J, paired):
        raise ValueError("factored file size does not match its header")
    MF, Jp = M0 * M1, J + (J & 1)
    off = 32

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(data, dtype, count, off)
        off += a.nbytes
        return a.copy()

    kx, ky, zb = take("<f8", M0), take("<f8", M1), take("<f8", Z + 1)
    ext = take("<c16", 12 * MF)
    kz = take("<c16", Z * 2 * Jp).reshape(Z, 2, Jp)
    if paired:
        beta = take("<c16", Z * 2 * Jp).reshape(Z, 2, Jp)
        Q = np.zeros((Z, 2, 3, MF, Jp if J else 0), np.complex64)
        if J:
            V = take("<c8", Z * 3 * MF * Jp).reshape(Z, 3, MF, Jp)
            sign = np.array([1.0, 1.0, -1.0])[:, None, None]
            for l in range(Z):
                v = V[l].astype(np.complex128)
                Q[l, 0] = v * beta[l, 0][None, None, :]
                Q[l, 1] = sign * v * beta[l, 1][None, None, :]
    else:
        Q = take("<c8", Z * 2 * 3 * MF * Jp).reshape(Z, 2, 3, MF, Jp) if J else np.zeros((Z, 2, 3, MF, 0), np.complex64)
    return FactoredSet(M0, M1, Z, J, rule, kx, ky, zb, ext, kz, Q)


def factor_cw(cw: CoupledWaveStructure, rule: int = 0) -> FactoredSet:
    """The separable set of a volume-solver .cw structure (the host form of scw_sep_from_cw):
    the structure is checked exactly (kx per column, ky per row of the harmonic grid, one kz
    per mode across harmonics) and every amplitude re-referenced to its plane in FP64."""
    Pi = np.asarray(cw.Pi, np.complex128).reshape(-1, 6)
    MF, ZL = len(Pi), len(cw.Layers)
    if MF == 0 or ZL < 2:
        raise ValueError("not a volume-solver .cw (needs incident waves and >= 2 boundaries)")
    Z = ZL - 1
    M1 = 1
    while M1 < MF and Pi[M1, 3] == Pi[0, 3]:
        M1 += 1
    if MF % M1:
        raise ValueError("incident block is not an M0 x M1 harmonic grid")
    M0 = MF // M1
    kx = Pi[::M1, 3].real.copy()[:M0]
    ky = Pi[:M1, 4].real.copy()
    p = np.arange(MF)
    gx, gy = kx[p // M1], ky[p % M1]

    def grid_ok(w):
        return (np.array_equal(w[:, 3], gx.astype(np.complex128)) and np.array_equal(w[:, 4], gy.astype(np.complex128)))

    L0, LZ = cw.Layers[0], cw.Layers[-1]
    blocks = []
    zb = np.array([L.z for L in cw.Layers], np.float64)
    for w, zr in ((Pi, 0.0), (np.asarray(L0.Pr).reshape(-1, 6), zb[0]), (np.asarray(LZ.Pt).reshape(-1, 6), zb[-1])):
        if len(w) != MF or not grid_ok(w):
            raise ValueError("exterior waves are not separable")
        f = np.exp(1j * w[:, 5] * zr)
        blocks.append(((w[:, :3] * f[:, None]).T, w[:, 5]))
    ext = np.concatenate([b[0].ravel() for b in blocks] + [b[1] for b in blocks])
    J = len(np.asarray(L0.Pt).reshape(-1, 6)) // MF
    Jp = J + (J & 1)
    kz = np.zeros((Z, 2, Jp), np.complex128)
    Q = np.zeros((Z, 2, 3, MF, Jp), np.complex64)
    for l in range(Z):
        for h, (w, zr) in enumerate(((cw.Layers[l].Pt, zb[l]), (cw.Layers[l + 1].Pr, zb[l + 1]))):
            w = np.asarray(w).reshape(-1, 6)
            if len(w) != MF * J:
                raise ValueError(f"slice {l} mode blocks are not MF x J")
            w = w.reshape(MF, J, 6)
            kj = w[0, :, 5]
            if not (np.array_equal(w[:, :, 5], np.broadcast_to(kj, (MF, J))) and
                    np.array_equal(w[:, :, 3], np.broadcast_to(gx[:, None], (MF, J)).astype(np.complex128)) and
                    np.array_equal(w[:, :, 4], np.broadcast_to(gy[:, None], (MF, J)).astype(np.complex128))):
                raise ValueError(f"slice {l} waves are not separable")
            kz[l, h, :J] = kj
            f = np.exp(1j * kj * zr)
            Q[l, h, :, :, :J] = np.moveaxis(w[:, :, :3] * f[None, :, None], 2, 0).astype(np.complex64)
    return FactoredSet(M0, M1, Z, J, rule, kx, ky, zb, ext, kz, Q)


def to_cw(fs: FactoredSet) -> CoupledWaveStructure:
    """The wave lists of the set in the order the volume solver writes them (harmonic outer,
    mode inner), each amplitude wound back to z = 0 from its plane."""
    MF, J = fs.MF, fs.J
    p = np.arange(MF)
    gx = fs.kx[p // fs.M1].astype(np.complex128)
    gy = fs.ky[p % fs.M1].astype(np.complex128)

    def exterior(block, zr):
        a, kz = fs.exterior(block)
        f = np.exp(-1j * kz * zr)
        return np.stack([a[0] * f, a[1] * f, a[2] * f, gx, gy, kz], axis=1)

    def modes(l, h, zr):
        kj = fs.kz[l, h, :J]
        a = fs.Q[l, h, :, :, :J].astype(np.complex128) * np.exp(-1j * kj * zr)[None, None, :]
        out = np.empty((MF, J, 6), np.complex128)
        out[:, :, 0], out[:, :, 1], out[:, :, 2] = a[0], a[1], a[2]
        out[:, :, 3], out[:, :, 4], out[:, :, 5] = gx[:, None], gy[:, None], kj[None, :]
        return out.reshape(-1, 6)

    cw = CoupledWaveStructure()
    cw.Pi = exterior("inc", 0.0)
    empty = np.zeros((0, 6), np.complex128)
    for l in range(fs.Z + 1):
        zr = fs.zb[l]
        Pr = exterior("refl", zr) if l == 0 else (modes(l - 1, 1, zr) if J else empty)
        Pt = exterior("trans", zr) if l == fs.Z else (modes(l, 0, zr) if J else empty)
        cw.Layers.append(HomogeneousLayer(z=float(zr), Pr=Pr, Pt=Pt))
    return cw


def _cw_layout(path):
    """Byte offsets of a .cw file (CoupledWaveStructure.h:72-100): (Pi offset, nPi, [(z, Pr
    offset, nPr, Pt offset, nPt) per layer]), from the counts alone."""
    size = __import__("os").path.getsize(path)
    with open(path, "rb") as f:
        def u64():
            b = f.read(8)
            if len(b) != 8:
                raise ValueError("truncated .cw file")
            return int(np.frombuffer(b, "<u8")[0])
        u64()                                   # sizeof(T)
        npi = u64()
        pi_off = f.tell()
        f.seek(96 * npi, 1)
        nl = u64()
        layers = []
        for _ in range(nl):
            b = f.read(8)
            if len(b) != 8:
                raise ValueError("truncated .cw layer")
            z = float(np.frombuffer(b, "<f8")[0])
            npr = u64()
            pr_off = f.tell()
            f.seek(96 * npr, 1)
            npt = u64()
            pt_off = f.tell()
            f.seek(96 * npt, 1)
            layers.append((z, pr_off, npr, pt_off, npt))
        if f.tell() > size:
            raise ValueError("truncated .cw file")
    return pi_off, npi, layers


def convert_cw_file(src, dst, rule: int = 0) -> FactoredSet:
    """Factors a volume-solver .cw file into a .cwf file, streaming: the .cw is memory-mapped
    and read one slice's two mode blocks at a time, so host memory stays at one slice however
    large the file (about 63 GB at MF = 1600, 64 slices).  Returns the set with an empty Q."""
    pi_off, npi, layers = _cw_layout(src)
    mm = np.memmap(src, dtype=np.uint8, mode="r")

    def block(off, n):
        return np.frombuffer(mm, "<c16", 6 * n, off).reshape(n, 6)

    head = CoupledWaveStructure()
    head.Pi = block(pi_off, npi)
    ZL = len(layers)
    if ZL < 2:
        raise ValueError("not a volume-solver .cw (needs incident waves and >= 2 boundaries)")
    # exterior blocks and the harmonic grid from a structure holding only the exterior waves
    z0, pr0, npr0, pt0, npt0 = layers[0]
    zZ, prZ, nprZ, ptZ, nptZ = layers[-1]
    head.Layers = [HomogeneousLayer(z=z0, Pr=block(pr0, npr0), Pt=np.zeros((0, 6), np.complex128)),
                   HomogeneousLayer(z=zZ, Pr=np.zeros((0, 6), np.complex128), Pt=block(ptZ, nptZ))]
    fs = factor_cw(head, rule)                  # J = 0 here: exterior only
    MF = fs.MF
    J = npt0 // MF
    Jp = J + (J & 1)
    Z = ZL - 1
    zb = np.array([L[0] for L in layers], np.float64)
    p = np.arange(MF)
    gx, gy = fs.kx[p // fs.M1].astype(np.complex128), fs.ky[p % fs.M1].astype(np.complex128)

    def modes(off, n, zr, l):
        if n != MF * J:
            raise ValueError(f"slice {l} mode blocks are not MF x J")
        w = block(off, n).reshape(MF, J, 6)
        kj = w[0, :, 5].copy()
        if not (np.array_equal(w[:, :, 5], np.broadcast_to(kj, (MF, J))) and
                np.array_equal(w[:, :, 3], np.broadcast_to(gx[:, None], (MF, J))) and
                np.array_equal(w[:, :, 4], np.broadcast_to(gy[:, None], (MF, J)))):
            raise ValueError(f"slice {l} waves are not separable")
        q = np.zeros((3, MF, Jp), np.complex64)
        q[:, :, :J] = np.moveaxis(w[:, :, :3] * np.exp(1j * kj * zr)[None, :, None], 2, 0).astype(np.complex64)
        return kj, q

    kz = np.zeros((Z, 2, Jp), np.complex128)
    for l in range(Z):                          # kz of every slice first (the file order)
        for h, (off, n, zr) in enumerate(((layers[l][3], layers[l][4], zb[l]), (layers[l + 1][1], layers[l + 1][2], zb[l + 1]))):
            if n != MF * J:
                raise ValueError(f"slice {l} mode blocks are not MF x J")
            kz[l, h, :J] = block(off, J)[:, 5]
    with open(dst, "wb") as f:
        f.write(MAGIC)
        f.write(np.array([fs.M0, fs.M1, Z, J, rule, 0], dtype="<i4").tobytes())
        for a in (fs.kx, fs.ky, zb):
            f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(fs.ext, dtype="<c16").tobytes())
        f.write(kz.astype("<c16").tobytes())
        if J:
            for l in range(Z):
                for off, n, zr in ((layers[l][3], layers[l][4], zb[l]), (layers[l + 1][1], layers[l + 1][2], zb[l + 1])):
                    kj, q = modes(off, n, zr, l)
                    f.write(q.astype("<c8").tobytes())
    return FactoredSet(fs.M0, fs.M1, Z, J, rule, fs.kx, fs.ky, zb, fs.ext, kz, np.zeros((Z, 2, 3, MF, 0), np.complex64))


def main(argv=None) -> int:
    """``python -m scwatter_gb300.factored in.cw out.cwf`` factors a volume-solver .cw file;
    ``python -m scwatter_gb300.factored in.cwf out.cw`` writes the wave lists back."""
    ap = argparse.ArgumentParser(prog="scwatter_gb300.factored", description="convert between .cw and .cwf")
    ap.add_argument("input")
    ap.add_argument("output")
    a = ap.parse_args(argv)
    if a.input.endswith(".cwf"):
        to_cw(read_cwf(a.input)).save(a.output)
    else:
        import os
        if not os.path.exists(a.input):
            print(f"ERROR: file {a.input} not found", file=sys.stderr)
            return 1
        try:
            convert_cw_file(a.input, a.output)
        except ValueError as e:
            print(f"ERROR: {a.input}: {e}", file=sys.stderr)
            return 2
    return 0


if __name__ == "__main__":
    sys.exit(main())
