"""Shared helpers for the tests (not collected)."""
import numpy as np

from oracle import solve_oracle as so
from scwatter_gb300 import cw as cwmod


def rel_l2(got, ref, floor=1e-3):
    """Per-component relative L2 error; a component whose norm is below ``floor`` times the
    whole field's norm is measured against that floor instead (near-zero components)."""
    got = np.asarray(got).reshape(-1, 3).astype(np.complex128)
    ref = np.asarray(ref).reshape(-1, 3).astype(np.complex128)
    tot = np.linalg.norm(ref)
    out = []
    for c in range(3):
        den = max(np.linalg.norm(ref[:, c]), floor * tot, 1e-300)
        out.append(float(np.linalg.norm(got[:, c] - ref[:, c]) / den))
    return out


def to_structure(c: so.CW) -> cwmod.CoupledWaveStructure:
    S = cwmod.CoupledWaveStructure()
    S.Pi = c.Pi
    S.Layers = [cwmod.HomogeneousLayer(z=c.z[l], Pr=c.Pr[l], Pt=c.Pt[l]) for l in range(len(c.z))]
    return S


def solved_case(shape=(3, 16, 16), coef=(5, 5), seed=1, direction=(0, 0, 1), external=False,
                ex=(1, 0), ey=(0, 0), lam=1.0):
    from scwatter_gb300 import samples
    s = samples.spheres(shape, n_spheres=2, radius=(3, 5), seed=seed)
    prm = so.SolveParams(lam=lam, direction=direction, ex=ex, ey=ey,
                         size=(float(shape[2]), float(shape[1]), float(shape[0])), coef=coef, external=external)
    r = so.solve(s, prm)
    return s, prm, r, so.pack(r, prm)
