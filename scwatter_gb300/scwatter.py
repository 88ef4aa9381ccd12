"""Command-line front end with the options of the reference program sCWatter
(sCWatter.cpp:506-527): solves a sample volume on the GPU and writes the .cw file.

    python -m scwatter_gb300.scwatter --sample s.npy --lambda 1 --coef 20 20 --size 64 64 20 --output c.cw

``--sample`` is an .npy file of complex (or real) refractive index, ``[Z, Y, X]`` or
``[Y, X]``.  ``--log`` is accepted and prints the stage timings.
"""
from __future__ import annotations

import argparse
import sys
import time

import numpy as np


def parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(prog="scwatter", description="coupled-wave solve of a sample volume on the GPU")
    p.add_argument("--sample", required=True, help="input sample as an .npy file")
    p.add_argument("--lambda", dest="lam", type=float, default=1.0, help="incident field vacuum wavelength")
    p.add_argument("--direction", type=float, nargs=3, default=[0.0, 0.0, 1.0], help="incoming field direction")
    p.add_argument("--ex", type=float, nargs=2, default=[0.0, 0.0], help="x component of the electrical field")
    p.add_argument("--ey", type=float, nargs=2, default=[1.0, 0.0], help="y component of the electrical field")
    p.add_argument("--ez", type=float, nargs=2, default=[0.0, 0.0], help="z component of the electrical field")
    p.add_argument("--n", type=float, nargs="+", default=[1.0, 1.0],
                   help="real refractive index of the upper and lower layers")
    p.add_argument("--kappa", type=float, nargs="+", default=[0.0], help="absorbance of the lower layer")
    p.add_argument("--size", type=float, nargs=3, default=[10.0, 10.0, 2.0], help="real size of the sample")
    p.add_argument("--z", type=float, default=0.0, help="the center of the sample along z")
    p.add_argument("--output", default="c.cw", help="output filename for the coupled wave structure")
    p.add_argument("--coef", type=int, nargs="+", default=None, help="number of Fourier coefficients (1 or 2 values)")
    p.add_argument("--psf", action="store_true", help="every harmonic carries the incident field")
    p.add_argument("--external", action="store_true", help="save waves for the external field only")
    p.add_argument("--log", action="store_true", help="print stage timings")
    p.add_argument("--npz", action="store_true", help="skip Ez of the modes (Px and Py only)")
    p.add_argument("--device", type=int, default=0, help="CUDA device")
    p.add_argument("--factored", default=None,
                   help="also write the compact factored coefficient file (.cwf) the evaluator reads directly")
    p.add_argument("--eig-fp64", action="store_true",
                   help="FP64 Householder + QR eigen-solver for every slice (default: FP32 + FP64 refinement)")
    return p


def main(argv=None) -> int:
    a = parser().parse_args(argv)
    from . import evaluator as ev
    from . import solver
    if len(a.n) != 2:
        print("the volume solver takes exactly two media: --n n_upper n_lower", file=sys.stderr)
        return 2
    from . import _lib, samples
    t0 = time.perf_counter()
    ctx = ev.Context(a.device)
    try:                                      # streamed from the file into device memory
        sample = samples.npy_to_device(ctx, a.sample)
    except _lib.ScwError:
        sample = np.load(a.sample)
    sol = solver.solve(sample, lam=a.lam, direction=a.direction, ex=a.ex, ey=a.ey, ez=a.ez, n=a.n, kappa=a.kappa,
                       size=a.size, z=a.z, coef=a.coef, external=a.external, pz=not a.npz, psf=a.psf, ctx=ctx,
                       eig_fp64=a.eig_fp64)
    t1 = time.perf_counter()
    sol.save(a.output)
    if a.factored:
        sol.to_sep().save(a.factored)
    t2 = time.perf_counter()
    Y, X = sample.shape[-2], sample.shape[-1]
    print(f"Field saved in {a.output}.")
    print(f"Number of pixels (x, y): [{X},{Y}]")
    print(f"Number of sublayers: {sol.Z}")
    print(f"Number of Fourier coefficients (Mx, My): [{sol.M[0]},{sol.M[1]}]")
    if a.log:
        print(f"solve {t1 - t0:.3f} s, write {t2 - t1:.3f} s, {ctx.launches} kernel launches")
    return 0


if __name__ == "__main__":
    sys.exit(main())
