"""Headless replacement of the viewer program sCWatterView (sCWatterView.cpp:679-796).

    python -m scwatter_gb300.scwatterview c.cw --nogui --resolution 8 --size 100 --axis 1 --output xz.npy

Options and defaults follow the reference (input file positional, --cuda/-c device, --size
extent, --resolution log2 of the plane edge, --output, --axis 0 = yz / 1 = xz / 2 = xy plane,
--center, --slice).  As in the reference, the evaluation point of the three planes is
plane_position, whose component along --axis is --slice (the other two stay 0), and the planes
span center +- size / 2.  The selected plane is saved as an [N, N, 3] complex64 .npy file.

The window, OpenGL textures and interactive controls are not built (no graphics stack on
this machine).  Their display processing runs on the GPU instead (csrc/view.cu) and can be
written out: --scalar {x, y, z, intensity} with --scalar-output (complex64 [N, N]) and
--image-output (uint8 [N, N, 3] RGB, the reference's real (green) / imaginary (blue) colour
mapping over the range of all three planes).
Evaluation uses the plain summation kernel (gpu_cw_evaluate); --method tf32x3 / bf16x3 / fp32
selects the separable evaluator for structures on a separable Fourier grid.
"""
from __future__ import annotations

import argparse
import ctypes
import os
import sys
import time

import numpy as np

MODES = {"x": 0, "y": 1, "z": 2, "intensity": 3}


def parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(prog="scwatterview", description="headless field evaluation of a .cw structure")
    p.add_argument("input", nargs="?", default="c.cw",
                   help="coupled wave structure (.cw) or compact factored coefficient file (.cwf)")
    p.add_argument("--cuda", "-c", type=int, default=0, help="CUDA device number")
    p.add_argument("--nogui", action="store_true", help="save an output file without loading the GUI")
    p.add_argument("--verbose", "-v", action="store_true")
    p.add_argument("--size", type=float, default=100.0, help="extent of the evaluated planes")
    p.add_argument("--resolution", type=int, default=8, help="plane edge 2^resolution")
    p.add_argument("--output", default="xz.npy", help="output file of the selected plane")
    p.add_argument("--axis", type=int, default=1, help="axis to cut (0 = X, 1 = Y, 2 = Z)")
    p.add_argument("--center", type=float, nargs=3, default=[0.0, 0.0, 0.0], help="centre of the sampled volume")
    p.add_argument("--slice", type=float, default=0.0, help="coordinate along the selected axis")
    p.add_argument("--method", default="plain", choices=["plain", "tf32x3", "bf16x3", "fp32"])
    p.add_argument("--scalar", default="x", choices=list(MODES))
    p.add_argument("--scalar-output", default=None)
    p.add_argument("--image-output", default=None)
    return p


def main(argv=None) -> int:
    a = parser().parse_args(argv)
    if not a.nogui:
        print("the interactive viewer needs a graphics stack, which this machine lacks; use --nogui", file=sys.stderr)
        return 2
    if a.cuda < 0:
        print("CPU-only evaluation (--cuda -1) is not supported: every evaluation runs on the GPU", file=sys.stderr)
        return 2
    import torch
    from . import _lib
    from . import evaluator as ev
    from . import separable as sp
    from .cw import CoupledWaveStructure

    t0 = time.perf_counter()
    factored = str(a.input).endswith(".cwf")
    if factored and a.method == "plain":
        print("a factored coefficient file (.cwf) is evaluated by the GEMM-form methods only", file=sys.stderr)
        return 2
    S = CoupledWaveStructure()
    if not os.path.exists(a.input) or (not factored and not S.load(a.input)):
        print(f"ERROR: file {a.input} not found", file=sys.stderr)
        return 1
    N = 2 ** a.resolution
    f = np.float32
    extent = f(a.size)
    d = extent / f(N - 1)                              # float arithmetic, as EvaluateVectorSlices
    xs, ys, zs = (f(a.center[i]) - extent / f(2) for i in range(3))
    plane = [0.0, 0.0, 0.0]
    plane[a.axis] = a.slice
    ctx = ev.Context(a.cuda)
    if a.method == "plain":
        obj = ev.WaveSet.from_cw(ctx, S)
        E_xy, E_xz, E_yz = obj.evaluate_planes_host(xs, ys, zs, plane[0], plane[1], plane[2], d, N)
    else:
        m = {"tf32x3": sp.TF32X3, "bf16x3": sp.BF16X3, "fp32": sp.FP32}[a.method]
        obj = sp.SeparableSet.load(ctx, a.input) if factored else sp.SeparableSet.from_cw(ctx, S)
        E_xy, E_xz, E_yz = obj.evaluate_planes_host(xs, ys, zs, plane[0], plane[1], plane[2], d, N, method=m)
    t1 = time.perf_counter()
    sel = {0: E_yz, 1: E_xz, 2: E_xy}[a.axis]
    np.save(a.output, np.ascontiguousarray(sel.reshape(N, N, 3)))
    if a.verbose:
        print(f"Evaluation (no gui) takes:{t1 - t0}s")
    if a.scalar_output or a.image_output:
        dE = torch.from_numpy(np.stack([E_xy, E_yz, E_xz]).reshape(-1, 3)).cuda()
        dS = torch.empty(dE.shape[0], dtype=torch.complex64, device="cuda")
        torch.cuda.synchronize()
        n = dE.shape[0]
        _lib.call("scw_view_scalar", ctx.handle, ctypes.c_void_p(dE.data_ptr()), n, MODES[a.scalar],
                  ctypes.c_void_p(dS.data_ptr()))
        mm = (ctypes.c_float * 4)()
        _lib.call("scw_view_minmax", ctx.handle, ctypes.c_void_p(dS.data_ptr()), n, mm)
        idx = {2: 0, 0: 1, 1: 2}[a.axis]          # position of the selected plane in the stack
        if a.scalar_output:
            np.save(a.scalar_output, dS.view(3, N, N)[idx].cpu().numpy())
        if a.image_output:
            prm = (ctypes.c_float * 12)(mm[0], mm[1], mm[2], mm[3], 0.0, 1.0, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0)
            rgb = torch.empty((n, 3), dtype=torch.uint8, device="cuda")
            _lib.call("scw_view_color", ctx.handle, ctypes.c_void_p(dS.data_ptr()), n, prm,
                      ctypes.c_void_p(rgb.data_ptr()))
            ctx.synchronize()
            np.save(a.image_output, rgb.view(3, N, N, 3)[idx].cpu().numpy())
    return 0


if __name__ == "__main__":
    sys.exit(main())
