"""Viewer display processing on the GPU (sCWatterView.cpp:200-352) against its CPU restatement,
and the headless viewer front end (sCWatterView.cpp:679-796) against the FP64 oracle."""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle_lib as ol
from oracle import solve_oracle as so
from oracle import view_oracle as vo
from tests._util import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from scwatter_gb300 import evaluator as ev
    return ev.Context(0)


def test_scalar_minmax_color_match_cpu(ctx):
    import torch
    from scwatter_gb300 import _lib
    rng = np.random.default_rng(0)
    n = 3 * 37 * 37
    E = (rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))).astype(np.complex64)
    E[5, 1] = np.nan
    dE = torch.from_numpy(E).cuda()
    for mode in range(4):
        dS = torch.empty(n, dtype=torch.complex64, device="cuda")
        torch.cuda.synchronize()
        _lib.call("scw_view_scalar", ctx.handle, ctypes.c_void_p(dE.data_ptr()), n, mode, ctypes.c_void_p(dS.data_ptr()))
        ctx.synchronize()
        S = dS.cpu().numpy()
        ref = vo.scalar(E, mode)
        assert np.array_equal(S.view(np.uint32), ref.view(np.uint32)) or np.allclose(S, ref, equal_nan=True)
        mm = (ctypes.c_float * 4)()
        _lib.call("scw_view_minmax", ctx.handle, ctypes.c_void_p(dS.data_ptr()), n, mm)
        assert tuple(mm) == pytest.approx(vo.minmax(ref), rel=0, abs=0)
        for show in [(1, 1), (1, 0), (0, 1)]:
            prm = (ctypes.c_float * 12)(mm[0], mm[1], mm[2], mm[3], 0.2, 1.0, 0.0, 0.0, 0.5, 1.0, show[0], show[1])
            rgb = torch.empty((n, 3), dtype=torch.uint8, device="cuda")
            _lib.call("scw_view_color", ctx.handle, ctypes.c_void_p(dS.data_ptr()), n, prm,
                      ctypes.c_void_p(rgb.data_ptr()))
            ctx.synchronize()
            want = vo.color(ref, mm[0], mm[1], mm[2], mm[3], (0.2, 1.0, 0.0), (0.0, 0.5, 1.0), bool(show[0]),
                            bool(show[1]))
            assert np.array_equal(rgb.cpu().numpy(), want)


@pytest.mark.parametrize("axis,method", [(1, "plain"), (2, "tf32x3"), (0, "plain")])
def test_headless_viewer_writes_the_selected_plane(tmp_path, axis, method):
    from scwatter_gb300 import scwatterview
    golden = os.path.join(os.path.dirname(__file__), "golden", "spheres_2x8x8_c3.cw")
    out = tmp_path / "plane.npy"
    img = tmp_path / "img.npy"
    sc = tmp_path / "s.npy"
    rc = scwatterview.main([golden, "--nogui", "--resolution", "4", "--size", "9", "--axis", str(axis),
                            "--slice", "0.3", "--center", "0.5", "-0.5", "0.2", "--output", str(out),
                            "--method", method, "--scalar", "intensity", "--scalar-output", str(sc),
                            "--image-output", str(img)])
    assert rc == 0
    got = np.load(out)
    N = 16
    f = np.float32
    d = f(9) / f(N - 1)
    st = [f(0.5) - f(9) / f(2), f(-0.5) - f(9) / f(2), f(0.2) - f(9) / f(2)]
    cw = so.cw_from_bytes(open(golden, "rb").read())
    W, b, e, zl = so.unpack(cw)
    thr = ol.thresholds(zl, "gpu")
    if axis == 2:
        P = ol.plane_points(ol.AXIS_XY, st[0], st[1], 0.3, d, N)
    elif axis == 1:
        P = ol.plane_points(ol.AXIS_XZ, st[0], st[2], 0.3, d, N)
    else:
        P = ol.plane_points(ol.AXIS_YZ, st[1], st[2], 0.3, d, N)
    ref = ol.eval_points_f64(W, b, e, thr, P.reshape(-1, 3)).reshape(N, N, 3)
    assert max(rel_l2(got, ref)) < 2e-5
    s = np.load(sc)
    assert np.allclose(s, vo.scalar(got, vo.INTENSITY))
    im = np.load(img)
    assert im.shape == (N, N, 3) and im.dtype == np.uint8 and im[..., 0].max() == 0


def test_headless_viewer_refuses_gui_and_cpu():
    from scwatter_gb300 import scwatterview
    assert scwatterview.main(["x.cw"]) == 2
    assert scwatterview.main(["x.cw", "--nogui", "--cuda", "-1"]) == 2
