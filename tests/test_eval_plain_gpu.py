"""Plain CUDA summation evaluator vs the FP64 oracle (gpuEvaluator.cu:28-165 semantics)."""
import numpy as np
import pytest

from oracle import oracle_lib as ol
from oracle import solve_oracle as so
from tests._util import rel_l2, solved_case, to_structure

pytestmark = pytest.mark.gpu

# Plain form: FP32 per-point phase after an FP64 re-base to each 16x32 tile centre,
# FP32 accumulation per 256-wave batch, FP64 accumulation across batches.
TOL_PLAIN = 2e-5


@pytest.fixture(scope="module")
def ctx():
    from scwatter_gb300 import evaluator as ev
    return ev.Context(0)


@pytest.fixture(scope="module")
def case():
    return solved_case(shape=(3, 16, 16), coef=(5, 5), seed=1)


def _oracle_planes(W, b, e, zl, rule, x_start, y_start, z_start, x, y, z, d, N):
    thr = ol.thresholds(zl, rule)
    out = []
    for axis, a0, b0, c in [(ol.AXIS_XY, x_start, y_start, z), (ol.AXIS_XZ, x_start, z_start, y),
                            (ol.AXIS_YZ, y_start, z_start, x)]:
        P = ol.plane_points(axis, a0, b0, c, d, N)
        out.append(ol.eval_points_f64(W, b, e, thr, P.reshape(-1, 3)).reshape(N, N, 3))
    return out


@pytest.mark.parametrize("N,zplane", [(64, 0.25), (37, -2.0), (48, 5.3)])
def test_planes_vs_fp64_oracle(ctx, case, N, zplane):
    from scwatter_gb300 import evaluator as ev
    _, _, _, c = case
    W, b, e, zl = so.unpack(c)
    ws = ev.WaveSet.from_cw(ctx, to_structure(c))
    ext = 24.0
    d = np.float32(ext / (N - 1))
    xs, ys, zs = np.float32(-ext / 2), np.float32(-ext / 2), np.float32(-ext / 2)
    got = ws.evaluate_planes_host(xs, ys, zs, 0.7, -1.3, zplane, d, N)
    ref = _oracle_planes(W, b, e, zl, "gpu", xs, ys, zs, 0.7, -1.3, zplane, d, N)
    for g, r, name in zip(got, ref, ["xy", "xz", "yz"]):
        err = rel_l2(g, r)
        assert max(err) < TOL_PLAIN, (name, err)


def test_float_table_dropin_path(ctx, case):
    """gpu_initialize from the float globals (waves wound to the origin), as the viewer does."""
    from scwatter_gb300 import evaluator as ev
    _, _, _, c = case
    S = to_structure(c)
    ev.cw_allocate(S)
    ev.cw_unpack(S)
    ev.gpu_initialize(0)
    N = 40
    E = [np.zeros(N * N * 3, np.complex64) for _ in range(3)]
    d = np.float32(20.0 / (N - 1))
    ev.gpu_cw_evaluate(E[0], E[1], E[2], -10.0, -10.0, -10.0, 0.0, 0.0, 0.4, d, N, 0)
    W32, b, e, zl = so.unpack(c, np.complex64)
    ref = _oracle_planes(W32.astype(np.complex128), b, e, zl, "gpu", np.float32(-10), np.float32(-10),
                         np.float32(-10), 0.0, 0.0, 0.4, d, N)
    for g, r in zip(E, ref):
        assert max(rel_l2(g, r)) < TOL_PLAIN


def test_cpu_region_rule_and_volume(ctx, case):
    from scwatter_gb300 import evaluator as ev
    import torch
    _, _, _, c = case
    W, b, e, zl = so.unpack(c)
    ws = ev.WaveSet.from_cw(ctx, to_structure(c))
    ws.set_region_rule(ev.REGION_RULE_CPU)
    Nx, Ny, Nz = 20, 17, 9
    dx, dy, dz = np.float32(0.9), np.float32(1.1), np.float32(0.5)
    x0, y0, z0 = np.float32(-8), np.float32(-9), np.float32(-2.5)
    out = torch.zeros((Nz, Ny, Nx, 3), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    ws.eval_volume_device(x0, y0, z0, dx, dy, dz, Nx, Ny, Nz, out.data_ptr())
    ctx.synchronize()
    got = out.cpu().numpy()
    ix = (x0 + dx * np.arange(Nx, dtype=np.float32)).astype(np.float32)
    iy = (y0 + dy * np.arange(Ny, dtype=np.float32)).astype(np.float32)
    iz = (z0 + dz * np.arange(Nz, dtype=np.float32)).astype(np.float32)
    P = np.stack(np.meshgrid(ix, iy, iz, indexing="xy"), -1)  # [Ny, Nx, Nz, 3]
    P = np.transpose(P, (2, 0, 1, 3))
    ref = ol.eval_points_f64(W, b, e, ol.thresholds(zl, "cpu"), P.reshape(-1, 3)).reshape(Nz, Ny, Nx, 3)
    assert max(rel_l2(got, ref)) < TOL_PLAIN


def test_deterministic_and_external_mode(ctx):
    from scwatter_gb300 import evaluator as ev
    _, _, _, c = solved_case(shape=(2, 12, 12), coef=(3, 3), seed=4, external=True)
    W, b, e, zl = so.unpack(c)
    ws = ev.WaveSet.from_cw(ctx, to_structure(c))
    N = 33
    args = (np.float32(-6), np.float32(-6), np.float32(-6), 0.1, 0.2, 0.0, np.float32(12 / 32), N)
    a = ws.evaluate_planes_host(*args)
    bb = ws.evaluate_planes_host(*args)
    for x, y in zip(a, bb):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    # internal field is zero in --external mode (interior layers have no waves)
    ref = _oracle_planes(W, b, e, zl, "gpu", *args[:3], 0.1, 0.2, 0.0, args[6], N)
    for g, r in zip(a, ref):
        assert max(rel_l2(g, r)) < TOL_PLAIN
