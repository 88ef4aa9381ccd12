"""Separable (GEMM-form) evaluator vs the FP64 oracle (same field as gpu_cw_evaluate)."""
import numpy as np
import pytest

from oracle import oracle_lib as ol
from oracle import solve_oracle as so
from tests._util import rel_l2, solved_case, to_structure

pytestmark = pytest.mark.gpu

# Separable form: FP64-reduced phases rounded to FP32; FP32 stage-1 sums per 256-mode chunk
# with FP64 running sums; FP32 (SIMT) or 3-product split tensor-core output GEMM.
TOL_SEP = 1e-5
TOL = {1: TOL_SEP, 2: TOL_SEP, 3: 1e-4}     # FP32 SIMT, 3xTF32, split-BF16 (16-bit operands)


@pytest.fixture(scope="module")
def ctx():
    from scwatter_gb300 import evaluator as ev
    return ev.Context(0)


def _planes_oracle(c, rule, xs, ys, zs, x, y, z, d, N):
    W, b, e, zl = so.unpack(c)
    thr = ol.thresholds(zl, rule)
    out = []
    for axis, a0, b0, cc in [(ol.AXIS_XY, xs, ys, z), (ol.AXIS_XZ, xs, zs, y), (ol.AXIS_YZ, ys, zs, x)]:
        P = ol.plane_points(axis, a0, b0, cc, d, N)
        out.append(ol.eval_points_f64(W, b, e, thr, P.reshape(-1, 3)).reshape(N, N, 3))
    return out


@pytest.mark.parametrize("method", [1, 2, 3])
@pytest.mark.parametrize("shape,coef,direction", [((3, 16, 16), (5, 5), (0, 0, 1)),
                                                  ((2, 12, 16), (5, 3), (0.2, 0.1, 1.0))])
def test_solved_cw_planes(ctx, shape, coef, direction, method):
    from scwatter_gb300.separable import SeparableSet
    _, _, _, c = solved_case(shape=shape, coef=coef, seed=2, direction=direction)
    sep = SeparableSet.from_cw(ctx, to_structure(c))
    M0, M1, Z, J = sep.info()
    assert (M0, M1, Z) == (coef[0], coef[1], shape[0])
    N = 48
    ext = float(max(shape[1], shape[2]) + 8)
    d = np.float32(ext / (N - 1))
    xs = ys = zs = np.float32(-ext / 2)
    got = sep.evaluate_planes_host(xs, ys, zs, 0.3, -0.6, 0.2, d, N, method=method)
    ref = _planes_oracle(c, "gpu", xs, ys, zs, 0.3, -0.6, 0.2, d, N)
    for g, r, name in zip(got, ref, ["xy", "xz", "yz"]):
        err = rel_l2(g, r)
        assert max(err) < TOL[method], (name, err)


@pytest.mark.parametrize("method", [1, 2, 3])
def test_synthetic_volume(ctx, method):
    import torch
    from scwatter_gb300 import synthetic
    from scwatter_gb300.separable import SeparableSet
    fs = synthetic.make_factored(M0=6, M1=4, Z=3, size=(12.0, 10.0, 3.0), seed=5)
    sep = SeparableSet.from_factored(ctx, fs)
    Nx, Ny, Nz = 37, 21, 11
    x0, y0, z0 = np.float32(-7), np.float32(-6), np.float32(-2.5)
    dx, dy, dz = np.float32(0.4), np.float32(0.55), np.float32(0.5)
    out = torch.zeros((Nz, Ny, Nx, 3), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    sep.eval_volume_device(x0, y0, z0, dx, dy, dz, Nx, Ny, Nz, out.data_ptr(), method=method)
    ctx.synchronize()
    got = out.cpu().numpy()
    Pi, zsl, Pr, Pt = synthetic.to_cw_arrays(fs)
    c = so.CW(Pi=Pi, z=zsl, Pr=Pr, Pt=Pt)
    W, b, e, zl = so.unpack(c)
    ix = (x0 + dx * np.arange(Nx, dtype=np.float32)).astype(np.float32)
    iy = (y0 + dy * np.arange(Ny, dtype=np.float32)).astype(np.float32)
    iz = (z0 + dz * np.arange(Nz, dtype=np.float32)).astype(np.float32)
    P = np.stack(np.meshgrid(iz, iy, ix, indexing="ij"), -1)[..., ::-1]   # [Nz, Ny, Nx, (x, y, z)]
    ref = ol.eval_points_f64(W, b, e, ol.thresholds(zl, "gpu"), P.reshape(-1, 3)).reshape(Nz, Ny, Nx, 3)
    assert max(rel_l2(got, ref)) < TOL[method]


@pytest.mark.parametrize("Nx", [200, 199])
@pytest.mark.parametrize("method,tol", [(2, 2e-6), (3, 5e-5)])
def test_tensor_core_matches_simt_many_tiles(ctx, method, tol, Nx):
    """Enough rows that every CTA runs several row tiles (both TMEM accumulators, both
    operand buffers), columns not a multiple of the 128-wide tile."""
    import torch
    from scwatter_gb300 import synthetic
    from scwatter_gb300.separable import SeparableSet
    fs = synthetic.make_factored(M0=10, M1=8, Z=4, size=(20.0, 16.0, 4.0), seed=9)
    sep = SeparableSet.from_factored(ctx, fs)
    Ny, Nz = 64, 40
    args = (np.float32(-10), np.float32(-8), np.float32(-3), np.float32(0.1), np.float32(0.25), np.float32(0.15),
            Nx, Ny, Nz)
    outs = []
    for m in (1, method):
        o = torch.zeros((Nz, Ny, Nx, 3), dtype=torch.complex64, device="cuda")
        torch.cuda.synchronize()
        sep.eval_volume_device(*args, o.data_ptr(), method=m)
        ctx.synchronize()
        outs.append(o.cpu().numpy())
    assert max(rel_l2(outs[1], outs[0])) < tol


def test_not_separable_is_rejected(ctx):
    """A .cw whose waves do not share a harmonic grid is refused with SCW_ERR_UNSUPPORTED."""
    from scwatter_gb300 import _lib
    from scwatter_gb300.separable import SeparableSet
    _, _, _, c = solved_case(shape=(2, 12, 12), coef=(3, 3), seed=3)
    S = to_structure(c)
    S.Layers[1].Pr = S.Layers[1].Pr.copy()
    S.Layers[1].Pr[5, 5] += 0.125        # one mode's kz differs across harmonics
    with pytest.raises(_lib.ScwError) as ei:
        SeparableSet.from_cw(ctx, S)
    assert ei.value.status == 9


def _trimmed(fs, J):
    """The factored sample with only the first J modes per half (odd J exercises the padded
    device rows)."""
    import dataclasses
    return dataclasses.replace(fs, gamma_dn=fs.gamma_dn[:, :J], gamma_up=fs.gamma_up[:, :J],
                               Q_dn=fs.Q_dn[..., :J], Q_up=fs.Q_up[..., :J])


@pytest.mark.parametrize("odd", [False, True])
def test_volume_from_host_amplitudes(ctx, odd):
    """scw_sep_eval_volume_host (slices uploaded while earlier ones are evaluated, planes read
    back as they finish) against the device-resident evaluation of the same set; the set it
    runs on starts with zero amplitudes, so every interior value must come from Q_host.  The
    grid reaches above and below the sample (exterior planes need no upload) and is long
    enough for several output slabs per slice."""
    import torch
    from scwatter_gb300 import synthetic
    from scwatter_gb300.separable import SeparableSet, TF32X3
    fs = synthetic.make_factored(M0=6, M1=4, Z=5, size=(12.0, 10.0, 5.0), seed=11)
    if odd:
        fs = _trimmed(fs, 2 * fs.MF - 3)
    J = fs.gamma_dn.shape[1]
    ref_set = SeparableSet.from_factored(ctx, fs)
    zero = dataclasses_zero(fs)
    set_ = SeparableSet.from_factored(ctx, zero)
    Nx, Ny, Nz = 45, 23, 70
    args = (np.float32(-7), np.float32(-6), np.float32(-3.5), np.float32(0.3), np.float32(0.5), np.float32(0.1),
            Nx, Ny, Nz)
    ref = torch.zeros((Nz, Ny, Nx, 3), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    ref_set.eval_volume_device(*args, ref.data_ptr(), method=TF32X3)
    ctx.synchronize()
    ref = ref.cpu().numpy()
    Qh = torch.empty((fs.Z, 2, 3, fs.MF, J), dtype=torch.complex64, pin_memory=True)
    Qh[:, 0] = torch.from_numpy(np.ascontiguousarray(fs.Q_dn, dtype=np.complex64))
    Qh[:, 1] = torch.from_numpy(np.ascontiguousarray(fs.Q_up, dtype=np.complex64))
    # one slice per upload, 3 planes per read-back slab: many slabs cycle through the 3 slots
    set_.set_streaming(chunk_bytes=1, slab_bytes=3 * Nx * Ny * 24)
    for out in (None, torch.empty((Nz, Ny, Nx, 3), dtype=torch.complex64, pin_memory=True)):
        got = set_.eval_volume_host(Qh, *args, out=out, method=TF32X3)
        got = got.numpy() if hasattr(got, "numpy") and not isinstance(got, np.ndarray) else got
        assert np.isfinite(got).all()
        assert max(rel_l2(got, ref, floor=0.0)) < 1e-6
    set_.set_streaming()                 # defaults: every slice in one upload chunk here
    got = set_.eval_volume_host(Qh, *args, method=TF32X3)
    assert max(rel_l2(got, ref, floor=0.0)) < 1e-6
    # the set's own device copy now holds the uploaded amplitudes
    again = torch.zeros((Nz, Ny, Nx, 3), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    set_.eval_volume_device(*args, again.data_ptr(), method=TF32X3)
    ctx.synchronize()
    assert max(rel_l2(again.cpu().numpy(), ref, floor=0.0)) < 1e-6


def dataclasses_zero(fs):
    import dataclasses
    return dataclasses.replace(fs, Q_dn=np.zeros_like(fs.Q_dn), Q_up=np.zeros_like(fs.Q_up))


def test_volume_from_host_rejects_wrong_shape(ctx):
    from scwatter_gb300 import synthetic
    from scwatter_gb300.separable import SeparableSet
    fs = synthetic.make_factored(M0=4, M1=4, Z=2, size=(8.0, 8.0, 2.0), seed=1)
    s = SeparableSet.from_factored(ctx, fs)
    with pytest.raises(ValueError):
        s.eval_volume_host(np.zeros((2, 2, 3, 16, 31), np.complex64), 0, 0, 0, 1, 1, 1, 4, 4, 4)


def _volume_oracle(fs, grid):
    from scwatter_gb300 import synthetic
    Pi, zsl, Pr, Pt = synthetic.to_cw_arrays(fs)
    W, b, e, zl = so.unpack(so.CW(Pi=Pi, z=zsl, Pr=Pr, Pt=Pt))
    x0, y0, z0, dx, dy, dz, Nx, Ny, Nz = grid
    ix = (x0 + dx * np.arange(Nx, dtype=np.float32)).astype(np.float32)
    iy = (y0 + dy * np.arange(Ny, dtype=np.float32)).astype(np.float32)
    iz = (z0 + dz * np.arange(Nz, dtype=np.float32)).astype(np.float32)
    P = np.stack(np.meshgrid(iz, iy, ix, indexing="ij"), -1)[..., ::-1]
    return ol.eval_points_f64(W, b, e, ol.thresholds(zl, "gpu"), P.reshape(-1, 3)).reshape(Nz, Ny, Nx, 3)


def _eval_device(ctx, sep, grid, method):
    import torch
    *geo, Nx, Ny, Nz = grid
    o = torch.zeros((Nz, Ny, Nx, 3), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    sep.eval_volume_device(*geo, Nx, Ny, Nz, o.data_ptr(), method=method)
    ctx.synchronize()
    return o.cpu().numpy()


PAIRED_GRID = (np.float32(-7), np.float32(-6), np.float32(-2.5), np.float32(0.4), np.float32(0.55), np.float32(0.5),
               37, 21, 11)


@pytest.mark.parametrize("method", [1, 2, 3])
def test_paired_set_volume(ctx, method):
    """A paired set (one block V per slice, amplitudes folded into the FP64 phases) against the
    FP64 oracle summing the same waves, Q_dn = V diag(beta_dn), Q_up = diag(1, 1, -1) V diag(beta_up)."""
    from scwatter_gb300 import synthetic
    from scwatter_gb300.separable import SeparableSet
    ps = synthetic.make_paired(M0=6, M1=4, Z=3, size=(12.0, 10.0, 3.0), seed=5)
    sep = SeparableSet.from_paired(ctx, ps)
    assert sep.form() == 1
    got = _eval_device(ctx, sep, PAIRED_GRID, method)
    ref = _volume_oracle(ps.to_factored(), PAIRED_GRID)
    assert max(rel_l2(got, ref, floor=0.0)) < TOL[method]


def test_paired_set_matches_two_half_set(ctx):
    """The same coefficients as a paired set and as a two-half set give the same volume."""
    from scwatter_gb300 import synthetic
    from scwatter_gb300.separable import TF32X3, SeparableSet
    ps = synthetic.make_paired(M0=8, M1=6, Z=4, size=(16.0, 12.0, 4.0), seed=8)
    a = _eval_device(ctx, SeparableSet.from_paired(ctx, ps), PAIRED_GRID, TF32X3)
    b = _eval_device(ctx, SeparableSet.from_factored(ctx, ps.to_factored()), PAIRED_GRID, TF32X3)
    assert max(rel_l2(a, b, floor=0.0)) < 1e-6


@pytest.mark.parametrize("odd", [False, True])
def test_paired_set_from_host_amplitudes(ctx, odd):
    """scw_sep_eval_volume_host on a paired set: one block [3][MF][J] per slice from host memory."""
    import dataclasses
    import torch
    from scwatter_gb300 import synthetic
    from scwatter_gb300.separable import TF32X3, SeparableSet
    ps = synthetic.make_paired(M0=6, M1=4, Z=5, size=(12.0, 10.0, 5.0), seed=12)
    if odd:
        J = 2 * 24 - 3
        base = dataclasses.replace(ps.base, gamma_dn=ps.base.gamma_dn[:, :J], gamma_up=ps.base.gamma_up[:, :J])
        ps = dataclasses.replace(ps, base=base, V=ps.V[..., :J], beta_dn=ps.beta_dn[:, :J], beta_up=ps.beta_up[:, :J])
    grid = (np.float32(-7), np.float32(-6), np.float32(-3.5), np.float32(0.3), np.float32(0.5), np.float32(0.1),
            45, 23, 70)
    ref = _eval_device(ctx, SeparableSet.from_paired(ctx, ps), grid, TF32X3)
    zero = dataclasses.replace(ps, V=np.zeros_like(ps.V))
    s = SeparableSet.from_paired(ctx, zero)
    assert s.host_block_shape() == ps.V.shape
    Vh = torch.from_numpy(np.ascontiguousarray(ps.V)).pin_memory()
    s.set_streaming(chunk_bytes=1, slab_bytes=3 * 45 * 23 * 24)
    got = s.eval_volume_host(Vh, *grid, method=TF32X3)
    assert max(rel_l2(got, ref, floor=0.0)) < 1e-6


def test_paired_factored_file_round_trip(ctx, tmp_path):
    """A paired set is written as SCWSEP02 (half the amplitude bytes), reads back to the same
    field bit for bit, and the host reader rebuilds its two-half blocks."""
    from scwatter_gb300 import factored, synthetic
    from scwatter_gb300.separable import TF32X3, SeparableSet
    ps = synthetic.make_paired(M0=5, M1=4, Z=3, size=(10.0, 8.0, 3.0), seed=2)
    s1 = SeparableSet.from_paired(ctx, ps)
    f = tmp_path / "p.cwf"
    s1.save(f)
    assert f.read_bytes()[:8] == b"SCWSEP02"
    s2 = SeparableSet.load(ctx, f)
    assert s2.form() == 1
    a = _eval_device(ctx, s1, PAIRED_GRID, TF32X3)
    b = _eval_device(ctx, s2, PAIRED_GRID, TF32X3)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    host = factored.read_cwf(f)
    fs = ps.to_factored()
    np.testing.assert_allclose(host.Q[:, 0], fs.Q_dn, rtol=0, atol=1e-7 * np.abs(fs.Q_dn).max())
    np.testing.assert_allclose(host.Q[:, 1], fs.Q_up, rtol=0, atol=1e-7 * np.abs(fs.Q_up).max())


@pytest.mark.parametrize("dz,Nz", [(1.0, 4), (0.5, 8), (0.3, 11), (0.1, 31)])
def test_contraction_tile_shapes_bit_identical(ctx, dz, Nz):
    """Both contraction tile shapes (scw_sep_set_tiles: default rows per warp, or half) give the
    same volume bit for bit, for plane densities that select 1 to 8 planes per contraction
    group, on a paired and a two-half set."""
    from scwatter_gb300 import synthetic
    from scwatter_gb300.separable import TF32X3, SeparableSet
    ps = synthetic.make_paired(M0=8, M1=6, Z=3, size=(16.0, 12.0, 3.0), seed=11)
    grid = (np.float32(-7), np.float32(-6), np.float32(-1.6), np.float32(0.4), np.float32(0.55), np.float32(dz),
            37, 21, Nz)
    for sep in (SeparableSet.from_paired(ctx, ps), SeparableSet.from_factored(ctx, ps.to_factored())):
        a = _eval_device(ctx, sep, grid, TF32X3)
        sep.set_tiles(1)
        b = _eval_device(ctx, sep, grid, TF32X3)
        sep.set_tiles(0)
        assert np.array_equal(a, b)


@pytest.mark.parametrize("M0,method", [(44, 2), (48, 2), (48, 3), (80, 3)])
def test_tensor_core_wide_synthesis_axis(ctx, M0, method):
    """The widest synthesis axes the tensor-core kernels take (3xTF32 up to 48 harmonics, split-BF16
    up to 80): every 16-byte core column of the B operand built, against the FP64 oracle."""
    from scwatter_gb300 import synthetic
    from scwatter_gb300.separable import SeparableSet
    fs = synthetic.make_factored(M0=M0, M1=3, Z=2, size=(2.0 * M0, 6.0, 2.0), seed=13)
    sep = SeparableSet.from_factored(ctx, fs)
    grid = (np.float32(-M0), np.float32(-2.5), np.float32(-0.9), np.float32(2.0 * M0 / 149), np.float32(1.0),
            np.float32(0.6), 150, 6, 3)
    got = _eval_device(ctx, sep, grid, method)
    ref = _volume_oracle(fs, grid)
    assert max(rel_l2(got, ref, floor=0.0)) < TOL[method]


@pytest.mark.parametrize("method", [1, 2, 3])
def test_pipelined_slab_matches_one_pass_volume(ctx, method):
    """With the pipeline on (scw_sep_set_pipeline), a slab of >= 32 planes is evaluated in chunks
    whose two stages overlap on two streams (the output GEMM on half the SMs); every plane equals
    the one-pass volume bit for bit, and so does the slab evaluated with per-kernel timing on
    (stages in sequence)."""
    import torch
    from scwatter_gb300 import synthetic
    from scwatter_gb300.separable import SeparableSet
    ps = synthetic.make_paired(M0=8, M1=6, Z=3, size=(16.0, 12.0, 3.0), seed=21)
    sep = SeparableSet.from_paired(ctx, ps)
    sep.set_pipeline(4, 2)
    x0, y0, z0, dx, dy, dz, Nx, Ny, Nz = (np.float32(-7), np.float32(-6), np.float32(-1.7), np.float32(0.1),
                                          np.float32(0.2), np.float32(0.05), 200, 64, 70)
    vol = _eval_device(ctx, sep, (x0, y0, z0, dx, dy, dz, Nx, Ny, Nz), method)
    outs = []
    for timing in (False, True):
        o = torch.zeros((Nz - 3, Ny, Nx, 3), dtype=torch.complex64, device="cuda")
        ctx.set_timing(timing)
        torch.cuda.synchronize()
        sep.eval_slab_device(x0, y0, z0, dx, dy, dz, Nx, Ny, 3, Nz, o.data_ptr(), method=method)
        ctx.synchronize()
        ctx.set_timing(False)
        outs.append(o.cpu().numpy())
    assert np.array_equal(outs[0], vol[3:]) and np.array_equal(outs[1], vol[3:])
