"""The allocation-free plane entry point against the ordinary one.

``scw_eval_plane_device_static`` exists for callers that must not allocate GPU memory while
they run (a host that pre-sizes one device pool and counts any other cudaMalloc as a leak, a
frame loop that may not stall on the allocator, a plug-in host that forbids device
allocation): its split-K scratch is an array compiled into the library.  These tests call it
through the C ABI, twice in a row per plane, and compare each result with
``scw_eval_plane_device`` on the same wave set.  The file is named so pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from tests._util import rel_l2, solved_case, to_structure

pytestmark = pytest.mark.gpu

# same tolerance as the plain evaluator's own tests: the two entry points split the wave
# lists differently, so their FP32 partial sums round differently
TOL_PLAIN = 2e-5


@pytest.fixture(scope="module")
def waves():
    from scwatter_gb300 import evaluator as ev
    ctx = ev.Context(0)
    _, _, _, c = solved_case(shape=(3, 16, 16), coef=(5, 5), seed=1)
    ws = ev.WaveSet.from_cw(ctx, to_structure(c))
    return ctx, ws


def _plane(name, ws, axis, a0, b0, c, d, N, poison):
    import torch
    from scwatter_gb300 import _lib
    out = torch.full((N, N, 3), complex(float("nan"), float("nan")) if poison else 0j, dtype=torch.complex64,
                     device="cuda")
    torch.cuda.synchronize()
    _lib.call(name, ws.handle, int(axis), ctypes.c_float(a0), ctypes.c_float(b0), ctypes.c_float(c),
              ctypes.c_float(d), int(N), ctypes.c_void_p(out.data_ptr()))
    return out


# (axis, a_start, b_start, c, d, N): split-K planes crossing several regions per tile,
# an xy plane, and planes with more tiles than the scratch array holds (run unsplit)
PLANES = [
    (2, -12.0, -12.0, 0.7, 24.0 / 47, 48),
    (1, -10.0, -3.0, -1.3, 6.0 / 39, 40),
    (0, -8.0, -8.0, 0.25, 16.0 / 63, 64),
    (1, -6.0, -6.0, 0.5, 12.0 / 1099, 1100),
]


@pytest.mark.parametrize("plane", PLANES)
def test_static_matches_device_entry_twice(waves, plane):
    ctx, ws = waves
    axis, a0, b0, c, d, N = plane
    ref = _plane("scw_eval_plane_device", ws, axis, a0, b0, c, d, N, False)
    ctx.synchronize()
    ref = ref.cpu().numpy()
    got = []
    for _ in range(2):
        g = _plane("scw_eval_plane_device_static", ws, axis, a0, b0, c, d, N, True)
        ctx.synchronize()
        got.append(g.cpu().numpy())
    for g in got:
        assert np.isfinite(g).all()
        assert max(rel_l2(g, ref)) < TOL_PLAIN
    # the scratch keeps the previous call's contents; a repeated call gives the same bits
    assert np.array_equal(got[0].view(np.uint32), got[1].view(np.uint32))


def test_static_two_planes_back_to_back(waves):
    """Two different planes in a row on one stream, then both checked."""
    ctx, ws = waves
    a, b = PLANES[0], PLANES[2]
    ga = _plane("scw_eval_plane_device_static", ws, *a, True)
    gb = _plane("scw_eval_plane_device_static", ws, *b, True)
    ctx.synchronize()
    ra = _plane("scw_eval_plane_device", ws, *a, False)
    rb = _plane("scw_eval_plane_device", ws, *b, False)
    ctx.synchronize()
    assert max(rel_l2(ga.cpu().numpy(), ra.cpu().numpy())) < TOL_PLAIN
    assert max(rel_l2(gb.cpu().numpy(), rb.cpu().numpy())) < TOL_PLAIN


def test_static_rejects_oversized_plane(waves):
    from scwatter_gb300 import _lib
    _, ws = waves
    with pytest.raises(_lib.ScwError) as e:
        _lib.call("scw_eval_plane_device_static", ws.handle, 0, ctypes.c_float(0), ctypes.c_float(0),
                  ctypes.c_float(0), ctypes.c_float(1), 16385, ctypes.c_void_p(16))
    assert e.value.status == 1 and "maximum" in str(e.value)


def test_static_allocates_no_device_memory(waves):
    """The entry point's one promise: after a first call (which may load the library's GPU
    module on the device), further calls with caller-allocated outputs leave the device's free
    memory exactly where it was."""
    import torch
    from scwatter_gb300 import _lib
    ctx, ws = waves
    axis, a0, b0, c, d, N = PLANES[0]                    # a split-K plane: both kernels run
    outs = [torch.zeros((N, N, 3), dtype=torch.complex64, device="cuda") for _ in range(4)]

    def call(o):
        _lib.call("scw_eval_plane_device_static", ws.handle, int(axis), ctypes.c_float(a0), ctypes.c_float(b0),
                  ctypes.c_float(c), ctypes.c_float(d), int(N), ctypes.c_void_p(o.data_ptr()))

    call(outs[0])
    ctx.synchronize()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for o in outs[1:]:
        call(o)
    ctx.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    for o in outs[1:]:
        assert torch.equal(o, outs[0])
