"""Host-level split over processes (one GPU each): z-slab and batch partitioning (CPU).

The world_size-2 test runs two gloo ranks on the CPU: each evaluates its weighted z-slab of a
small separable sample's volume (with the FP64 oracle standing in for its GPU) at the z-values
the whole volume gives its planes, the slabs are gathered, and the result must equal the
single-process volume bit for bit.
"""
import os
import socket

import numpy as np
import pytest

from scwatter_gb300 import shard


def test_slab_bounds_cover_every_plane_once():
    for Nz in (0, 1, 5, 64, 257):
        for world in (1, 2, 3, 8):
            b = [shard.slab_bounds(Nz, world, r) for r in range(world)]
            assert b[0][0] == 0 and b[-1][1] == Nz
            for (a0, a1), (c0, c1) in zip(b, b[1:]):
                assert a1 == c0 and a0 <= a1
            sizes = [k1 - k0 for k0, k1 in b]
            assert max(sizes) - min(sizes) <= 1


def test_slab_bounds_follow_the_weights():
    w = np.array([1.0] * 10 + [9.0] * 10)          # exterior planes cheap, interior planes dear
    b = [shard.slab_bounds(20, 2, r, w) for r in range(2)]
    loads = [w[k0:k1].sum() for k0, k1 in b]
    assert b[0][0] == 0 and b[1][1] == 20 and b[0][1] == b[1][0]
    assert abs(loads[0] - loads[1]) <= 9.0
    assert shard.slab_bounds(4, 2, 0, np.zeros(4)) == (0, 2)
    with pytest.raises(ValueError):
        shard.slab_bounds(4, 2, 2)


def test_lpt_partition():
    costs = [7, 3, 5, 5, 2, 9, 1]
    parts = shard.lpt_partition(costs, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(costs)))
    loads = sorted(sum(costs[i] for i in p) for p in parts)
    assert loads == [10, 11, 11]


def test_region_of_z_matches_the_reference_rules():
    from oracle import oracle_lib as ol
    zl = np.array([-1.0, 0.0, 1.0])
    z = np.array([-2, -1.0005, -0.9995, 0.0, 0.9999, 1.0, 3.0], np.float32)
    for rule in ("gpu", "cpu"):
        thr = ol.thresholds(zl, rule)
        want = [sum(1 for t in thr if float(v) >= t) for v in z]
        assert list(shard.region_of_z(z, zl, rule)) == want


def _case():
    from oracle import solve_oracle as so
    from scwatter_gb300 import synthetic
    fs = synthetic.make_factored(M0=4, M1=3, Z=3, size=(8.0, 6.0, 3.0), seed=4)
    Pi, zsl, Pr, Pt = synthetic.to_cw_arrays(fs)
    W, b, e, zl = so.unpack(so.CW(Pi=Pi, z=zsl, Pr=Pr, Pt=Pt))
    grid = dict(x0=np.float32(-4), y0=np.float32(-3), z0=np.float32(-2.3), dx=np.float32(0.5), dy=np.float32(0.6),
                dz=np.float32(0.2), Nx=9, Ny=7, Nz=23)
    return W, b, e, zl, grid


def _eval_planes(W, b, e, zl, g, k0, k1):
    from oracle import oracle_lib as ol
    zs = shard.plane_z(g["z0"], g["dz"], g["Nz"])[k0:k1]
    ix = (g["x0"] + g["dx"] * np.arange(g["Nx"], dtype=np.float32)).astype(np.float32)
    iy = (g["y0"] + g["dy"] * np.arange(g["Ny"], dtype=np.float32)).astype(np.float32)
    P = np.stack(np.meshgrid(zs, iy, ix, indexing="ij"), -1)[..., ::-1]
    f = ol.eval_points_f64(W, b, e, ol.thresholds(zl, "gpu"), P.reshape(-1, 3), nthreads=1)
    return f.reshape(k1 - k0, g["Ny"], g["Nx"], 3).astype(np.complex64)


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        W, b, e, zl, g = _case()
        waves = np.asarray(e) - np.asarray(b)
        w = shard.plane_weights(g["z0"], g["dz"], g["Nz"], zl, waves)
        k0, k1 = shard.slab_bounds(g["Nz"], world, rank, w)
        slab = _eval_planes(W, b, e, zl, g, k0, k1)
        full = shard.gather_slabs(slab, k0, k1, g["Nz"])
        if rank == 0:
            np.save(out_path, full.numpy())
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_gloo_ranks_reassemble_the_volume(tmp_path):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    out = str(tmp_path / "gathered.npy")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = np.load(out)
    W, b, e, zl, g = _case()
    ref = _eval_planes(W, b, e, zl, g, 0, g["Nz"])
    assert got.shape == ref.shape
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
