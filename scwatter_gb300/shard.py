"""Host-level split of the field evaluation and of batches over processes, one GPU each.

The path shards without any exchange of data (evaluation planes, samples and per-slice
eigen-solves are independent): the reference evaluates plane by plane (gpuEvaluator.cu:131-165)
and solves one sample per sCWatter run (sCWatter.cpp:501-988).  So N processes, one per GPU,
each take

* a contiguous z-slab of the evaluation grid (:func:`slab_bounds`), balanced by the plane
  weights (points x modes per plane), and evaluate it with the slab entry points
  (``scw_sep_eval_slab_device`` / ``scw_sep_eval_slab_host``), which give every plane the
  z-value the whole volume gives it -- the slabs put together are the single-process volume;
* a longest-processing-time share of a batch's samples (:func:`lpt_partition`).

No collective is on the data path.  :func:`gather_slabs` reassembles a volume on one rank
after the fact (for checks and output), over whatever process group the caller has.
"""
from __future__ import annotations

import os

import numpy as np


def rank_env():
    """(world_size, rank, local_rank) of this process, from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def region_of_z(z, z_layers, rule="gpu"):
    """Region index (0 .. L) of each z under the reference's region rules: the last boundary l
    with z >= z_l - 0.001 (gpuEvaluator.cu:34) or z >= z_l (cpuEvaluator.cpp:303) gives l + 1."""
    zl = np.asarray(z_layers, dtype=np.float32).astype(np.float64)
    thr = zl - 0.001 if rule == "gpu" else zl
    z = np.asarray(z, dtype=np.float32).astype(np.float64)
    return np.searchsorted(thr, z, side="right")


def plane_z(z_start, dz, Nz):
    """z of each plane as the evaluators compute it: z_start + dz * k, rounded to float after the
    product and after the sum."""
    k = np.arange(Nz, dtype=np.float32)
    return (np.float32(z_start) + (np.float32(dz) * k).astype(np.float32)).astype(np.float32)


def plane_weights(z_start, dz, Nz, z_layers, waves_per_region, rule="gpu"):
    """Work of each plane in modes per point: the wave count of the region it lies in."""
    r = region_of_z(plane_z(z_start, dz, Nz), z_layers, rule)
    return np.asarray(waves_per_region, dtype=np.float64)[r]


def slab_bounds(Nz, world, rank, weights=None):
    """[k0, k1) of rank's z-slab: contiguous, in rank order, covering 0 .. Nz exactly once, with the
    cut points where the running weight comes nearest r / world of the total (equal plane counts when
    weights is None or all zero).  Ranks beyond the number of planes get empty slabs."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    w = np.ones(Nz) if weights is None else np.asarray(weights, dtype=np.float64)
    if len(w) != Nz:
        raise ValueError("one weight per plane")
    if Nz == 0:
        return 0, 0
    if w.sum() <= 0:
        w = np.ones(Nz)
    c = np.concatenate([[0.0], np.cumsum(w)])
    cuts = [0]
    for r in range(1, world):
        # the plane boundary whose prefix weight is nearest r/world of the total
        t = c[-1] * r / world
        k = int(np.searchsorted(c, t, side="left"))
        if 0 < k <= Nz and t - c[k - 1] < c[k] - t:
            k -= 1
        cuts.append(min(max(k, cuts[-1]), Nz))
    cuts.append(Nz)
    return cuts[rank], cuts[rank + 1]


def lpt_partition(costs, world):
    """Longest-processing-time assignment: items in decreasing cost, each to the least-loaded
    rank.  Returns one sorted index list per rank."""
    loads = np.zeros(world)
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i)):
        r = int(np.argmin(loads))
        parts[r].append(i)
        loads[r] += float(costs[i])
    return [sorted(p) for p in parts]


def gather_slabs(slab, k0, k1, Nz, group=None, dst=0):
    """Reassembles the [Nz, ...] volume on rank ``dst`` from every rank's [k1 - k0, ...] slab
    (torch.distributed, any backend; CPU tensors for gloo).  Returns the volume on ``dst``, None
    elsewhere."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    t = torch.as_tensor(np.ascontiguousarray(slab)) if not isinstance(slab, torch.Tensor) else slab.contiguous()
    bounds = torch.tensor([k0, k1], dtype=torch.int64)
    all_bounds = [torch.zeros(2, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(all_bounds, bounds, group=group)
    tail = tuple(t.shape[1:])
    flat = t.reshape(-1).view(torch.float32) if t.is_complex() else t.reshape(-1)
    sizes = [int(b[1] - b[0]) * int(np.prod(tail)) * (2 if t.is_complex() else 1) for b in all_bounds]
    mx = max(sizes) if sizes else 0
    buf = torch.zeros(mx, dtype=flat.dtype)
    buf[: flat.numel()] = flat
    bufs = [torch.zeros(mx, dtype=flat.dtype) for _ in range(world)]
    dist.all_gather(bufs, buf, group=group)
    if rank != dst:
        return None
    out = torch.zeros((Nz,) + tail, dtype=t.dtype)
    for b, part, n in zip(all_bounds, bufs, sizes):
        a0, a1 = int(b[0]), int(b[1])
        if a1 > a0:
            piece = part[:n]
            piece = piece.view(torch.complex64) if t.dtype == torch.complex64 else piece
            out[a0:a1] = piece.reshape((a1 - a0,) + tail)
    return out
