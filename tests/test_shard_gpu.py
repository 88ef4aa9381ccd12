"""z-slabs evaluated separately (as one process per GPU would) put together are the whole volume.

On one GPU the slabs run one after the other; each is evaluated by the slab entry points, which
give every plane the z-value the whole volume gives it, so the reassembled volume must equal the
single-call volume bit for bit.
"""
import numpy as np
import pytest

from scwatter_gb300 import shard

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [2, 3])
def test_slabs_reassemble_the_volume(world):
    import torch
    from scwatter_gb300 import evaluator as ev
    from scwatter_gb300 import synthetic
    from scwatter_gb300.separable import TF32X3, SeparableSet
    ctx = ev.Context(0)
    fs = synthetic.make_factored(M0=8, M1=6, Z=4, size=(16.0, 12.0, 4.0), seed=3)
    sep = SeparableSet.from_factored(ctx, fs)
    g = dict(x0=np.float32(-9), y0=np.float32(-7), z0=np.float32(-2.7), dx=np.float32(0.3), dy=np.float32(0.45),
             dz=np.float32(0.07), Nx=61, Ny=33, Nz=80)
    args = (g["x0"], g["y0"], g["z0"], g["dx"], g["dy"], g["dz"])
    whole = torch.zeros((g["Nz"], g["Ny"], g["Nx"], 3), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    sep.eval_volume_device(*args, g["Nx"], g["Ny"], g["Nz"], whole.data_ptr(), method=TF32X3)
    ctx.synchronize()
    whole = whole.cpu().numpy()
    MF, J = fs.MF, fs.gamma_dn.shape[1]
    waves = np.array([2 * MF] + [4 * MF * MF] * fs.Z + [MF])      # per region: exterior, slices, exterior
    w = shard.plane_weights(g["z0"], g["dz"], g["Nz"], fs.z, waves)
    Qh = torch.empty((fs.Z, 2, 3, MF, J), dtype=torch.complex64, pin_memory=True)
    Qh[:, 0] = torch.from_numpy(fs.Q_dn.astype(np.complex64))
    Qh[:, 1] = torch.from_numpy(fs.Q_up.astype(np.complex64))
    dev, host = np.zeros_like(whole), np.zeros_like(whole)
    for r in range(world):
        k0, k1 = shard.slab_bounds(g["Nz"], world, r, w)
        if k1 == k0:
            continue
        slab = torch.zeros((k1 - k0, g["Ny"], g["Nx"], 3), dtype=torch.complex64, device="cuda")
        torch.cuda.synchronize()
        sep.eval_slab_device(*args, g["Nx"], g["Ny"], k0, k1, slab.data_ptr(), method=TF32X3)
        ctx.synchronize()
        dev[k0:k1] = slab.cpu().numpy()
        host[k0:k1] = sep.eval_slab_host(Qh, *args, g["Nx"], g["Ny"], k0, k1, method=TF32X3)
    assert np.array_equal(dev.view(np.uint32), whole.view(np.uint32))
    assert np.array_equal(host.view(np.uint32), whole.view(np.uint32))
