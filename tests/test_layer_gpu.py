"""Homogeneous multilayer solve (sCWatterLayer) on the GPU against its CPU restatement, and
the restatement against the coupled-wave solve of the same stack (a physics cross-check)."""
import numpy as np
import pytest

from oracle import layer_oracle as lo
from oracle import oracle_lib as ol
from oracle import solve_oracle as so
from tests._util import rel_l2


def _waves(count, n0=1.0, lam=2.0, seed=0):
    from scwatter_gb300.layer import incident_waves
    if count == 1:
        return incident_waves((0.3, -0.2, 1.0), [1, 0.5j, 0], n0, lam)
    return incident_waves((0.1, 0.2, 1.0), [1, 0.5j, 0], n0, lam, alpha=0.5, beta=0.1, samples=(count, 3),
                          mode="polar")


def test_oracle_single_interface_is_fresnel():
    """L = 2: the reflected / transmitted amplitudes of a TE wave are Fresnel's."""
    n1, n2, lam = 1.0, 1.5, 1.0
    th = 0.4
    d = np.array([np.sin(th), 0.0, np.cos(th)])
    k = 2 * np.pi / lam
    wave = np.array([0, 1, 0, d[0] * n1 * k, 0, d[2] * n1 * k], complex)   # E along y: TE
    x, _ = lo.solve_layers(wave, [n1, n2], [0.0], [0.0], lam)
    ct = np.cos(th)
    cs = np.sqrt(1 - (n1 / n2 * np.sin(th)) ** 2)
    r = (n1 * ct - n2 * cs) / (n1 * ct + n2 * cs)
    t = 2 * n1 * ct / (n1 * ct + n2 * cs)
    assert abs(x[0, 3 + 1] - r) < 1e-12 and abs(x[0, 6 + 1] - t) < 1e-12


def test_oracle_slab_matches_coupled_wave_solve():
    """A homogeneous slab: the layered solution and the coupled-wave solve give the same field."""
    lam, nslab, th = 1.0, 1.4 + 0.02j, 0.2
    sample = np.full((2, 8, 8), nslab, complex)
    d = (np.sin(th), 0.0, np.cos(th))
    prm = so.SolveParams(lam=lam, direction=d, ex=(0, 0), ey=(1, 0), size=(8.0, 8.0, 2.0), coef=(1, 1))
    cw_rcwa = so.pack(so.solve(sample, prm), prm)
    # the layered program uses M_PI in k; the volume solver its truncated PI: match wavelengths
    lam_l = lam * np.pi / so.PI_REF
    k = 2 * np.pi / lam_l
    dd = np.array(d) / np.linalg.norm(d)
    wave = np.array([0, 1, 0, dd[0] * k, 0, dd[2] * k], complex)
    _, cw_l = lo.solve_layers(wave, [1.0, nslab.real, 1.0], [nslab.imag, 0.0], [-1.0, 1.0], lam_l)
    pts = np.stack([np.zeros(40), np.zeros(40), np.linspace(-3, 3, 40)], 1)
    f = []
    for cw in (cw_rcwa, cw_l):
        W, b, e, zl = so.unpack(cw)
        f.append(ol.eval_points_f64(W, b, e, ol.thresholds(zl, "cpu"), pts))
    assert max(rel_l2(f[0], f[1])) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("count,L", [(1, 4), (8, 3), (5, 6)])
def test_gpu_matches_cpu(count, L):
    from scwatter_gb300 import evaluator as ev
    from scwatter_gb300.layer import solve_layers
    rng = np.random.default_rng(L)
    n = [1.0] + list(rng.uniform(1.2, 1.8, L - 1))
    kappa = list(rng.uniform(0, 0.05, L - 1))
    z = list(np.cumsum(rng.uniform(0.5, 2.0, L - 1)) - 2.0)
    lam = 2.0
    waves = _waves(count, n[0], lam)
    ctx = ev.Context(0)
    x, S = solve_layers(ctx, waves, n, kappa, z, lam)
    xr, cw = lo.solve_layers(waves, n, kappa, z, lam)
    assert np.abs(x - xr).max() < 1e-11 * np.abs(xr).max()
    for L_, pr, pt in zip(S.Layers, cw.Pr, cw.Pt):
        np.testing.assert_allclose(L_.Pr, pr, rtol=0, atol=1e-11)
        np.testing.assert_allclose(L_.Pt, pt, rtol=0, atol=1e-11)


@pytest.mark.gpu
def test_command_line(tmp_path):
    from scwatter_gb300 import layer
    from scwatter_gb300.cw import CoupledWaveStructure
    out = tmp_path / "a.cw"
    rc = layer.main(["--alpha", "0", "--output", str(out), "--output_sample", str(tmp_path / "s.npy")])
    assert rc == 0
    S = CoupledWaveStructure()
    assert S.load(str(out)) and len(S.Layers) == 3 and len(S.Pi) == 1
    assert np.load(tmp_path / "s.npy").shape == (2, 1, 1)
