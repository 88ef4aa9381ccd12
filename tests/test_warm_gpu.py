"""Learned eigen warm start: the network's kernels against the CPU oracle, the warm eigen-solver's
gates and fallback, and what the trained network gains over the homogeneous-medium guess."""
import numpy as np
import pytest

from oracle import mlp_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from scwatter_gb300 import evaluator as ev
    return ev.Context(0)


def test_mlp_forward_and_gradients_match_cpu_oracle(ctx):
    import torch
    from scwatter_gb300.warmstart import MLP
    n_in, width, n_out, B = 12, 16, 10, 7
    net = MLP(ctx, n_in, width, n_out, seed=3)
    rng = np.random.default_rng(0)
    X = rng.standard_normal((B, n_in)).astype(np.float32)
    T = rng.standard_normal((B, n_out)).astype(np.float32)
    p = net.params()
    Y = net.forward(torch.from_numpy(X).cuda()).cpu().numpy()
    Yr, _ = mlp_oracle.forward(p, X, n_in, width, n_out)
    assert np.abs(Y - Yr).max() < 1e-5 * max(1.0, np.abs(Yr).max())
    loss, g = net.gradients(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda())
    lr_, gr = mlp_oracle.loss_and_grad(p, X, T, n_in, width, n_out)
    assert abs(loss - lr_) < 1e-5 * lr_
    assert np.linalg.norm(g - gr) / np.linalg.norm(gr) < 1e-5
    # central differences of the oracle confirm the oracle's own gradient on a few parameters
    for i in rng.choice(len(p), 6, replace=False):
        e = np.zeros_like(p, dtype=np.float64)
        e[i] = 1e-6
        fd = (mlp_oracle.loss_and_grad(p + e, X, T, n_in, width, n_out)[0] -
              mlp_oracle.loss_and_grad(p - e, X, T, n_in, width, n_out)[0]) / 2e-6
        assert abs(fd - gr[i]) < 1e-6 + 1e-4 * abs(gr[i])


def test_mlp_training_reduces_loss(ctx):
    import torch
    from scwatter_gb300.warmstart import MLP
    rng = np.random.default_rng(1)
    n_in, n_out, B = 8, 6, 256
    A = rng.standard_normal((n_out, n_in))
    X = rng.standard_normal((B, n_in)).astype(np.float32)
    T = np.tanh(X @ A.T).astype(np.float32)
    net = MLP(ctx, n_in, 64, n_out, seed=0)
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()
    first = net.train_step(Xd, Td, 3e-3)
    for _ in range(300):
        last = net.train_step(Xd, Td, 3e-3)
    assert last < 0.05 * first


def _grf_problems(ctx, count, Z=4, M=4, seed=0):
    from scwatter_gb300 import samples
    from scwatter_gb300.warmstart import layer_problems
    out = []
    for s in range(count):
        vol = samples.gaussian_random_field((Z, 16, 16), corr_px=4.0, n_range=(1.0, 1.6), kappa_max=0.02,
                                            seed=seed + s)
        out.append(layer_problems(ctx, vol, lam=1.0, direction=(0.2, 0.1, 1.0), size=(16.0, 16.0, float(Z)),
                                  coef=(M, M)))
    return out


def _max_residual(PQ, W, V):
    import torch
    R = torch.bmm(PQ, V) - V * W[:, None, :]
    rn = torch.linalg.vector_norm(R, dim=1) / (torch.linalg.matrix_norm(PQ)[:, None] *
                                                torch.linalg.vector_norm(V, dim=1))
    return float(rn.max())


def test_warm_eig_near_exact_shifts_accepted(ctx):
    from scwatter_gb300.warmstart import plain_eig, warm_eig
    lp = _grf_problems(ctx, 1)[0]
    W0, V0 = plain_eig(ctx, lp.PQ)
    rng = np.random.default_rng(2)
    w0 = W0.cpu().numpy()
    noise = 1e-6 * np.abs(w0).max() * (rng.standard_normal(w0.shape) + 1j * rng.standard_normal(w0.shape))
    import torch
    sh = torch.from_numpy(w0 + noise).cuda()
    W, V, acc, st = warm_eig(ctx, lp.PQ, sh)
    assert acc.all() and st["fell_back"] == 0 and st["max_residual"] <= 1e-11
    w = W.cpu().numpy()
    for l in range(w.shape[0]):
        d = np.abs(w0[l][:, None] - w[l][None, :]).min(axis=1)
        assert d.max() < 1e-10 * np.abs(w0[l]).max()
    assert _max_residual(lp.PQ, W, V) < 1e-11


def test_warm_eig_duplicate_modes_fall_back(ctx):
    import torch
    from scwatter_gb300.warmstart import plain_eig, warm_eig
    lp = _grf_problems(ctx, 1, seed=5)[0]
    W0, _ = plain_eig(ctx, lp.PQ)
    w0 = W0.cpu().numpy()
    sh = torch.from_numpy(np.repeat(w0.mean(axis=1, keepdims=True), w0.shape[1], axis=1)).cuda()
    W, V, acc, st = warm_eig(ctx, lp.PQ, sh)
    assert not acc.any() and st["fell_back"] == w0.shape[0]       # mode count gate
    assert _max_residual(lp.PQ, W, V) < 1e-11                    # the plain solver's answer
    w = W.cpu().numpy()
    for l in range(w.shape[0]):
        d = np.abs(w0[l][:, None] - w[l][None, :]).min(axis=1)
        assert d.max() < 1e-12 * np.abs(w0[l]).max()


def test_trained_network_beats_homogeneous_guess(ctx):
    """A/B: shifts from the trained network vs the homogeneous-medium values on held-out layers."""
    import torch
    from scwatter_gb300.warmstart import WarmStart, plain_eig, sorted_desc, warm_eig
    probs = _grf_problems(ctx, 84, seed=100)
    eigs, coefs, bases, modes = [], [], [], []
    for lp in probs:
        W0, _ = plain_eig(ctx, lp.PQ)
        eigs.append(sorted_desc(W0.cpu().numpy()))
        coefs.append(lp.coef)
        bases.append(lp.baseline)
        modes.append(lp.modes)
    eigs, coefs, bases, modes = (np.concatenate(eigs), np.concatenate(coefs), np.concatenate(bases),
                                 np.concatenate(modes))
    ntr = 80 * 4
    MF = probs[0].M0 * probs[0].M1
    ws = WarmStart(ctx, MF, width=512, seed=0)
    hist = ws.fit(coefs[:ntr], eigs[:ntr], bases[:ntr], epochs=400, lr=1e-3, batch=64)
    assert hist[-1] < 0.2 * hist[0]
    pred = ws.predict(coefs[ntr:], bases[ntr:])
    err_mlp = np.abs(pred - eigs[ntr:]).mean()
    err_base = np.abs(bases[ntr:] - eigs[ntr:]).mean()
    assert err_mlp < 0.5 * err_base
    PQ = torch.cat([lp.PQ for lp in probs[80:]])
    W_m, V_m, acc_m, st_m = warm_eig(ctx, PQ, torch.from_numpy(pred).cuda(), modes[ntr:])
    _, _, acc_b, st_b = warm_eig(ctx, PQ, torch.from_numpy(bases[ntr:]).cuda(), modes[ntr:])
    # why per-eigenpair inverse iteration is not accepted: it reaches the intended eigenpair only
    # when the shift lies within half the gap to the nearest other eigenvalue
    truth = eigs[ntr:]
    gaps = np.array([[np.min(np.abs(row[i] - np.delete(row, i))) for i in range(len(row))] for row in truth])
    reach_m = float(np.mean(np.abs(pred - truth) < 0.5 * gaps))
    reach_b = float(np.mean(np.abs(bases[ntr:] - truth) < 0.5 * gaps))
    print(f"held-out layers {len(acc_m)}: accepted with network {acc_m.sum()} (mean RQI iterations "
          f"{st_m['mean_iterations']:.2f}, repaired tasks {st_m['repaired']}), with the homogeneous guess "
          f"{acc_b.sum()} ({st_b['mean_iterations']:.2f}, {st_b['repaired']}); "
          f"mean |shift - eigenvalue| {err_mlp:.3e} vs {err_base:.3e}; shifts within half the nearest gap "
          f"{reach_m:.3f} vs {reach_b:.3f}")
    # strict gains of the network over the homogeneous-medium guess: closer shifts (asserted
    # above) and less repair work.  Acceptance is out of reach for both: the shifts would have to
    # lie within half the gap to the nearest other eigenvalue, and (measured) hardly any do, so
    # inverse iteration from them lands on neighbours and the mode-count gate refuses the layer
    assert st_m["repaired"] < st_b["repaired"]
    assert reach_m <= 0.05 and reach_b <= 0.05
    assert _max_residual(PQ, W_m, V_m) < 1e-11         # accepted or fallen back, always correct
