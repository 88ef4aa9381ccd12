"""Pins of the FP64 oracle by physics known answers (the reference ships no golden vectors).

* homogeneous slab, s- and p-polarised, normal and oblique incidence, lossless and absorbing,
  one and several slices: the field from the oracle's solve + packing + evaluation equals an
  independent transfer-matrix solution;
* tangential E is continuous across every boundary of a heterogeneous sample;
* the oracle's helper quirks (fftShift2d, orthogonalize, Eigen_Sort order) behave as the
  reference code they restate.
"""
import numpy as np
import pytest

from oracle import oracle_lib as ol
from oracle import solve_oracle as so
from scwatter_gb300 import samples
from tests._util import solved_case


def _slab_1d(ns, lam, z0, z1, sx, zq, pol):
    k = 2 * so.PI_REF / lam
    eps = [1.0 + 0j, ns ** 2, 1.0 + 0j]
    kz = [k * np.sqrt(e - sx ** 2 + 0j) for e in eps]
    D = z1 - z0
    inc = np.exp(1j * kz[0] * z0)
    e = np.exp(1j * kz[1] * D)
    g = [kz[i] if pol == "te" else kz[i] / (k * eps[i]) for i in range(3)]
    A = np.array([[1, -1, -e, 0], [-g[0], -g[1], g[1] * e, 0], [0, e, 1, -1], [0, g[1] * e, -g[1], -g[2]]], complex)
    r, a, b, t = np.linalg.solve(A, np.array([-inc, -g[0] * inc, 0, 0], complex))
    F, B, I = [], [], []
    for z in zq:
        if z < z0:
            i, f, bb = 0, np.exp(1j * kz[0] * z), r * np.exp(-1j * kz[0] * (z - z0))
        elif z < z1:
            i, f, bb = 1, a * np.exp(1j * kz[1] * (z - z0)), b * np.exp(-1j * kz[1] * (z - z1))
        else:
            i, f, bb = 2, t * np.exp(1j * kz[2] * (z - z1)), 0
        F.append(f), B.append(bb), I.append(i)
    F, B = np.array(F), np.array(B)
    if pol == "te":
        return F + B, None
    gi = np.array([g[i] for i in I])
    ez = np.array([-(k * sx) / (k * eps[i]) for i in I]) * (F + B)
    return gi * (F - B), ez


@pytest.mark.parametrize("ns,nl,sx", [(1.5 + 0j, 1, 0.0), (1.3 + 0.05j, 3, 0.0), (1.5, 2, 0.3), (2.0 + 0.1j, 4, 0.4)])
def test_slab_te(ns, nl, sx):
    s = samples.slab((nl, 6, 6), ns)
    prm = so.SolveParams(lam=1.0, direction=(sx, 0.0, np.sqrt(1 - sx ** 2)), ex=(0, 0), ey=(1, 0), ez=(0, 0),
                         size=(6.0, 6.0, 2.0), coef=(3, 3))
    r = so.solve(s, prm)
    W, b, e, zl = so.unpack(so.pack(r, prm))
    zq = np.linspace(-3, 3, 41).astype(np.float32)
    pts = np.stack([np.zeros_like(zq), np.zeros_like(zq), zq], 1)
    E = ol.eval_points_f64(W, b, e, ol.thresholds(zl, "cpu"), pts)
    ey, _ = _slab_1d(ns, 1.0, r.z[0], r.z[-1], sx, zq.astype(np.float64), "te")
    assert np.abs(E[:, 1] - ey).max() < 1e-12
    assert np.abs(E[:, 0]).max() < 1e-12 and np.abs(E[:, 2]).max() < 1e-12


@pytest.mark.parametrize("ns,nl,sx", [(1.5 + 0j, 1, 0.3), (1.3 + 0.05j, 3, 0.5)])
def test_slab_tm_including_ez_from_h(ns, nl, sx):
    s = samples.slab((nl, 6, 6), ns)
    ct = np.sqrt(1 - sx ** 2)
    prm = so.SolveParams(lam=1.0, direction=(sx, 0, ct), ex=(ct, 0), ey=(0, 0), ez=(-sx, 0), size=(6.0, 6.0, 2.0),
                         coef=(3, 3))
    r = so.solve(s, prm)
    W, b, e, zl = so.unpack(so.pack(r, prm))
    zq = np.linspace(-3, 3, 41).astype(np.float32)
    pts = np.stack([np.zeros_like(zq), np.zeros_like(zq), zq], 1)
    E = ol.eval_points_f64(W, b, e, ol.thresholds(zl, "cpu"), pts)
    ex, ez = _slab_1d(ns, 1.0, r.z[0], r.z[-1], sx, zq.astype(np.float64), "tm")
    assert np.abs(E[:, 0] - ex).max() < 1e-12
    assert np.abs(E[:, 2] - ez).max() < 1e-12


@pytest.mark.parametrize("coef,shape,direction", [((5, 5), (3, 16, 16), (0, 0, 1)), ((5, 3), (2, 16, 12), (0.2, 0.1, 1)),
                                                  ((4, 6), (2, 12, 16), (0, 0, 1))])
def test_tangential_continuity(coef, shape, direction):
    _, _, _, c = solved_case(shape=shape, coef=coef, seed=1, direction=direction, ex=(1, 0), ey=(0.3, 0.2))
    W, b, e, zl = so.unpack(c)
    rng = np.random.default_rng(0)
    for l, zz in enumerate(zl):
        pts = np.stack([rng.uniform(-5, 5, 8), rng.uniform(-5, 5, 8), np.full(8, zz)], 1).astype(np.float32)
        A = ol.eval_points_f64(W[b[l]:e[l]], [0], [e[l] - b[l]], [], pts)
        B = ol.eval_points_f64(W[b[l + 1]:e[l + 1]], [0], [e[l + 1] - b[l + 1]], [], pts)
        assert np.abs(A[:, :2] - B[:, :2]).max() <= 1e-12 * max(1.0, np.abs(A[:, :2]).max())


def test_fft_shift_quirk_and_numpy_agreement():
    for m, n in [(4, 6), (5, 7), (5, 6), (1, 1)]:
        a = np.arange(m * n).reshape(m, n)
        assert np.array_equal(so.fft_shift_2d(a), np.fft.fftshift(a))
    # even rows, odd columns: the reference builds column index [2, 0, 1, 2, 3] for n = 5
    a = np.arange(4 * 5).reshape(4, 5)
    assert np.array_equal(so.fft_shift_2d(a)[0], a[2, [2, 0, 1, 2, 3]])


def test_orthogonalize_and_sort_order():
    E = so.orthogonalize([1, 0, 0], [0, 0, 1])
    assert np.allclose(E, [1, 0, 0])
    d = np.array([0.6, 0, 0.8])
    E = so.orthogonalize([1, 0, 0], d)
    assert abs(np.dot(E, d)) < 1e-15
    ev = np.array([1 + 0.5j, -1 - 0.5j, 2 + 0.1j, -2 - 0.1j])
    V = np.eye(4)
    w, _ = so.eigen_sort(ev, V)
    # even slots: largest Im first; odd slots: smallest Im first (sCWatter.cpp:207-212)
    assert np.allclose(w, [1 + 0.5j, -1 - 0.5j, 2 + 0.1j, -2 - 0.1j])
