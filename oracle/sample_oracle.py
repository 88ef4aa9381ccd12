"""CPU restatement of the device sample generators (test infrastructure only).

``grf`` restates ``scw_gen_grf`` (scwatter_gb300/csrc/samples.cu) in FP64 numpy: splitmix64
counter noise with Box-Muller, periodic separable Gaussian filter truncated at 4 correlation
lengths, min-max normalisation and the affine map to the refractive index.  The generator has
no reference counterpart (the reference generates samples with tilesample.py, which needs
scikit-image); the restatement pins the device stream bit-for-bit in its integer part and to
rounding in its floating-point part.
"""
import numpy as np

_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def unit(h):
    return ((np.asarray(h, dtype=np.uint64) >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def noise(shape, seed):
    idx = np.arange(int(np.prod(shape)), dtype=np.uint64)
    base = mix64(np.uint64(seed) ^ mix64(idx))
    with np.errstate(over="ignore"):
        u1, u2 = unit(mix64(base)), unit(mix64(base + np.uint64(1)))
    return (np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)).reshape(shape)


def grf(shape, corr_px=8.0, n_range=(1.0, 1.6), kappa_max=0.02, seed=0):
    g = noise(shape, seed)
    R = int(np.ceil(4.0 * corr_px))
    t = np.arange(-R, R + 1)
    w = np.exp(-0.5 * t.astype(np.float64) ** 2 / (corr_px * corr_px))
    w /= w.sum()
    for axis in (2, 1, 0):
        g = sum(w[k + R] * np.roll(g, -k, axis=axis) for k in range(-R, R + 1))
    lo, hi = g.min(), g.max()
    tt = (g - lo) / max(hi - lo, 1e-30)
    with np.errstate(over="ignore"):
        kappa = kappa_max * unit(mix64(mix64(np.uint64(seed)) ^ np.uint64(0x6B617070615F3031)))
    return (n_range[0] + (n_range[1] - n_range[0]) * tt) + 1j * (kappa * tt)
