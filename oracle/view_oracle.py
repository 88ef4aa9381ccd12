"""CPU restatement of the viewer's display processing (test infrastructure only).

sCWatterView.cpp:300-352 EvaluateScalarSlices, :268-297 CalculateMinMax, :194-220 clamp and
EvaluateColorValue, :222-262 EvaluateColorSlices; float32 arithmetic with every operation
rounded separately, as the reference's host code computes it.
"""
import numpy as np

X, Y, Z, INTENSITY = 0, 1, 2, 3


def scalar(E, mode):
    """E [..., 3] complex64 -> S [...] complex64."""
    E = np.asarray(E, dtype=np.complex64)
    if mode < 3:
        return E[..., mode].copy()
    re, im = E.real.astype(np.float32), E.imag.astype(np.float32)
    s = np.zeros(E.shape[:-1], np.float32)
    for c in range(3):
        p = (re[..., c] * re[..., c]).astype(np.float32) + (im[..., c] * im[..., c]).astype(np.float32)
        s = (s + p.astype(np.float32)).astype(np.float32)
    return (s + 0j).astype(np.complex64)


def minmax(*planes):
    """real min, real max, imaginary min, imaginary max over all planes (CalculateMinMax)."""
    v = np.concatenate([np.asarray(p, np.complex64).ravel() for p in planes])
    return (float(np.nanmin(v.real)), float(np.nanmax(v.real)), float(np.nanmin(v.imag)), float(np.nanmax(v.imag)))


def _clamp(v):
    v = np.where(np.isnan(v), np.float32(0), v)
    return np.clip(v, np.float32(0), np.float32(1)).astype(np.float32)


def color(S, real_low, real_high, imag_low, imag_high, real_color=(0.0, 1.0, 0.0), imag_color=(0.0, 0.0, 1.0),
          show_real=True, show_imag=True):
    """RGB bytes [..., 3] (EvaluateColorValue, then channel * 255 truncated to unsigned char)."""
    S = np.asarray(S, np.complex64)
    f = np.float32
    with np.errstate(divide="ignore", invalid="ignore"):
        rn = _clamp(((S.real.astype(f) - f(real_low)).astype(f) / (f(real_high) - f(real_low))).astype(f))
        inn = _clamp(((S.imag.astype(f) - f(imag_low)).astype(f) / (f(imag_high) - f(imag_low))).astype(f))
    out = np.zeros(S.shape + (3,), np.uint8)
    for c in range(3):
        x = np.zeros(S.shape, f)
        if show_real:
            x = (x + (rn * f(real_color[c])).astype(f)).astype(f)
        if show_imag:
            x = (x + (inn * f(imag_color[c])).astype(f)).astype(f)
        out[..., c] = (x * f(255)).astype(f).astype(np.uint8)
    return out
