"""CPU restatement of the reference program sCWatterLayer (test infrastructure only).

sCWatterLayer.cpp:119-267 (InitLayerProperties, InitSz, SetBoundaryConditions,
SetGaussianConstraints, SetBoundaryConstraints, mat2waves) and :356-425 (per incident wave:
solve, wind each layer's waves to its interface, build the CoupledWaveStructure), in FP64
numpy, for one or more incident plane waves given as records [E0x, E0y, E0z, kx, ky, kz].
The focused-beam samplers (tira's SolidAnglePolar / SolidAngleMC) are not part of the reference
sources; callers pass the incident waves.
"""
import numpy as np

from oracle import solve_oracle as so


def layer_system(wave, ri, z, n0, k):
    """A (6L x 6L), b (6L) for one incident plane wave; ri: L complex indices."""
    L = len(ri)
    N = 6 * L
    A = np.zeros((N, N), complex)
    b = np.zeros(N, complex)
    kr = np.real(wave[3:6])
    s = kr / np.linalg.norm(kr)                                        # p.getDirection()
    sz = np.sqrt(np.asarray(ri, complex) ** 2 - (s[0] * n0) ** 2 - (s[1] * n0) ** 2)

    def M(row, layer, d, c):
        return row, layer * 6 + d * 3 + c

    T, R = 0, 1
    for c in range(3):
        A[M(c, 0, T, c)] = 1
        b[c] = wave[c]
        A[M(3 + c, L - 1, R, c)] = 1
    start = 6
    for l in range(L - 1):
        A[M(start + l, l, R, 0)] = s[0]
        A[M(start + l, l, R, 1)] = s[1]
        A[M(start + l, l, R, 2)] = -sz[l]
    start += L - 2
    for l in range(1, L):
        A[M(start + l, l, T, 0)] = s[0]
        A[M(start + l, l, T, 1)] = s[1]
        A[M(start + l, l, T, 2)] = sz[l]
    start = 6 + 2 * (L - 1)
    for l in range(L - 1):
        zn = z[l] if l == 0 else z[l] - z[l - 1]
        zp = 0.0 if l == L - 2 else z[l] - z[l + 1]
        en = np.exp(1j * k * sz[l] * zn)
        ep = np.exp(-1j * k * sz[l + 1] * zp)
        r0 = start + 4 * l
        A[M(r0, l, T, 0)] = en
        A[M(r0, l, R, 0)] = 1
        A[M(r0, l + 1, T, 0)] = -1
        A[M(r0, l + 1, R, 0)] = -ep
        A[M(r0 + 1, l, T, 1)] = en
        A[M(r0 + 1, l, R, 1)] = 1
        A[M(r0 + 1, l + 1, T, 1)] = -1
        A[M(r0 + 1, l + 1, R, 1)] = -ep
        A[M(r0 + 2, l, T, 2)] = s[1] * en
        A[M(r0 + 2, l, T, 1)] = -sz[l] * en
        A[M(r0 + 2, l, R, 2)] = s[1]
        A[M(r0 + 2, l, R, 1)] = sz[l]
        A[M(r0 + 2, l + 1, T, 2)] = -s[1]
        A[M(r0 + 2, l + 1, T, 1)] = sz[l + 1]
        A[M(r0 + 2, l + 1, R, 2)] = -s[1] * ep
        A[M(r0 + 2, l + 1, R, 1)] = -sz[l + 1] * ep
        A[M(r0 + 3, l, T, 0)] = sz[l] * en
        A[M(r0 + 3, l, T, 2)] = -s[0] * en
        A[M(r0 + 3, l, R, 0)] = -sz[l]
        A[M(r0 + 3, l, R, 2)] = -s[0]
        A[M(r0 + 3, l + 1, T, 0)] = -sz[l + 1]
        A[M(r0 + 3, l + 1, T, 2)] = s[0]
        A[M(r0 + 3, l + 1, R, 0)] = sz[l + 1] * ep
        A[M(r0 + 3, l + 1, R, 2)] = s[0] * ep
    return A, b, s, sz


def solve_layers(waves, n, kappa, z, lam):
    """Returns (x [count, 6L], cw) for the incident waves (each row [E0xyz, kxyz])."""
    L = len(n)
    ri = [complex(n[0], 0.0)] + [complex(n[l], kappa[l - 1]) for l in range(1, L)]
    k_vac = 2 * np.pi / lam
    xs = []
    Pi, Pr, Pt = [], [[] for _ in range(L - 1)], [[] for _ in range(L - 1)]
    for w in np.atleast_2d(waves):
        A, b, s, sz = layer_system(w, ri, z, n[0], k_vac)
        x = np.linalg.solve(A, b)
        xs.append(x)
        Pi.append(w)
        sn = s * n[0]
        for l in range(L - 1):
            r = np.array([x[l * 6 + 3], x[l * 6 + 4], x[l * 6 + 5], sn[0] * k_vac, sn[1] * k_vac, -sz[l] * k_vac])
            t = np.array([x[(l + 1) * 6], x[(l + 1) * 6 + 1], x[(l + 1) * 6 + 2], sn[0] * k_vac, sn[1] * k_vac,
                          sz[l + 1] * k_vac])
            Pr[l].append(so._wind(r[None], z[l])[0])
            Pt[l].append(so._wind(t[None], z[l])[0])
    cw = so.CW(Pi=np.array(Pi, complex), z=list(z[:L - 1]), Pr=[np.array(v, complex) for v in Pr],
               Pt=[np.array(v, complex) for v in Pt])
    return np.array(xs), cw
