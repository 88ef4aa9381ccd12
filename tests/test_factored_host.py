"""The compact factored coefficient file on the host (scwatter_gb300/factored.py): the
factoring of golden volume-solver .cw structures, the file layout, and the wave lists rebuilt
from the file against the original .cw records (amplitudes at complex64 precision)."""
import os

import numpy as np
import pytest

from oracle import solve_oracle as so
from scwatter_gb300 import factored
from scwatter_gb300.cw import CoupledWaveStructure, HomogeneousLayer

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    c = so.cw_from_bytes(open(os.path.join(GOLDEN, name), "rb").read())
    S = CoupledWaveStructure()
    S.Pi = np.asarray(c.Pi, np.complex128)
    S.Layers = [HomogeneousLayer(z=c.z[l], Pr=np.asarray(c.Pr[l]), Pt=np.asarray(c.Pt[l])) for l in range(len(c.z))]
    return S


def _close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    assert np.all(np.abs(a - b) <= 2e-7 * np.abs(b) + 1e-300)


@pytest.mark.parametrize("name", ["spheres_2x8x8_c3.cw", "oblique_3x10x12_c3x5.cw"])
def test_factor_write_read_rebuild(tmp_path, name):
    S = _load(name)
    fs = factored.factor_cw(S)
    MF, Z = fs.MF, fs.Z
    assert fs.J == 2 * MF and Z == len(S.Layers) - 1
    f = tmp_path / "c.cwf"
    factored.write_cwf(f, fs)
    assert os.path.getsize(f) == factored.file_size(fs.M0, fs.M1, Z, fs.J)
    raw = f.read_bytes()
    assert raw[:8] == b"SCWSEP01"
    assert list(np.frombuffer(raw, "<i4", 6, 8)) == [fs.M0, fs.M1, Z, fs.J, 0, 0]
    g = factored.read_cwf(f)
    factored.write_cwf(tmp_path / "d.cwf", g)
    assert (tmp_path / "d.cwf").read_bytes() == raw
    R = factored.to_cw(g)
    # k vectors and z are exact, amplitudes within complex64 rounding
    assert np.array_equal(R.Pi[:, 3:], S.Pi[:, 3:])
    _close(R.Pi[:, :3], S.Pi[:, :3])
    for L0, L1 in zip(R.Layers, S.Layers):
        assert L0.z == L1.z
        for a, b in ((L0.Pr, L1.Pr), (L0.Pt, L1.Pt)):
            b = np.asarray(b).reshape(-1, 6)
            assert np.array_equal(a[:, 3:], b[:, 3:])
            _close(a[:, :3], b[:, :3])


def test_malformed_inputs(tmp_path):
    S = _load("spheres_2x8x8_c3.cw")
    bad = _load("spheres_2x8x8_c3.cw")
    bad.Layers[1].Pt = bad.Layers[1].Pt[:-1]
    with pytest.raises(ValueError):
        factored.factor_cw(bad)
    f = tmp_path / "c.cwf"
    factored.write_cwf(f, factored.factor_cw(S))
    data = f.read_bytes()
    for blob in (data[:-8], b"SCWSEP02" + data[8:]):
        (tmp_path / "x.cwf").write_bytes(blob)
        with pytest.raises(ValueError):
            factored.read_cwf(tmp_path / "x.cwf")


def test_command_line_round_trip(tmp_path):
    from scwatter_gb300.cw import CoupledWaveStructure as CWS
    src = os.path.join(GOLDEN, "oblique_3x10x12_c3x5.cw")
    f, back = tmp_path / "g.cwf", tmp_path / "g.cw"
    assert factored.main([src, str(f)]) == 0
    assert factored.main([str(f), str(back)]) == 0
    A, B = CWS(), CWS()
    assert A.load(src) and B.load(str(back))
    assert np.array_equal(A.Pi[:, 3:], B.Pi[:, 3:]) and len(A.Layers) == len(B.Layers)
    for L0, L1 in zip(A.Layers, B.Layers):
        assert L0.z == L1.z and L0.Pr.shape == L1.Pr.shape and L0.Pt.shape == L1.Pt.shape
        _close(L1.Pt[:, :3], L0.Pt[:, :3])
    assert factored.main([str(tmp_path / "missing.cw"), str(f)]) == 1


@pytest.mark.parametrize("name", ["spheres_2x8x8_c3.cw", "oblique_3x10x12_c3x5.cw"])
def test_streaming_conversion_matches_in_memory(tmp_path, name):
    a, b = tmp_path / "stream.cwf", tmp_path / "memory.cwf"
    factored.convert_cw_file(os.path.join(GOLDEN, name), a)
    factored.write_cwf(b, factored.factor_cw(_load(name)))
    assert a.read_bytes() == b.read_bytes()
    (tmp_path / "t.cw").write_bytes(open(os.path.join(GOLDEN, name), "rb").read()[:-50])
    with pytest.raises(ValueError):
        factored.convert_cw_file(tmp_path / "t.cw", tmp_path / "t.cwf")


def test_paired_file_read_on_the_host(tmp_path):
    """SCWSEP02 (paired set: beta and one block V per slice) read without a GPU: the two-half
    blocks are Q_dn = V diag(beta_dn), Q_up = diag(1, 1, -1) V diag(beta_up)."""
    import numpy as np
    from scwatter_gb300 import factored
    rng = np.random.default_rng(3)
    M0, M1, Z, J = 3, 2, 2, 12
    MF = M0 * M1
    kx, ky, zb = rng.standard_normal(M0), rng.standard_normal(M1), np.arange(Z + 1.0)
    ext = rng.standard_normal(12 * MF) + 1j * rng.standard_normal(12 * MF)
    kz = rng.standard_normal((Z, 2, J)) + 1j * rng.standard_normal((Z, 2, J))
    beta = rng.standard_normal((Z, 2, J)) + 1j * rng.standard_normal((Z, 2, J))
    V = (rng.standard_normal((Z, 3, MF, J)) + 1j * rng.standard_normal((Z, 3, MF, J))).astype(np.complex64)
    path = tmp_path / "p.cwf"
    with open(path, "wb") as f:
        f.write(b"SCWSEP02")
        f.write(np.array([M0, M1, Z, J, 0, 0], "<i4").tobytes())
        for a in (kx, ky, zb):
            f.write(a.astype("<f8").tobytes())
        for a in (ext, kz, beta):
            f.write(a.astype("<c16").tobytes())
        f.write(V.astype("<c8").tobytes())
    assert path.stat().st_size == factored.file_size(M0, M1, Z, J, paired=True)
    fs = factored.read_cwf(path)
    s = np.array([1.0, 1.0, -1.0])[:, None, None]
    for l in range(Z):
        v = V[l].astype(np.complex128)
        np.testing.assert_allclose(fs.Q[l, 0], (v * beta[l, 0]).astype(np.complex64))
        np.testing.assert_allclose(fs.Q[l, 1], (s * v * beta[l, 1]).astype(np.complex64))
    path.write_bytes(path.read_bytes()[:-8])
    import pytest
    with pytest.raises(ValueError):
        factored.read_cwf(path)
