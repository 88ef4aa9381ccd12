"""Sample volumes: the .npy header reader of scw_npy_read (no GPU needed for the shape) and the
oracle restatement of the device Gaussian random field."""
import numpy as np
import pytest

from oracle import sample_oracle as smo


def _lib_or_skip():
    try:
        from scwatter_gb300 import _lib
        _lib.load()
        return _lib
    except OSError as e:                                   # library not built
        pytest.skip(str(e))


@pytest.mark.parametrize("arr,want", [
    (np.zeros((3, 4, 5), np.complex128), (3, 4, 5)),
    (np.zeros((4, 5), np.complex128), (1, 4, 5)),
    (np.zeros((2, 3, 7), np.float64), (2, 3, 7)),
    (np.asfortranarray(np.zeros((4, 6), np.complex128)), (1, 4, 6)),
])
def test_npy_shape_from_header(tmp_path, arr, want):
    _lib_or_skip()
    from scwatter_gb300 import samples
    p = tmp_path / "a.npy"
    np.save(p, arr)
    assert samples.npy_shape(p) == want


def test_npy_header_version_2_and_bad_files(tmp_path):
    _lib = _lib_or_skip()
    from scwatter_gb300 import samples
    p = tmp_path / "v2.npy"
    with open(p, "wb") as f:
        np.lib.format.write_array(f, np.zeros((2, 3, 4), np.complex128), version=(2, 0))
    assert samples.npy_shape(p) == (2, 3, 4)
    bad = tmp_path / "bad.npy"
    bad.write_bytes(b"not an npy file at all")
    with pytest.raises(_lib.ScwError):
        samples.npy_shape(bad)
    np.save(bad, np.zeros((2, 2), np.int32))
    with pytest.raises(_lib.ScwError):
        samples.npy_shape(bad)
    np.save(bad, np.zeros((2, 2, 2, 2), np.complex128))
    with pytest.raises(_lib.ScwError):
        samples.npy_shape(bad)
    with pytest.raises(_lib.ScwError):
        samples.npy_shape(tmp_path / "missing.npy")


def test_grf_oracle_statistics():
    v = smo.grf((8, 32, 32), corr_px=3.0, n_range=(1.0, 1.6), kappa_max=0.02, seed=11)
    assert v.shape == (8, 32, 32)
    assert abs(v.real.min() - 1.0) < 1e-12 and abs(v.real.max() - 1.6) < 1e-12
    assert 0.0 <= v.imag.min() and v.imag.max() <= 0.02
    # smooth: neighbours correlate strongly, the noise itself does not
    g = v.real - v.real.mean()
    c = np.mean(g * np.roll(g, 1, axis=2)) / np.mean(g * g)
    n = smo.noise((8, 32, 32), 11)
    c0 = np.mean(n * np.roll(n, 1, axis=2)) / np.mean(n * n)
    assert c > 0.9 and abs(c0) < 0.05
    assert abs(n.mean()) < 0.05 and abs(n.std() - 1.0) < 0.05
