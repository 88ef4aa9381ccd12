"""The .cw coefficient format and the unpacking of the native library (host-only calls)."""
import os

import numpy as np
import pytest

from oracle import solve_oracle as so
from scwatter_gb300 import _lib
from scwatter_gb300 import cw as cwmod
from scwatter_gb300 import evaluator as ev
from tests._util import solved_case, to_structure


@pytest.fixture(scope="module")
def case():
    return solved_case(shape=(2, 12, 12), coef=(3, 3), seed=3)


def test_save_bytes_equal_oracle_writer(case, tmp_path):
    _, _, _, c = case
    fn = str(tmp_path / "a.cw")
    to_structure(c).save(fn)
    assert open(fn, "rb").read() == so.cw_to_bytes(c)


def test_load_round_trip(case, tmp_path):
    _, _, _, c = case
    fn = str(tmp_path / "a.cw")
    with open(fn, "wb") as f:
        f.write(so.cw_to_bytes(c))
    S = cwmod.CoupledWaveStructure()
    assert S.load(fn)
    assert np.array_equal(S.Pi, c.Pi)
    for l in range(len(c.z)):
        assert S.Layers[l].z == c.z[l]
        assert np.array_equal(S.Layers[l].Pr, c.Pr[l]) and np.array_equal(S.Layers[l].Pt, c.Pt[l])


def test_missing_and_truncated_files(case, tmp_path):
    _, _, _, c = case
    assert cwmod.CoupledWaveStructure().load(str(tmp_path / "missing.cw")) is False
    data = so.cw_to_bytes(c)
    for cut in [4, 12, 100, len(data) // 2, len(data) - 1]:
        fn = str(tmp_path / f"t{cut}.cw")
        with open(fn, "wb") as f:
            f.write(data[:cut])
        with pytest.raises(_lib.ScwError) as ei:
            cwmod.CoupledWaveStructure().load(fn)
        assert ei.value.status == 3
    # a wave count far beyond the file size is a format error, not an allocation attempt
    bad = bytearray(data)
    bad[8:16] = np.uint64(1 << 60).tobytes()
    fn = str(tmp_path / "huge.cw")
    with open(fn, "wb") as f:
        f.write(bad)
    with pytest.raises(_lib.ScwError):
        cwmod.CoupledWaveStructure().load(fn)


def test_allocate_unpack_match_reference_layout(case):
    _, _, _, c = case
    S = to_structure(c)
    ev.cw_allocate(S)
    ev.cw_unpack(S)
    W, b, e, zl = so.unpack(c, np.complex64)
    assert ev.layers == len(c.z)
    assert np.array_equal(ev.W, W)
    assert np.array_equal(ev.waves_begin, b) and np.array_equal(ev.waves_end, e)
    assert np.array_equal(ev.z_layers, zl.astype(np.float32))


def test_get_plane_index(case):
    _, _, _, c = case
    S = to_structure(c)
    z = list(c.z)
    # CoupledWaveStructure.h:141-147: first layer whose z <= query, plus one; else 0
    assert S.getPlaneIndex(z[0] - 1.0) == 0
    assert S.getPlaneIndex(z[0]) == 1
    assert S.getPlaneIndex(z[-1] + 5.0) == 1


def test_empty_structure(tmp_path):
    S = cwmod.CoupledWaveStructure()
    fn = str(tmp_path / "e.cw")
    S.save(fn)
    T = cwmod.CoupledWaveStructure()
    assert T.load(fn) and T.total_waves() == 0 and T.Layers == []
