"""Coefficient storage: the streaming .cw writer (CoupledWaveStructure.h:72-100 layout) against
the in-memory structure, and the compact factored coefficient file (.cwf) written and read back
by the separable evaluator and the headless viewer."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from scwatter_gb300 import evaluator as ev
    return ev.Context(0)


def _solve(ctx, external=False):
    from scwatter_gb300 import samples, solver
    vol = samples.spheres((3, 16, 16), n_spheres=2, radius=(2.0, 5.0), seed=5)
    return solver.solve(vol, lam=1.0, direction=(0.2, -0.1, 1.0), ex=(1.0, 0.0), ey=(0.0, 0.0), size=(16.0, 16.0, 3.0),
                        coef=(4, 5), external=external, ctx=ctx)


@pytest.mark.parametrize("external", [False, True])
def test_streaming_cw_writer_is_byte_identical(ctx, tmp_path, external):
    sol = _solve(ctx, external)
    a, b = tmp_path / "stream.cw", tmp_path / "memory.cw"
    sol.save(a)                                   # scw_solution_write_cw
    sol.to_cw().save(b)                           # scw_solution_to_cw + scw_cw_save
    assert a.read_bytes() == b.read_bytes()
    assert os.path.getsize(a) > 0


def test_factored_file_round_trip(ctx, tmp_path):
    from scwatter_gb300 import separable as sp
    sol = _solve(ctx)
    s1 = sol.to_sep()
    f = tmp_path / "c.cwf"
    s1.save(f)
    s2 = sp.SeparableSet.load(ctx, f)
    assert s1.info() == s2.info()
    # a solve gives a paired set (SCWSEP02): kz and beta [Z][2][Jp] complex128, one block V
    # [Z][3][MF][Jp] complex64 -- half the amplitude bytes of the two-block file
    assert s1.form() == 1 and s2.form() == 1
    assert f.read_bytes()[:8] == b"SCWSEP02"
    MF, Z = 20, 3
    J = 2 * MF
    Jp = J + (J & 1)
    want = 8 + 24 + 8 * (4 + 5 + Z + 1) + 16 * 12 * MF + 2 * 16 * Z * 2 * Jp + 8 * Z * 3 * MF * Jp
    assert os.path.getsize(f) == want
    for method in (sp.FP32, sp.TF32X3):
        e1 = s1.evaluate_planes_host(-8.0, -8.0, -3.0, 0.5, -0.25, 0.75, 0.5, 32, method=method)
        e2 = s2.evaluate_planes_host(-8.0, -8.0, -3.0, 0.5, -0.25, 0.75, 0.5, 32, method=method)
        for a, b in zip(e1, e2):
            assert np.array_equal(a, b)


def test_factored_file_from_cw_and_errors(ctx, tmp_path):
    from scwatter_gb300 import _lib
    from scwatter_gb300 import separable as sp
    from scwatter_gb300.cw import CoupledWaveStructure
    golden = os.path.join(os.path.dirname(__file__), "golden", "oblique_3x10x12_c3x5.cw")
    S = CoupledWaveStructure()
    assert S.load(golden)
    s1 = sp.SeparableSet.from_cw(ctx, S)
    f = tmp_path / "g.cwf"
    s1.save(f)
    s2 = sp.SeparableSet.load(ctx, f)
    e1 = s1.evaluate_planes_host(-4.0, -4.0, -2.0, 0.0, 0.0, 0.0, 0.4, 20)
    e2 = s2.evaluate_planes_host(-4.0, -4.0, -2.0, 0.0, 0.0, 0.0, 0.4, 20)
    assert all(np.array_equal(a, b) for a, b in zip(e1, e2))
    data = f.read_bytes()
    bad = tmp_path / "bad.cwf"
    for blob in (data[:-8], b"SCWSEP99" + data[8:], b"SCWSEP02" + data[8:], data[:20]):
        bad.write_bytes(blob)
        with pytest.raises(_lib.ScwError):
            sp.SeparableSet.load(ctx, bad)
    with pytest.raises(_lib.ScwError):
        sp.SeparableSet.load(ctx, tmp_path / "missing.cwf")


def test_cli_factored_output_drives_the_viewer(tmp_path):
    from scwatter_gb300 import samples, scwatter, scwatterview
    vol = samples.spheres((2, 12, 12), n_spheres=2, radius=(2.0, 4.0), seed=9)
    npy = tmp_path / "s.npy"
    np.save(npy, vol)
    cw, cwf = tmp_path / "c.cw", tmp_path / "c.cwf"
    assert scwatter.main(["--sample", str(npy), "--coef", "4", "4", "--size", "12", "12", "2", "--output", str(cw),
                          "--factored", str(cwf)]) == 0
    outs = []
    for src in (cw, cwf):
        o = tmp_path / (src.name + ".npy")
        assert scwatterview.main([str(src), "--nogui", "--resolution", "4", "--size", "10", "--axis", "1",
                                  "--method", "tf32x3", "--output", str(o)]) == 0
        outs.append(np.load(o))
    assert np.abs(outs[0] - outs[1]).max() <= 1e-5 * np.abs(outs[0]).max()
    assert scwatterview.main([str(cwf), "--nogui", "--method", "plain", "--output", str(tmp_path / "x.npy")]) == 2
