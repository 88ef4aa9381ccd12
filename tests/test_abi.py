"""The C-ABI library loads and exports every symbol that include/scwatter.h declares."""
import os
import re

from scwatter_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    out = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            src = open(os.path.join(ROOT, "include", name)).read()
            out |= set(re.findall(r"SCW_API\s+[\w\s\*]+?\b(scw_\w+)\s*\(", src))
    return out


def test_every_declared_symbol_is_exported():
    L = _lib.load()
    syms = declared_symbols()
    assert len(syms) > 20
    missing = [s for s in sorted(syms) if not hasattr(L, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    syms = declared_symbols()
    bound = set(_lib.exported_symbols())
    assert syms <= bound, sorted(syms - bound)


def test_errors_without_gpu_work_are_reported():
    import ctypes
    L = _lib.load()
    assert L.scw_cw_create(None) == 1            # SCW_ERR_ARG
    assert b"null" in L.scw_last_error()


def test_command_line_options_mirror_the_reference():
    """sCWatter's option names and defaults (sCWatter.cpp:506-527)."""
    from scwatter_gb300 import scwatter
    a = scwatter.parser().parse_args(["--sample", "x.npy"])
    assert a.lam == 1.0 and a.direction == [0.0, 0.0, 1.0] and a.ex == [0.0, 0.0] and a.ey == [1.0, 0.0]
    assert a.n == [1.0, 1.0] and a.kappa == [0.0] and a.size == [10.0, 10.0, 2.0] and a.output == "c.cw"
    a = scwatter.parser().parse_args(["--sample", "x.npy", "--direction", "0", "-0.5", "1", "--coef", "400", "--npz"])
    assert a.direction == [0.0, -0.5, 1.0] and a.coef == [400] and a.npz


def test_solve_parameter_block():
    from scwatter_gb300 import solver
    p = solver._params(0.5, (0, 0, 1), (1, 0), (0, 0), (0, 0), (1.0, 1.5), [0.02], (8, 8, 2), 0.1, [400], False,
                       True)
    assert list(p.coef) == [20, 20] and p.kappa == 0.02 and p.pz == 1 and p.psf == 0
    import pytest
    with pytest.raises(ValueError):
        solver._params(1, (0, 0, 1), (1, 0), (0, 0), (0, 0), (1.0, 1.2, 1.5), 0, (8, 8, 2), 0, None, False, True)


def test_viewer_options_mirror_the_reference():
    """sCWatterView's option names and defaults (sCWatterView.cpp:682-697)."""
    from scwatter_gb300 import scwatterview
    a = scwatterview.parser().parse_args(["--nogui"])
    assert a.input == "c.cw" and a.cuda == 0 and a.size == 100.0 and a.resolution == 8 and a.output == "xz.npy"
    assert a.axis == 1 and a.center == [0.0, 0.0, 0.0] and a.slice == 0.0
