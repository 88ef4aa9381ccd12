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
