"""The C-ABI library loads and exports every entry point include/rigc.h
declares (no compute call: this runs without a GPU)."""
import os
import re

from conftest import ROOT


def declared_entry_points():
    src = open(os.path.join(ROOT, "include", "rigc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(rigc_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_entry_points()
    assert "rigc_ctx_create" in names and "rigc_barrier_term" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol():
    import ctypes

    from rigc import _lib as L

    lib = L.load()
    for name in declared_entry_points():
        assert hasattr(lib, name), name
        assert isinstance(getattr(lib, name), ctypes._CFuncPtr)
    assert set(L.EXPORTS) == set(declared_entry_points())


def test_status_strings():
    from rigc import _lib as L

    lib = L.load()
    for code in range(7):
        assert lib.rigc_status_string(code)
