"""The C-ABI library builds, loads without a GPU, and exports every symbol
that include/seismic_gb300.h declares; host-only entry points work."""
import ctypes as C
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "seismic_gb300.h")


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "st_build", os.path.join(REPO, "03-seismic-tomography-compute_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    path = mod.build()
    from seismic_engine import _lib
    assert os.path.samefile(path, _lib.lib_path())
    return _lib.load()


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(st_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "st_solver_create" in syms and "st_shot_forward" in syms
    assert len(syms) >= 30


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_signatures_cover_header(lib):
    from seismic_engine import _lib
    missing = [s for s in declared_symbols() if s not in _lib.SIGNATURES]
    assert not missing, missing


def test_field_layout_host_only(lib):
    from seismic_engine import field_layout
    L = field_layout(256, 256, 256)
    assert L["NXh"] == 258 and L["NYh"] == 258 and L["ZOFF"] == 4
    assert L["NZP"] % 8 == 0 and L["NZP"] >= 256 + 5
    assert L["plane"] == L["NYh"] * L["NZP"] and L["elems"] == L["NXh"] * L["plane"]
    # TMA: row pitch a multiple of 16 bytes; interior rows start 16-byte aligned
    assert (L["NZP"] * 4) % 16 == 0 and (L["ZOFF"] * 4) % 16 == 0
    for n in (1, 3, 22, 130, 511):
        L = field_layout(n, n + 1, n + 2)
        assert L["NZP"] >= n + 2 + 5


def test_bad_arguments_report_errors(lib):
    from seismic_engine import _lib
    out = (C.c_int64 * 6)()
    rc = lib.st_field_layout(0, 4, 4, out)
    assert rc == _lib.ST_ERR_ARG
    assert b"extent" in lib.st_last_error()
    n = C.c_int(-1)
    assert lib.st_device_count(C.byref(n)) == 0 and n.value >= 0
