"""The C-ABI library builds for sm_103a, loads without a GPU and exports every symbol that
include/crg.h declares (no compute calls)."""
import ctypes
import os
import re

from cellular_raza_gb300 import _native, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "crg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(crg_[a-z0-9_]+)\s*\(", text)))


def test_header_matches_binding_list():
    assert declared_symbols() == sorted(_native.EXPORTED)


def test_library_builds_and_exports_every_symbol():
    path = build.build_library()
    lib = ctypes.CDLL(path)
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_status_strings_without_gpu():
    lib = _native.load()
    assert lib.crg_strerror(_native.CRG_EBOUNDARY).decode().startswith("agent outside")
    assert lib.crg_strerror(12345).decode() == "unknown status"
