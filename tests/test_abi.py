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


def test_noalloc_limits_are_checked_before_any_device_work():
    """crg_cell_list_noalloc rejects sizes beyond its fixed scratch on the host, before any
    CUDA call (so this runs without a GPU)."""
    from cellular_raza_gb300 import engine, workloads

    lib = _native.load()
    dom, _ = engine.to_c(workloads.spheres(10, 100.0, seed=1).model)
    null = ctypes.c_void_p(0)
    rc = lib.crg_cell_list_noalloc(ctypes.byref(dom), _native.NOALLOC_MAX_POINTS + 1, null, null,
                                   null, null, None)
    assert rc == _native.CRG_EINVAL
    dom, _ = engine.to_c(workloads.spheres(10, 2000.0, seed=1).model)  # 133^3 voxels
    rc = lib.crg_cell_list_noalloc(ctypes.byref(dom), 0, null, null, null, ctypes.c_void_p(8),
                                   None)
    assert rc == _native.CRG_EINVAL


def test_status_strings_without_gpu():
    lib = _native.load()
    assert lib.crg_strerror(_native.CRG_EBOUNDARY).decode().startswith("agent outside")
    assert lib.crg_strerror(12345).decode() == "unknown status"


def test_option_numbers_match_header():
    text = open(os.path.join(ROOT, "include", "crg.h")).read()
    declared = {m.group(1): int(m.group(2))
                for m in re.finditer(r"#define CRG_OPT_([A-Z_]+)\s+(\d+)", text)}
    bound = {k[4:]: v for k, v in vars(_native).items() if k.startswith("OPT_")}
    assert declared == bound


def test_options_need_a_handle():
    lib = _native.load()
    v = ctypes.c_int64(-1)
    assert lib.crg_get_option(None, _native.OPT_TILE, ctypes.byref(v)) == _native.CRG_EINVAL
    assert lib.crg_set_option(None, _native.OPT_TILE, 1) == _native.CRG_EINVAL
    assert v.value == -1


def test_integration_guide_binds_every_symbol():
    """INTEGRATION.md (the Rust host's binding guide) names every function the ABI declares."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    assert [s for s in declared_symbols() if s not in text] == []
