"""ctypes binding of libcrg.so (the C ABI declared in include/crg.h).

The library is built in-tree by ``cellular_raza_gb300.build.build_library``.  Loading fails
loudly when it is missing: there is no CPU fallback for the device path.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

CRG_OK, CRG_ECALC, CRG_EBOUNDARY, CRG_EINDEX, CRG_EDECOMPOSE = 0, 1, 2, 3, 4
CRG_EINVAL, CRG_ENOMEM, CRG_ECUDA, CRG_ETIMEDOUT, CRG_ENOTSUP = 5, 6, 7, 8, 9
KIND_SPHERE, KIND_ROD, KIND_BROWNIAN, KIND_LANGEVIN = 0, 1, 2, 3
KINDS = {"sphere": KIND_SPHERE, "rod": KIND_ROD, "brownian": KIND_BROWNIAN,
         "langevin": KIND_LANGEVIN}
PREC_F64, PREC_MIXED = 0, 1
WEIGHTS_CHILI, WEIGHTS_PHYSICAL = 0, 1
OPT_PREFILTER, OPT_GRAPH_CHUNK, OPT_BLOCK, OPT_PROFILE, OPT_DEBUG_FORCES = 1, 2, 3, 4, 5
OPT_KERNEL_VARIANT = 6
OPT_PASS_LIST = 7
OPT_TILE = 8
# CellIdentifier::Division(voxel, counter) = ID_DIVISION | voxel << 32 | counter
ID_DIVISION = 1 << 63
NO_PARENT = (1 << 64) - 1

# Every symbol include/crg.h declares (checked by tests/test_abi.py).
EXPORTED = [
    "crg_create", "crg_create_batch", "crg_upload", "crg_step", "crg_forces", "crg_download",
    "crg_agent_count", "crg_last_error", "crg_destroy", "crg_strerror", "crg_set_option",
    "crg_get_option",
    "crg_debug_forces", "crg_debug_neighbor_stats", "crg_profile", "crg_measure_fma_peaks",
    "crg_check_division",
    "crg_snapshot", "crg_get_stream", "crg_cell_list_noalloc", "crg_autotune",
    "crg_set_sim_stop", "crg_sim_download", "crg_clear_error", "crg_repack", "crg_step_count",
    "crg_checkpoint_size", "crg_checkpoint_save", "crg_checkpoint_load",
    "crg_set_spring_lengths", "crg_download_cycle",
    "crg_server_create", "crg_server_submit", "crg_server_wait", "crg_server_stats",
    "crg_server_destroy",
]
NOALLOC_MAX_POINTS = 1 << 20
NOALLOC_MAX_VOXELS = 1 << 20


class CrgDomain(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("voxel_mode", C.c_int32),
        ("min", C.c_double * 3),
        ("max", C.c_double * 3),
        ("interaction_range", C.c_double),
        ("n_voxels", C.c_int64 * 3),
        ("n_subdomains", C.c_int32),
        ("weight_mode", C.c_int32),
    ]


class CrgModel(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("n_vertices", C.c_int32),
        ("solver_order", C.c_int32),
        ("precision", C.c_int32),
        ("mass", C.c_double),
        ("damping", C.c_double),
        ("spring_tension", C.c_double),
        ("rigidity", C.c_double),
        ("spring_length", C.c_double),
        ("diffusion", C.c_double),
        ("radius", C.c_double),
        ("stiffness", C.c_double),
        ("cutoff", C.c_double),
        ("strength", C.c_double),
        ("dt", C.c_double),
        ("kb_temperature", C.c_double),
        ("rng_seed", C.c_uint64),
        ("cycle", C.c_int32),
        ("growth_rate", C.c_double),
        ("division_length", C.c_double),
        ("sense_range", C.c_double),
        ("sense_saturation", C.c_double),
    ]


class CrgError(RuntimeError):
    """A non-zero crg status.  ``code`` is the CRG_E* value."""

    def __init__(self, code: int, what: str = "", agent: int = -1, step: int = -1):
        msg = f"{what}: {strerror(code)} (code {code})"
        if agent >= 0 or step >= 0:
            msg += f" at agent {agent}, step {step}"
        super().__init__(msg)
        self.code, self.agent, self.step = code, agent, step


_lib = None


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load libcrg.so (building it first when it is absent and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"{path} is missing; run cellular_raza_gb300.build.build_library()")
        _build.build_library()
    L = C.CDLL(path)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    u64p = C.POINTER(C.c_uint64)
    u32p = C.POINTER(C.c_uint32)
    i64p = C.POINTER(C.c_int64)
    L.crg_create.argtypes = [C.POINTER(CrgDomain), C.POINTER(CrgModel), C.c_int64, C.POINTER(vp)]
    L.crg_create_batch.argtypes = [C.c_int32, C.POINTER(CrgDomain), C.POINTER(CrgModel), i64p,
                                   C.POINTER(vp)]
    L.crg_upload.argtypes = [vp, C.c_int64, i64p, dp, dp, u64p]
    L.crg_step.argtypes = [vp, C.c_int64]
    L.crg_forces.argtypes = [vp, C.c_int64, dp, dp]
    L.crg_download.argtypes = [vp, dp, dp, u64p, u32p]
    L.crg_agent_count.argtypes = [vp, i64p]
    L.crg_last_error.argtypes = [vp, i64p, i64p]
    L.crg_destroy.argtypes = [vp]
    L.crg_strerror.argtypes = [C.c_int32]
    L.crg_strerror.restype = C.c_char_p
    L.crg_set_option.argtypes = [vp, C.c_int32, C.c_int64]
    L.crg_get_option.argtypes = [vp, C.c_int32, i64p]
    L.crg_debug_forces.argtypes = [vp, dp, u64p]
    L.crg_debug_neighbor_stats.argtypes = [vp, u32p, u32p, u64p, u64p]
    L.crg_profile.argtypes = [vp, dp]
    L.crg_measure_fma_peaks.argtypes = [dp, dp]
    L.crg_check_division.argtypes = [C.c_int64, C.c_uint64, i64p, i64p]
    L.crg_snapshot.argtypes = [vp, C.c_int32]
    L.crg_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.crg_cell_list_noalloc.argtypes = [C.POINTER(CrgDomain), C.c_int64, vp, vp, vp, vp, vp]
    L.crg_autotune.argtypes = [vp, C.c_int64, i64p, i64p, dp]
    L.crg_set_sim_stop.argtypes = [vp, C.c_int32, C.c_int64]
    L.crg_checkpoint_size.argtypes = [vp, C.POINTER(C.c_int64)]
    L.crg_checkpoint_save.argtypes = [vp, C.c_void_p, C.c_int64]
    L.crg_checkpoint_load.argtypes = [vp, C.c_void_p, C.c_int64]
    L.crg_sim_download.argtypes = [vp, C.c_int32, i64p, dp, dp, u64p]
    L.crg_clear_error.argtypes = [vp, C.POINTER(C.c_int32)]
    L.crg_repack.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.c_int32,
                             C.POINTER(CrgDomain), C.POINTER(CrgModel), i64p, i64p, dp, dp,
                             C.POINTER(vp)]
    L.crg_step_count.argtypes = [vp, i64p]
    L.crg_set_spring_lengths.argtypes = [vp, dp]
    L.crg_download_cycle.argtypes = [vp, dp, dp, u64p]
    L.crg_server_create.argtypes = [C.c_int64, C.c_int32, C.POINTER(vp)]
    L.crg_server_submit.argtypes = [vp, C.POINTER(CrgDomain), C.POINTER(CrgModel), C.c_int64,
                                    dp, dp, C.c_int64, u64p]
    L.crg_server_wait.argtypes = [vp, C.c_uint64, C.c_double, i64p, dp, dp, u64p, dp]
    L.crg_server_stats.argtypes = [vp, i64p, i64p, i64p, i64p, i64p]
    L.crg_server_destroy.argtypes = [vp]
    for name in EXPORTED:
        f = getattr(L, name)
        if name != "crg_strerror":
            f.restype = C.c_int32
    _lib = L
    return L


def strerror(code: int) -> str:
    try:
        return load().crg_strerror(code).decode()
    except OSError:
        return f"status {code}"


def check(code: int, what: str, ctx=None):
    if code != CRG_OK:
        agent, step = -1, -1
        if ctx is not None:
            a, s = C.c_int64(-1), C.c_int64(-1)
            load().crg_last_error(ctx, C.byref(a), C.byref(s))
            agent, step = a.value, s.value
        raise CrgError(code, what, agent, step)
