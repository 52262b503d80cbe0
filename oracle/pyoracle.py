"""ctypes binding of the CPU oracle (oracle/chili_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``.  The product path never
imports this module.

The oracle restates cellular_raza's chili mechanics/interaction step
(cellular_raza-core/src/backend/chili/update_mechanics.rs:65-513, solvers.rs:23-347)
with NewtonDamped / MorsePotential / RodMechanics / RodInteraction
(cellular_raza-building-blocks/src/cell_building_blocks/{mechanics,interaction,
bacterial_rods}.rs) on a CartesianCuboid (domains/cartesian_cuboid_n.rs).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libchili_oracle.so")

KIND_SPHERE = 0
KIND_ROD = 1
KIND_BROWNIAN = 2
KIND_LANGEVIN = 3
KINDS = {"sphere": KIND_SPHERE, "rod": KIND_ROD, "brownian": KIND_BROWNIAN,
         "langevin": KIND_LANGEVIN}

OK, ECALC, EBOUNDARY, EINDEX, EDECOMPOSE, EINVAL = 0, 1, 2, 3, 4, 5


class OrConfig(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("kind", C.c_int32),
        ("n_vertices", C.c_int32),
        ("solver_order", C.c_int32),
        ("n_subdomains", C.c_int32),
        ("voxel_mode", C.c_int32),
        ("min", C.c_double * 3),
        ("max", C.c_double * 3),
        ("interaction_range", C.c_double),
        ("n_voxels", C.c_int64 * 3),
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
    ]


class OrDebug(C.Structure):
    _fields_ = [
        ("force_last", C.POINTER(C.c_double)),
        ("voxel_out", C.POINTER(C.c_uint32)),
        ("n_cand", C.POINTER(C.c_uint32)),
        ("n_inter", C.POINTER(C.c_uint32)),
        ("cand_hash", C.POINTER(C.c_uint64)),
        ("order_out", C.POINTER(C.c_uint64)),
        ("error_agent", C.c_int64),
        ("error_step", C.c_int64),
    ]


_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (three units in parallel)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-C", HERE, "-j3", "-s"], check=True)
    return LIB_PATH


ID_DIVISION = 1 << 63
NO_PARENT = (1 << 64) - 1


class OrCycle(C.Structure):
    _fields_ = [
        ("growth_rate", C.c_double),
        ("division_length", C.c_double),
        ("sense_range", C.c_double),
        ("sense_saturation", C.c_double),
        ("spring_length_in", C.POINTER(C.c_double)),
        ("cap_out", C.c_int64),
        ("n_out", C.c_int64),
        ("ids_out", C.POINTER(C.c_uint64)),
        ("parent_out", C.POINTER(C.c_uint64)),
        ("pos_out", C.POINTER(C.c_double)),
        ("vel_out", C.POINTER(C.c_double)),
        ("spring_length_out", C.POINTER(C.c_double)),
        ("growth_rate_out", C.POINTER(C.c_double)),
        ("voxel_out", C.POINTER(C.c_uint32)),
        ("error_agent", C.c_int64),
        ("error_step", C.c_int64),
    ]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        L.or_run.argtypes = [C.POINTER(OrConfig), C.c_int64, dp, dp, C.c_int64,
                             C.POINTER(OrDebug), dp]
        L.or_run.restype = C.c_int32
        L.or_run_cycle.argtypes = [C.POINTER(OrConfig), C.POINTER(OrCycle), C.c_int64, dp, dp,
                                   C.c_int64]
        L.or_run_cycle.restype = C.c_int32
        L.or_domain_voxels.argtypes = [C.POINTER(OrConfig), C.POINTER(C.c_int64), dp]
        L.or_get_decomp_res.argtypes = [C.c_uint64, C.c_uint64] + [C.POINTER(C.c_uint64)] * 3
        L.or_subdomain_map.argtypes = [C.POINTER(OrConfig), C.POINTER(C.c_uint32)]
        L.or_voxel_neighbors.argtypes = [C.POINTER(OrConfig), C.c_uint64, C.POINTER(C.c_uint64)]
        L.or_initial_voxels.argtypes = [C.POINTER(OrConfig), C.c_int64, dp,
                                        C.POINTER(C.c_uint32)]
        L.or_nearest_point_from_point_to_line.argtypes = [C.c_int32, dp, dp, dp, dp, dp, dp]
        L.or_nearest_point_from_point_to_line.restype = None
        L.or_morse.argtypes = [C.c_int32, dp, dp] + [C.c_double] * 5 + [dp, dp]
        L.or_morse.restype = C.c_int32
        u32p = C.POINTER(C.c_uint32)
        L.or_philox4x32_10.argtypes = [u32p, u32p, u32p]
        L.or_philox4x32_10.restype = None
        L.or_normals.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_int32, dp]
        L.or_normals.restype = None
        for name, n in (("or_euler", 4), ("or_adams_bashforth_2", 5), ("or_adams_bashforth_3", 6)):
            getattr(L, name).argtypes = [C.c_double] * n
            getattr(L, name).restype = C.c_double
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_config(model) -> OrConfig:
    """OrConfig from a cellular_raza_gb300.workloads.Model-like object (duck typed)."""
    c = OrConfig()
    c.dim = model.dim
    c.kind = KINDS[model.kind]
    c.n_vertices = model.n_vertices
    c.solver_order = model.solver_order
    c.n_subdomains = model.n_subdomains
    if model.n_voxels is None:
        c.voxel_mode = 0
        c.interaction_range = model.interaction_range
    else:
        c.voxel_mode = 1
        for i, n in enumerate(model.n_voxels):
            c.n_voxels[i] = int(n)
    for i in range(model.dim):
        c.min[i] = model.domain_min[i]
        c.max[i] = model.domain_max[i]
    c.mass = model.mass
    c.damping = model.damping
    c.spring_tension = model.spring_tension
    c.rigidity = model.rigidity
    c.spring_length = model.spring_length
    c.diffusion = model.diffusion
    c.radius = model.radius
    c.stiffness = model.stiffness
    c.cutoff = model.cutoff
    c.strength = model.strength
    c.dt = model.dt
    c.kb_temperature = getattr(model, "kb_temperature", 0.0)
    c.rng_seed = getattr(model, "rng_seed", 0)
    return c


class OracleError(RuntimeError):
    def __init__(self, code, agent=-1, step=-1):
        super().__init__(f"oracle error code {code} (agent {agent}, step {step})")
        self.code, self.agent, self.step = code, agent, step


def run(model, pos, vel, n_steps, debug=False):
    """Run n_steps chili steps; returns dict with pos, vel (and debug arrays)."""
    L = lib()
    cfg = make_config(model)
    pos = np.ascontiguousarray(pos, dtype=np.float64).copy()
    vel = np.ascontiguousarray(vel, dtype=np.float64).copy()
    n = pos.shape[0]
    out = {}
    dbg = OrDebug()
    dbg.error_agent = -1
    dbg.error_step = -1
    if debug:
        out["force"] = np.zeros_like(pos)
        out["voxel"] = np.zeros(n, np.uint32)
        out["n_cand"] = np.zeros(n, np.uint32)
        out["n_inter"] = np.zeros(n, np.uint32)
        out["cand_hash"] = np.zeros(n, np.uint64)
        out["order"] = np.zeros(n, np.uint64)
        dbg.order_out = out["order"].ctypes.data_as(C.POINTER(C.c_uint64))
        dbg.force_last = _dp(out["force"])
        dbg.voxel_out = out["voxel"].ctypes.data_as(C.POINTER(C.c_uint32))
        dbg.n_cand = out["n_cand"].ctypes.data_as(C.POINTER(C.c_uint32))
        dbg.n_inter = out["n_inter"].ctypes.data_as(C.POINTER(C.c_uint32))
        dbg.cand_hash = out["cand_hash"].ctypes.data_as(C.POINTER(C.c_uint64))
    el = C.c_double(0.0)
    rc = L.or_run(C.byref(cfg), n, _dp(pos), _dp(vel), int(n_steps), C.byref(dbg), C.byref(el))
    if rc != OK:
        raise OracleError(rc, dbg.error_agent, dbg.error_step)
    out["pos"], out["vel"], out["elapsed_s"] = pos, vel, el.value
    return out


def run_cycle(model, pos, vel, n_steps, spring_length=None):
    """Run n_steps chili steps of rods with the bacterial-rods cell cycle (growth limited by
    neighbour sensing, division past model.division_length).  Returns the agents in chili's
    storage order: ids, parent, pos, vel, spring_length, growth_rate, voxel."""
    L = lib()
    cfg = make_config(model)
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    vel = np.ascontiguousarray(vel, dtype=np.float64)
    n = pos.shape[0]
    cy = OrCycle()
    cy.growth_rate = model.growth_rate
    cy.division_length = model.division_length
    cy.sense_range = model.sense_range
    cy.sense_saturation = model.sense_saturation
    sl = None
    if spring_length is not None:
        sl = np.ascontiguousarray(spring_length, dtype=np.float64)
        cy.spring_length_in = _dp(sl)
    cap = max(2 * n, 64)
    while True:
        out = {"ids": np.zeros(cap, np.uint64), "parent": np.zeros(cap, np.uint64),
               "pos": np.zeros((cap,) + pos.shape[1:]), "vel": np.zeros((cap,) + pos.shape[1:]),
               "spring_length": np.zeros(cap), "growth_rate": np.zeros(cap),
               "voxel": np.zeros(cap, np.uint32)}
        cy.cap_out = cap
        cy.ids_out = out["ids"].ctypes.data_as(C.POINTER(C.c_uint64))
        cy.parent_out = out["parent"].ctypes.data_as(C.POINTER(C.c_uint64))
        cy.pos_out = _dp(out["pos"])
        cy.vel_out = _dp(out["vel"])
        cy.spring_length_out = _dp(out["spring_length"])
        cy.growth_rate_out = _dp(out["growth_rate"])
        cy.voxel_out = out["voxel"].ctypes.data_as(C.POINTER(C.c_uint32))
        rc = L.or_run_cycle(C.byref(cfg), C.byref(cy), n, _dp(pos), _dp(vel), int(n_steps))
        if rc == EINVAL and cy.n_out > cap:
            cap = int(cy.n_out)
            continue
        if rc != OK:
            raise OracleError(rc, cy.error_agent, cy.error_step)
        m = int(cy.n_out)
        return {k: v[:m] for k, v in out.items()}


def philox4x32_10(ctr, key):
    """One Philox4x32-10 block (four uint32 words) for counter ctr[4] and key key[2]."""
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().or_philox4x32_10(c, k, o)
    return [int(x) for x in o]


def normals(seed, step, agent_id, n):
    """The n standard normals of the stochastic mechanics for one agent and step."""
    out = np.zeros(n, np.float64)
    lib().or_normals(int(seed), int(step), int(agent_id), int(n), _dp(out))
    return out


def domain_voxels(model):
    cfg = make_config(model)
    nv = (C.c_int64 * 3)()
    dx = (C.c_double * 3)()
    rc = lib().or_domain_voxels(C.byref(cfg), nv, dx)
    if rc != OK:
        raise OracleError(rc)
    return [nv[i] for i in range(model.dim)], [dx[i] for i in range(model.dim)]


def subdomain_map(model):
    nv, _ = domain_voxels(model)
    out = np.zeros(int(np.prod(nv)), np.uint32)
    rc = lib().or_subdomain_map(C.byref(make_config(model)),
                                out.ctypes.data_as(C.POINTER(C.c_uint32)))
    if rc != OK:
        raise OracleError(rc)
    return out


def voxel_neighbors(model, plain):
    out = (C.c_uint64 * 26)()
    k = lib().or_voxel_neighbors(C.byref(make_config(model)), plain, out)
    if k < 0:
        raise OracleError(-k)
    return [out[i] for i in range(k)]


def initial_voxels(model, pos):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    out = np.zeros(pos.shape[0], np.uint32)
    rc = lib().or_initial_voxels(C.byref(make_config(model)), pos.shape[0], _dp(pos),
                                 out.ctypes.data_as(C.POINTER(C.c_uint32)))
    if rc != OK:
        raise OracleError(rc)
    return out


def get_decomp_res(n_voxel, n_regions):
    n, m, a = C.c_uint64(), C.c_uint64(), C.c_uint64()
    rc = lib().or_get_decomp_res(n_voxel, n_regions, C.byref(n), C.byref(m), C.byref(a))
    return None if rc else (n.value, m.value, a.value)


def nearest_point(point, a, b):
    d = len(point)
    p, a, b = (np.ascontiguousarray(x, np.float64) for x in (point, a, b))
    q = np.zeros(d)
    dist, t = C.c_double(), C.c_double()
    lib().or_nearest_point_from_point_to_line(d, _dp(p), _dp(a), _dp(b), C.byref(dist), _dp(q),
                                              C.byref(t))
    return dist.value, q, t.value


def morse(own, ext, own_radius, ext_radius, cutoff, strength, stiffness):
    d = len(own)
    o, e = np.ascontiguousarray(own, np.float64), np.ascontiguousarray(ext, np.float64)
    f1, f2 = np.zeros(d), np.zeros(d)
    lib().or_morse(d, _dp(o), _dp(e), own_radius, ext_radius, cutoff, strength, stiffness,
                   _dp(f1), _dp(f2))
    return f1, f2


def euler(x, dx, dt, dx_rand=0.0):
    return lib().or_euler(x, dx, dt, dx_rand)


def adams_bashforth_2(x, dx0, dx1, dt, dx_rand=0.0):
    return lib().or_adams_bashforth_2(x, dx0, dx1, dt, dx_rand)


def adams_bashforth_3(x, dx0, dx1, dx2, dt, dx_rand=0.0):
    return lib().or_adams_bashforth_3(x, dx0, dx1, dx2, dt, dx_rand)
