"""Python handle over the C ABI: one simulation or a batch of simulations on the GPU.

This is a thin owner of a ``crg_ctx*``; every call goes through libcrg.so.
"""
from __future__ import annotations

import ctypes as C
import struct
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _native as N
from .workloads import Model


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def to_c(model: Model):
    d = N.CrgDomain()
    d.dim = model.dim
    if model.n_voxels is None:
        d.voxel_mode = 0
        d.interaction_range = float(model.interaction_range)
    else:
        d.voxel_mode = 1
        for i, n in enumerate(model.n_voxels):
            d.n_voxels[i] = int(n)
    for i in range(model.dim):
        d.min[i] = float(model.domain_min[i])
        d.max[i] = float(model.domain_max[i])
    d.n_subdomains = int(model.n_subdomains)
    d.weight_mode = int(model.weight_mode)
    m = N.CrgModel()
    m.kind = N.KINDS[model.kind]
    m.n_vertices = int(model.n_vertices)
    m.solver_order = int(model.solver_order)
    m.precision = N.PREC_MIXED if model.precision == "mixed" else N.PREC_F64
    for f in ("mass", "damping", "spring_tension", "rigidity", "spring_length", "diffusion",
              "radius", "stiffness", "cutoff", "strength", "dt", "kb_temperature"):
        setattr(m, f, float(getattr(model, f)))
    m.rng_seed = int(model.rng_seed)
    m.cycle = 1 if getattr(model, "cycle", False) else 0
    for f in ("growth_rate", "division_length", "sense_range", "sense_saturation"):
        setattr(m, f, float(getattr(model, f, 0.0)))
    return d, m


class Simulation:
    """A crg handle holding one or more simulations advanced by the same launches."""

    def __init__(self, models: Sequence[Model], capacities: Sequence[int]):
        self._L = N.load()
        self.models = list(models)
        self.nc = self.models[0].nc
        self.dim = self.models[0].dim
        self.nv = self.models[0].n_vertices
        n = len(self.models)
        doms = (N.CrgDomain * n)()
        mods = (N.CrgModel * n)()
        for s, mdl in enumerate(self.models):
            doms[s], mods[s] = to_c(mdl)
        caps = (C.c_int64 * n)(*[int(c) for c in capacities])
        h = C.c_void_p()
        if n == 1:
            rc = self._L.crg_create(C.byref(doms[0]), C.byref(mods[0]), caps[0], C.byref(h))
        else:
            rc = self._L.crg_create_batch(n, doms, mods, caps, C.byref(h))
        N.check(rc, "crg_create")
        self._h = h
        self.counts: List[int] = [0] * n

    @classmethod
    def single(cls, model: Model, capacity: int) -> "Simulation":
        return cls([model], [capacity])

    # ------------------------------------------------------------------ lifecycle
    def close(self):
        if getattr(self, "_h", None):
            self._L.crg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------ data movement
    def upload(self, pos: np.ndarray, vel: np.ndarray, counts: Optional[Sequence[int]] = None,
               ids: Optional[np.ndarray] = None):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        n = pos.shape[0]
        if pos.size != n * self.nc or vel.shape != pos.shape:
            raise ValueError("pos/vel must have shape [n][n_vertices][dim]")
        cnt = None
        if len(self.models) > 1:
            if counts is None:
                raise ValueError("a batch upload needs per-simulation counts")
            cnt = (C.c_int64 * len(self.models))(*[int(c) for c in counts])
            self.counts = [int(c) for c in counts]
        else:
            self.counts = [n]
        idp = None
        if ids is not None:
            ids = np.ascontiguousarray(ids, dtype=np.uint64)
            idp = ids.ctypes.data_as(C.POINTER(C.c_uint64))
        rc = self._L.crg_upload(self._h, n, cnt, _dp(pos), _dp(vel), idp)
        N.check(rc, "crg_upload", self._h)

    def step(self, n_steps: int = 1):
        rc = self._L.crg_step(self._h, int(n_steps))
        N.check(rc, "crg_step", self._h)

    def forces(self, pos: np.ndarray) -> np.ndarray:
        """Interaction force of every agent of `pos` ([n][n_vertices][dim], each voxel's agents
        in chili's Vec order) as chili's step 1-3 accumulate it (crg_forces); the handle's
        agents become these with zero velocity."""
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        n = pos.shape[0]
        if pos.size != n * self.nc:
            raise ValueError("pos must have shape [n][n_vertices][dim]")
        out = np.empty_like(pos)
        N.check(self._L.crg_forces(self._h, n, _dp(pos), _dp(out)), "crg_forces", self._h)
        self.counts = [n]
        return out

    @property
    def steps_done(self) -> int:
        """Steps the handle's state has advanced since the last upload (crg_step_count)."""
        n = C.c_int64()
        N.check(self._L.crg_step_count(self._h, C.byref(n)), "crg_step_count")
        return n.value

    def clear_error(self):
        """Clears the handle's error (crg_clear_error); returns (code, simulation)."""
        sim = C.c_int32(-1)
        code = self._L.crg_clear_error(self._h, C.byref(sim))
        return code, sim.value

    @property
    def n_agents(self) -> int:
        n = C.c_int64()
        self._L.crg_agent_count(self._h, C.byref(n))
        return n.value

    def set_spring_lengths(self, spring_length: np.ndarray):
        """Cell cycle: per-rod spring lengths in the order of the last upload (before the
        first step)."""
        sl = np.ascontiguousarray(spring_length, dtype=np.float64)
        if sl.shape != (self.n_agents,):
            raise ValueError("one spring length per uploaded rod")
        N.check(self._L.crg_set_spring_lengths(self._h, _dp(sl)), "crg_set_spring_lengths",
                self._h)

    def download(self, order: str = "list") -> Dict[str, np.ndarray]:
        """Current state.  order="list": cell-list order; "id": per simulation sorted by id
        (ids 0..n-1 when upload was given no ids).  Cell-cycle handles add spring_length,
        growth_rate and parent."""
        n = self.n_agents
        if len(self.models) == 1:
            self.counts = [n]  # divisions change the count
        shape = (n, self.nv, self.dim)
        pos = np.empty(shape)
        vel = np.empty(shape)
        ids = np.empty(n, np.uint64)
        vox = np.empty(n, np.uint32)
        rc = self._L.crg_download(self._h, _dp(pos), _dp(vel),
                                  ids.ctypes.data_as(C.POINTER(C.c_uint64)),
                                  vox.ctypes.data_as(C.POINTER(C.c_uint32)))
        N.check(rc, "crg_download", self._h)
        out = {"pos": pos, "vel": vel, "ids": ids, "voxel": vox}
        if getattr(self.models[0], "cycle", False):
            out["spring_length"] = np.empty(n)
            out["growth_rate"] = np.empty(n)
            out["parent"] = np.empty(n, np.uint64)
            rc = self._L.crg_download_cycle(self._h, _dp(out["spring_length"]),
                                            _dp(out["growth_rate"]),
                                            out["parent"].ctypes.data_as(C.POINTER(C.c_uint64)))
            N.check(rc, "crg_download_cycle", self._h)
        if order == "id":
            out = self._by_id(out)
        return out

    def _by_id(self, out):
        # simulations occupy consecutive ranges of the cell list
        res = {k: np.empty_like(v) for k, v in out.items()}
        off = 0
        for c in self.counts:
            sl = slice(off, off + c)
            perm = np.argsort(out["ids"][sl], kind="stable")
            for k, v in out.items():
                res[k][sl] = v[sl][perm]
            off += c
        return res

    # ------------------------------------------------------------------ options / diagnostics
    def set_option(self, opt: int, value: int):
        N.check(self._L.crg_set_option(self._h, int(opt), int(value)), "crg_set_option")

    def get_option(self, opt: int) -> int:
        v = C.c_int64()
        N.check(self._L.crg_get_option(self._h, int(opt), C.byref(v)), "crg_get_option")
        return v.value

    def debug_forces(self) -> Dict[str, np.ndarray]:
        n = self.n_agents
        f = np.empty((n, self.nv, self.dim))
        ids = np.empty(n, np.uint64)
        rc = self._L.crg_debug_forces(self._h, _dp(f), ids.ctypes.data_as(C.POINTER(C.c_uint64)))
        N.check(rc, "crg_debug_forces")
        return {"force": f, "ids": ids}

    def neighbor_stats(self) -> Dict[str, np.ndarray]:
        n = self.n_agents
        nc = np.empty(n, np.uint32)
        ni = np.empty(n, np.uint32)
        h = np.empty(n, np.uint64)
        ids = np.empty(n, np.uint64)
        u32 = C.POINTER(C.c_uint32)
        u64 = C.POINTER(C.c_uint64)
        rc = self._L.crg_debug_neighbor_stats(self._h, nc.ctypes.data_as(u32),
                                              ni.ctypes.data_as(u32), h.ctypes.data_as(u64),
                                              ids.ctypes.data_as(u64))
        N.check(rc, "crg_debug_neighbor_stats")
        return {"n_cand": nc, "n_inter": ni, "cand_hash": h, "ids": ids}

    def snapshot(self, restore: bool = False):
        N.check(self._L.crg_snapshot(self._h, 1 if restore else 0), "crg_snapshot")

    def checkpoint(self) -> bytes:
        """The handle's whole simulation state as bytes (crg_checkpoint_save)."""
        n = C.c_int64()
        N.check(self._L.crg_checkpoint_size(self._h, C.byref(n)), "crg_checkpoint_size")
        buf = C.create_string_buffer(n.value)
        N.check(self._L.crg_checkpoint_save(self._h, buf, n.value), "crg_checkpoint_save", self._h)
        return buf.raw

    def resume(self, blob: bytes):
        """Restore a checkpoint taken from a handle with the same domains, models and
        capacities (crg_checkpoint_load); stepping continues bit for bit."""
        buf = C.create_string_buffer(blob, len(blob))
        N.check(self._L.crg_checkpoint_load(self._h, buf, len(blob)), "crg_checkpoint_load")
        # per-simulation agent ranges: the uint32 offsets after the 56-byte header
        n = len(self.models)
        off = struct.unpack_from(f"<{n + 1}I", blob, 56)
        self.counts = [off[s + 1] - off[s] for s in range(n)]

    def save_point(self, location: str, iteration: int, aux=None) -> List[str]:
        """Write the handle's state as a save point in chili's SerdeJson layout
        (``storage.export_cells``; single-simulation handles); returns the files written.
        ``engine.resume_save_point`` reads it back."""
        from . import storage as ST

        if len(self.models) != 1:
            raise ValueError("save points are written per simulation: single handles only")
        return ST.export_cells(location, iteration, self.models[0],
                               self.download(order="list"), aux)

    def stream(self) -> int:
        s = C.c_void_p()
        N.check(self._L.crg_get_stream(self._h, C.byref(s)), "crg_get_stream")
        return s.value or 0

    def autotune(self, steps: int = 5) -> Dict[str, float]:
        """Times every force-kernel shape on the current state and keeps the fastest."""
        v, b, ms = C.c_int64(), C.c_int64(), C.c_double()
        rc = self._L.crg_autotune(self._h, int(steps), C.byref(v), C.byref(b), C.byref(ms))
        N.check(rc, "crg_autotune", self._h)
        return {"variant": v.value, "block": b.value, "tile": self.get_option(N.OPT_TILE),
                "ms_per_step": ms.value}

    def profile(self):
        out = (C.c_double * 5)()
        N.check(self._L.crg_profile(self._h, out), "crg_profile")
        return {"force_ms": out[0], "sort_ms": out[1], "kernels": int(out[2]),
                "kernel_ms": out[3], "update_ms": out[4]}


def measure_fma_peaks():
    """Measured FP64 / FP32 FMA throughput (TFLOP/s) of the current GPU."""
    L = N.load()
    a, b = C.c_double(), C.c_double()
    N.check(L.crg_measure_fma_peaks(C.byref(a), C.byref(b)), "crg_measure_fma_peaks")
    return {"fp64_tflops": a.value, "fp32_tflops": b.value}


def resume_save_point(location: str, iteration: int, model: Model,
                      capacity: Optional[int] = None) -> "Simulation":
    """A handle holding the agents of a SerdeJson save point (written by
    ``storage.export_cells``, or by chili's own ``save_cells`` for agents in the same
    layout): positions, velocities and identifiers uploaded in the save point's storage
    order, which makes the handle's cell list the saved one; with the cell cycle also the
    spring lengths.  Solver history and the step counter are not part of a save point: an
    AB2 / AB3 solver restarts with its first step and a stochastic stream from step 0.
    ``capacity`` defaults to the agent count (16 times it with the cell cycle)."""
    from . import storage as ST

    recs = ST.load_cells(location, iteration)
    st = ST.state_from_records(recs, model.kind, model.dim)
    n = len(recs)
    cycle = getattr(model, "cycle", False)
    if capacity is None:
        capacity = 16 * n if cycle else n
    sim = Simulation.single(model, max(int(capacity), 1))
    try:
        sim.upload(st["pos"], st["vel"], ids=st["ids"])
        if cycle:
            sim.set_spring_lengths(st["spring_length"])
    except Exception:
        sim.close()
        raise
    return sim


def run(workload, n_steps: Optional[int] = None, options: Optional[Dict[int, int]] = None,
        order: str = "id", capacity: Optional[int] = None) -> Dict[str, np.ndarray]:
    """Upload a workload, run it and return the final state (ordered by id by default).
    ``options`` maps CRG_OPT_* values to settings.  A cell-cycle workload gets room for 16
    times its agents unless ``capacity`` says otherwise."""
    steps = workload.n_steps if n_steps is None else n_steps
    cycle = getattr(workload.model, "cycle", False)
    if capacity is None:
        capacity = 16 * workload.n if cycle else workload.n
    with Simulation.single(workload.model, capacity) as sim:
        for k, v in (options or {}).items():
            sim.set_option(k, v)
        sim.upload(workload.pos, workload.vel)
        if cycle and getattr(workload, "spring_length", None) is not None:
            sim.set_spring_lengths(workload.spring_length)
        sim.step(steps)
        return sim.download(order=order)
