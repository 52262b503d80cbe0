"""Python handle over the request server of libcrg.so (continuous batching of simulations).

    with Server(hbm_budget_bytes=160 << 30, steps_per_tick=32) as srv:
        t = srv.submit(workload, n_steps)
        result = srv.wait(t)          # {"pos", "vel", "ids", "latency_s"}
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional

import numpy as np

from . import _native as N
from .engine import to_c


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Server:
    def __init__(self, hbm_budget_bytes: int = 160 << 30, steps_per_tick: int = 32):
        self._L = N.load()
        h = C.c_void_p()
        N.check(self._L.crg_server_create(int(hbm_budget_bytes), int(steps_per_tick),
                                          C.byref(h)), "crg_server_create")
        self._h = h
        self._shapes: Dict[int, tuple] = {}

    def submit(self, workload, n_steps: Optional[int] = None) -> int:
        d, m = to_c(workload.model)
        pos = np.ascontiguousarray(workload.pos, dtype=np.float64)
        vel = np.ascontiguousarray(workload.vel, dtype=np.float64)
        steps = workload.n_steps if n_steps is None else n_steps
        t = C.c_uint64()
        rc = self._L.crg_server_submit(self._h, C.byref(d), C.byref(m), pos.shape[0], _dp(pos),
                                       _dp(vel), int(steps), C.byref(t))
        N.check(rc, "crg_server_submit")
        self._shapes[t.value] = pos.shape
        return t.value

    def wait(self, ticket: int, timeout_s: float = -1.0) -> Dict[str, np.ndarray]:
        shape = self._shapes.pop(ticket)
        pos, vel = np.empty(shape), np.empty(shape)
        ids = np.empty(shape[0], np.uint64)
        n, lat = C.c_int64(), C.c_double()
        rc = self._L.crg_server_wait(self._h, ticket, float(timeout_s), C.byref(n), _dp(pos),
                                     _dp(vel), ids.ctypes.data_as(C.POINTER(C.c_uint64)),
                                     C.byref(lat))
        if rc == N.CRG_ETIMEDOUT:
            self._shapes[ticket] = shape
        N.check(rc, "crg_server_wait")
        order = np.argsort(ids, kind="stable")
        return {"pos": pos[order], "vel": vel[order], "ids": ids[order],
                "latency_s": lat.value}

    def stats(self) -> Dict[str, int]:
        v = [C.c_int64() for _ in range(5)]
        self._L.crg_server_stats(self._h, *[C.byref(x) for x in v])
        return dict(zip(["queued", "active", "completed", "bytes_in_use", "agent_steps"],
                        [x.value for x in v]))

    def close(self):
        if getattr(self, "_h", None):
            self._L.crg_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
