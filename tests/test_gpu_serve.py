"""Served form: continuous batching of simulation requests.

Each request's result must be the same alone and in the mix (bitwise: every simulation's
arithmetic is independent of its pack neighbours), admission must respect the HBM budget,
and a device error raised by one simulation must fail that request only."""
import ctypes as C
import threading
import time

import numpy as np
import pytest

from cellular_raza_gb300 import _native as N
from cellular_raza_gb300 import engine as E
from cellular_raza_gb300 import serve as SV
from cellular_raza_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def small_stream(seed, n):
    reqs = W.request_stream(seed=seed, n_requests=n, rate_hz=200.0, n_lo=150, n_hi=6000,
                            steps_lo=20, steps_hi=150)
    return reqs


def test_served_results_equal_alone(gpu):
    reqs = small_stream(91, 10)
    out = {}
    with SV.Server(hbm_budget_bytes=8 << 30, steps_per_tick=16) as srv:
        t0 = time.perf_counter()
        tickets = []
        for r in reqs:  # arrivals spread over time: later ones join running packs
            delay = r.arrival_s - reqs[0].arrival_s - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            tickets.append((r, srv.submit(r.workload)))
        for r, t in tickets:
            out[r.rid] = srv.wait(t)
    for r in reqs:
        alone = E.run(r.workload)
        got = out[r.rid]
        assert np.array_equal(got["pos"], alone["pos"]), (r.rid, r.workload.model.precision)
        assert np.array_equal(got["vel"], alone["vel"])
        assert got["latency_s"] > 0


def test_admission_respects_budget(gpu):
    reqs = small_stream(92, 6)
    budget = max(1, int(1.2 * max(
        4 * r.workload.n * r.workload.model.nc * 8 + 400 * r.workload.n for r in reqs)))
    with SV.Server(hbm_budget_bytes=budget, steps_per_tick=8) as srv:
        tickets = [srv.submit(r.workload) for r in reqs]
        peak = 0
        done = 0
        results = {}
        while done < len(reqs):
            st = srv.stats()
            peak = max(peak, st["bytes_in_use"])
            assert st["bytes_in_use"] <= budget
            for t in list(tickets):
                try:
                    results[t] = srv.wait(t, timeout_s=0.01)
                    tickets.remove(t)
                    done += 1
                except N.CrgError as e:
                    assert e.code == N.CRG_ETIMEDOUT
        assert peak > 0
        # finished simulations leave their pack at the next rebuild, which returns their
        # bytes: the server ends at zero
        t0 = time.perf_counter()
        while srv.stats()["bytes_in_use"] and time.perf_counter() - t0 < 5.0:
            time.sleep(0.01)
        assert srv.stats()["bytes_in_use"] == 0
    assert len(results) == len(reqs)


def test_request_needing_more_than_half_the_budget_is_refused(gpu):
    """A pack rebuild holds a class's running simulations twice, so a request larger than
    half the budget could never be admitted: submit refuses it."""
    w = W.spheres(20_000, 340.0, seed=97, dim=3)
    with SV.Server(hbm_budget_bytes=4 << 20, steps_per_tick=8) as srv:
        with pytest.raises(N.CrgError) as e:
            srv.submit(w, 10)
        assert e.value.code == N.CRG_ENOMEM


def test_error_fails_only_its_request(gpu):
    good = W.spheres(800, 120.0, seed=93, dim=3)
    bad = W.spheres(500, 100.0, seed=94, dim=3, dt=1.0, damping=0.0, strength=0.0)
    bad.vel[7, 0, 0] = -1e5  # leaves the domain beyond the reflection in step 1
    with SV.Server(hbm_budget_bytes=4 << 30, steps_per_tick=8) as srv:
        tg = srv.submit(good, 40)
        tb = srv.submit(bad, 40)
        with pytest.raises(N.CrgError) as e:
            srv.wait(tb)
        assert e.value.code == N.CRG_EBOUNDARY
        got = srv.wait(tg)
    alone = E.run(good, 40)
    assert np.array_equal(got["pos"], alone["pos"])


def test_repack_keeps_device_state(gpu):
    """Kept simulations continue exactly as if never moved; new ones start fresh."""
    L = N.load()
    ws = W.ensemble(seed=95, n_sims=4, n_lo=300, n_hi=3000, precision="f64", n_steps=0)
    sim = E.Simulation([w.model for w in ws], [w.n for w in ws])
    sim.upload(np.concatenate([w.pos for w in ws]), np.concatenate([w.vel for w in ws]),
               counts=[w.n for w in ws])
    sim.step(25)
    extra = W.spheres(700, 130.0, seed=96, dim=3)
    d, m = E.to_c(extra.model)
    keep = (C.c_int32 * 2)(3, 1)
    caps = (C.c_int64 * 1)(extra.n)
    pos = np.ascontiguousarray(extra.pos)
    vel = np.ascontiguousarray(extra.vel)
    dp = C.POINTER(C.c_double)
    h = C.c_void_p()
    rc = L.crg_repack(sim._h, 2, keep, 1, C.byref(d), C.byref(m), caps, caps,
                      pos.ctypes.data_as(dp), vel.ctypes.data_as(dp), C.byref(h))
    N.check(rc, "crg_repack")
    sim.close()
    N.check(L.crg_step(h, 25), "crg_step")
    outs = []
    for k, n in enumerate([extra.n, ws[3].n, ws[1].n]):
        p = np.empty((n, 1, 3))
        ids = np.empty(n, np.uint64)
        nn = C.c_int64()
        N.check(L.crg_sim_download(h, k, C.byref(nn), p.ctypes.data_as(dp), None,
                                   ids.ctypes.data_as(C.POINTER(C.c_uint64))), "dl")
        outs.append(p[np.argsort(ids)])
    L.crg_destroy(h)
    assert np.array_equal(outs[0], E.run(extra, 25)["pos"])
    assert np.array_equal(outs[1], E.run(ws[3], 50)["pos"])
    assert np.array_equal(outs[2], E.run(ws[1], 50)["pos"])


def test_served_rods_and_stochastic_equal_alone(gpu):
    """Rod requests (pass-list kernels, their own pack class) and Brownian requests (random
    stream keyed by agent id and step) served while other requests come and go: each result
    equals its run alone."""
    ws = [W.rods(n=600 + 300 * k, side=200.0 + 40 * k, seed=120 + k) for k in range(3)]
    ws += [W.spheres(500 + 400 * k, 100.0 + 20 * k, 130 + k, 3, kind="brownian",
                     diffusion=0.3, kb_temperature=1.0, rng_seed=7 + k) for k in range(3)]
    steps = [40, 25, 60, 30, 45, 20]
    with SV.Server(hbm_budget_bytes=8 << 30, steps_per_tick=8) as srv:
        tickets = []
        for w, n in zip(ws, steps):
            tickets.append(srv.submit(w, n_steps=n))
            time.sleep(0.01)  # later requests join running packs
        out = [srv.wait(t) for t in tickets]
    for w, n, got in zip(ws, steps, out):
        alone = E.run(w, n)
        assert np.array_equal(got["pos"], alone["pos"])
        assert np.array_equal(got["vel"], alone["vel"])
