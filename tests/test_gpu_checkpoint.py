"""Checkpoint / resume (crg_checkpoint_*): a run split by a host checkpoint, resumed on a
fresh handle, equals the uninterrupted run bit for bit -- cell-list order, solver history,
step counter (and with it the random stream) and per-simulation stop steps included."""
import ctypes as C

import numpy as np
import pytest

from cellular_raza_gb300 import _native as N
from cellular_raza_gb300 import engine as E
from cellular_raza_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def split_run(models, counts, pos, vel, first, second, stops=None):
    def make():
        s = E.Simulation(models, counts)
        return s

    a = make()
    a.upload(pos, vel, counts=counts if len(models) > 1 else None)
    for sim, stop in (stops or {}).items():
        N.check(a._L.crg_set_sim_stop(a._h, C.c_int32(sim), C.c_int64(stop)), "stop")
    a.step(first)
    blob = a.checkpoint()
    a.step(second)
    straight = a.download(order="id")
    a.close()
    b = make()
    b.resume(blob)
    b.step(second)
    resumed = b.download(order="id")
    b.close()
    return straight, resumed


def assert_same(x, y):
    for k in ("pos", "vel", "voxel"):
        assert np.array_equal(x[k], y[k]), k


def test_rods_ab3_resume_bitwise(gpu):
    r = W.rods_2d(seed=71, n=20_000, n_subdomains=16, solver_order=3)
    straight, resumed = split_run([r.model], [r.n], r.pos, r.vel, 30, 40)
    assert_same(straight, resumed)


def test_mixed_batch_with_stop_steps_resume_bitwise(gpu):
    ws = W.ensemble(seed=72, n_sims=4, n_lo=300, n_hi=4000, precision="mixed", n_steps=60)
    straight, resumed = split_run([w.model for w in ws], [w.n for w in ws],
                                  np.concatenate([w.pos for w in ws]),
                                  np.concatenate([w.vel for w in ws]), 25, 35,
                                  stops={1: 40, 3: 10})
    assert_same(straight, resumed)


@pytest.mark.parametrize("dim,order", [(2, 1), (3, 2)])
def test_cell_cycle_resume_bitwise(gpu, dim, order):
    """Growing, dividing rods: spring lengths, growth rates, parents and the voxels'
    division counters travel with the checkpoint, so the resumed colony names its daughters
    and grows exactly as the uninterrupted one."""
    w = W.rod_colony(n=150, side=300.0 if dim == 2 else 120.0, seed=74, dim=dim,
                     n_subdomains=2, solver_order=order)
    cap = 16 * w.n

    def make():
        return E.Simulation.single(w.model, cap)

    a = make()
    a.upload(w.pos, w.vel)
    a.set_spring_lengths(w.spring_length)
    a.step(90)
    blob = a.checkpoint()
    n_at_checkpoint = a.n_agents
    a.step(110)
    straight = a.download(order="list")
    a.close()
    b = make()
    b.resume(blob)
    assert b.n_agents == n_at_checkpoint and b.steps_done == 90
    b.step(110)
    resumed = b.download(order="list")
    b.close()
    assert len(straight["ids"]) > n_at_checkpoint > w.n  # divisions on both sides
    for k in ("ids", "parent", "voxel", "pos", "vel", "spring_length", "growth_rate"):
        assert np.array_equal(straight[k], resumed[k]), k


def test_brownian_stream_continues_after_resume(gpu):
    w = W.spheres(2500, 140.0, 73, 3, kind="brownian", diffusion=0.4, kb_temperature=1.5,
                  rng_seed=5, solver_order=2)
    straight, resumed = split_run([w.model], [w.n], w.pos, w.vel, 17, 23)
    assert_same(straight, resumed)


def test_checkpoint_rejects_other_handles(gpu):
    w = W.spheres_3d(seed=74, n=2000)
    r = W.rods(n=500, side=200.0, seed=75)
    a = E.Simulation([w.model], [w.n])
    a.upload(w.pos, w.vel)
    a.step(3)
    blob = a.checkpoint()
    a.close()
    b = E.Simulation([r.model], [r.n])
    with pytest.raises(N.CrgError):
        b.resume(blob)
    with pytest.raises(N.CrgError):
        b.resume(blob[:100])
    b.close()


def test_checkpoint_rejects_other_parameters_and_damaged_cell_starts(gpu):
    """A blob loads only into a handle with the same domains, models and capacities (a hash of
    every field is in the header), and cell starts that could index outside the arrays are
    refused before anything reaches the device."""
    import math
    import struct

    w = W.spheres_3d(seed=76, n=2000)
    a = E.Simulation([w.model], [w.n])
    a.upload(w.pos, w.vel)
    a.step(3)
    blob = a.checkpoint()
    a.close()
    other = E.Simulation([w.model.replace(dt=0.02)], [w.n])  # same shapes, other dt
    with pytest.raises(N.CrgError) as e:
        other.resume(blob)
    assert e.value.code == N.CRG_EINVAL
    other.close()
    # the cell starts are the blob's last n_vox + 1 uint32 values before the step counter
    m = w.model
    n_vox = math.prod(max(1, math.floor((m.domain_max[k] - m.domain_min[k]) /
                                        m.interaction_range)) for k in range(m.dim))
    at = len(blob) - 8 - 4 * (n_vox + 1)
    bad = bytearray(blob)
    struct.pack_into("<I", bad, at + 4 * 5, 0xFFFFFF00)  # start[5] far past n_agents
    same = E.Simulation([w.model], [w.n])
    with pytest.raises(N.CrgError) as e:
        same.resume(bytes(bad))
    assert e.value.code == N.CRG_EINVAL
    same.resume(blob)  # the intact blob still loads
    same.step(2)
    same.close()
