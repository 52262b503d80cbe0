"""Cell cycle of rods on the GPU (bacterial-rods agent: neighbour-limited growth and division)
against the oracle, in chili's storage order.

Bars: agent identifiers (Division(voxel, counter) included), parents and voxels bit-exact;
positions, velocities, spring lengths and growth rates within 1e-9 relative (norm-wise) --
exp and sqrt round the same on both sides, but exp comes from different libms, so the
trajectories may part in the last bits."""
import numpy as np
import pytest

from cellular_raza_gb300 import _native as N
from cellular_raza_gb300 import engine as E
from cellular_raza_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-9


def rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / den) if den > 0 else float(np.max(np.abs(a)))


def gpu_run(w, steps, capacity=None, options=None):
    return E.run(w, steps, order="list", capacity=capacity, options=options)


def check(got, ref):
    assert got["ids"].shape == ref["ids"].shape
    assert np.array_equal(got["ids"], ref["ids"])
    assert np.array_equal(got["parent"], ref["parent"])
    assert np.array_equal(got["voxel"], ref["voxel"])
    assert rel(got["pos"], ref["pos"]) <= TOL
    assert rel(got["vel"], ref["vel"]) <= TOL
    assert rel(got["spring_length"], ref["spring_length"]) <= TOL
    assert rel(got["growth_rate"], ref["growth_rate"]) <= TOL


@pytest.mark.parametrize("dim,n_sub,order", [(2, 1, 1), (2, 4, 1), (3, 2, 1), (2, 3, 2),
                                             (3, 2, 3)])
def test_colony_matches_oracle(gpu, oracle, dim, n_sub, order):
    w = W.rod_colony(n=150, side=300.0 if dim == 2 else 120.0, seed=3, dim=dim,
                     n_subdomains=n_sub, solver_order=order)
    steps = 200
    ref = oracle.run_cycle(w.model, w.pos, w.vel, steps, spring_length=w.spring_length)
    assert len(ref["ids"]) > w.n  # the run divides
    got = gpu_run(w, steps)
    check(got, ref)


def test_colony_kernel_variants_agree(gpu):
    """The division path behind every rod force kernel: identical bits."""
    w = W.rod_colony(n=150, seed=5, n_subdomains=2)
    a = gpu_run(w, 120)
    for variant in (1, 2, 3):
        b = gpu_run(w, 120, options={N.OPT_KERNEL_VARIANT: variant})
        for k in ("ids", "parent", "pos", "vel", "spring_length"):
            assert np.array_equal(a[k], b[k]), (variant, k)


def test_cycle_without_growth_equals_plain_rods(gpu):
    """Growth 0 and every spring length at the model's: no division, and the rods move
    exactly as without the cycle."""
    w = W.rod_colony(n=150, seed=6, growth_rate=0.0)
    plain = W.Workload(w.name, w.model.replace(cycle=False), w.pos, w.vel, 100)
    cyc = W.Workload(w.name, w.model, w.pos, w.vel, 100)
    a = E.run(plain, 100, order="list")
    b = E.run(cyc, 100, order="list")
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["ids"], b["ids"])
    assert np.all(b["spring_length"] == w.model.spring_length)


@pytest.mark.parametrize("room", [0, 2])
def test_capacity_grows_with_the_colony(gpu, room):
    """A colony on a handle with room for `room` more rods: a step whose divisions do not
    fit grows the handle (state moved through a checkpoint) and is taken again.  The run
    equals one with ample room bit for bit, and the handle keeps its stream."""
    w = W.rod_colony(n=150, seed=3)
    ref = gpu_run(w, 200)
    assert len(ref["ids"]) > w.n + room  # the handle has to grow
    with E.Simulation.single(w.model, w.n + room) as sim:
        stream = sim.stream()
        sim.upload(w.pos, w.vel)
        sim.set_spring_lengths(w.spring_length)
        sim.step(120)
        sim.step(80)
        assert sim.stream() == stream
        assert sim.steps_done == 200
        got = sim.download(order="list")
    for k in ("ids", "parent", "voxel", "pos", "vel", "spring_length", "growth_rate"):
        assert np.array_equal(got[k], ref[k]), k


def test_spring_lengths_only_before_the_first_step(gpu):
    w = W.rod_colony(n=50, seed=3)
    with E.Simulation.single(w.model, 4 * w.n) as sim:
        sim.upload(w.pos, w.vel)
        sim.set_spring_lengths(w.spring_length)
        sim.step(1)
        with pytest.raises(N.CrgError) as e:
            sim.set_spring_lengths(w.spring_length)
        assert e.value.code == N.CRG_EINVAL
        with pytest.raises(N.CrgError):
            sim.snapshot()


def test_autotune_on_a_colony(gpu):
    """The autotuner on a dividing colony: its trials start from a host checkpoint, the
    state is unchanged afterwards, and the run goes on exactly as an untuned one."""
    w = W.rod_colony(n=150, seed=8, n_subdomains=2)
    ref = gpu_run(w, 60)
    with E.Simulation.single(w.model, 16 * w.n) as sim:
        sim.upload(w.pos, w.vel)
        sim.set_spring_lengths(w.spring_length)
        sim.step(30)
        before = sim.download(order="list")
        tune = sim.autotune(5)
        assert tune["ms_per_step"] > 0
        after = sim.download(order="list")
        for k in ("ids", "pos", "vel", "spring_length"):
            assert np.array_equal(before[k], after[k]), k
        assert sim.steps_done == 30
        sim.step(30)
        got = sim.download(order="list")
    for k in ("ids", "parent", "pos", "vel", "spring_length", "growth_rate"):
        assert np.array_equal(got[k], ref[k]), k
