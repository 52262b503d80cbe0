"""Error semantics and the forces-only entry point, through the C ABI, against the oracle.

* A BoundaryError stops a simulation as chili stops it: the failing step is not committed
  and later steps leave the simulation unchanged, so a single-simulation handle holds the
  state after its last good step, bit for bit the oracle's state after that many steps.
  In a batch the other simulations run on unaffected.
* crg_forces returns the interaction force chili accumulates in steps 1-3, in the caller's
  order: norm-wise relative error <= 1e-12 against the oracle's accumulated force.
"""
import numpy as np
import pytest

from cellular_raza_gb300 import _native as N
from cellular_raza_gb300 import engine as E
from cellular_raza_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / den) if den > 0 else float(np.max(np.abs(a)))


def colliding_pair(seed=0):
    """Two spheres that meet at step 2 (dt 1, no damping, Morse strength 2): the repulsion
    they get there (~1,500) carries sphere 1 past twice the box at step 3, a BoundaryError,
    while sphere 0 still reflects back inside.  Eight more spheres sit far apart at rest."""
    w = W.spheres(10, 1000.0, seed=seed, dim=3, dt=1.0, damping=0.0, strength=2.0)
    pos = np.zeros((10, 1, 3))
    vel = np.zeros((10, 1, 3))
    pos[0, 0] = (800.0, 500.0, 500.0)
    vel[0, 0] = (18.59, 0.0, 0.0)
    pos[1, 0] = (820.0, 500.0, 500.0)
    for k in range(8):
        pos[2 + k, 0] = (100.0 + 100.0 * k, 150.0 + 80.0 * (k % 3), 700.0 - 60.0 * (k % 4))
    return W.Workload("colliding_pair", w.model, pos, vel, 64)


def test_oracle_reports_the_planted_error(oracle):
    w = colliding_pair()
    oracle.run(w.model, w.pos, w.vel, 2)  # two good steps
    with pytest.raises(oracle.OracleError) as e:
        oracle.run(w.model, w.pos, w.vel, 3)
    assert e.value.code == oracle.EBOUNDARY and e.value.agent == 1 and e.value.step == 3


def test_boundary_error_freezes_at_last_good_step(gpu, oracle):
    """A 64-step graphed call whose error is at step 3: the error names agent 1 and step 3,
    and the handle holds the state after step 2, equal to the oracle's."""
    w = colliding_pair()
    ref = oracle.run(w.model, w.pos, w.vel, 2, debug=True)
    with E.Simulation.single(w.model, w.n) as sim:
        sim.set_option(N.OPT_GRAPH_CHUNK, 32)
        sim.upload(w.pos, w.vel)
        with pytest.raises(N.CrgError) as e:
            sim.step(64)
        assert e.value.code == N.CRG_EBOUNDARY and e.value.agent == 1 and e.value.step == 3
        assert sim.steps_done == 2
        got = sim.download(order="id")
        assert rel(got["pos"], ref["pos"]) <= TOL and rel(got["vel"], ref["vel"]) <= TOL
        assert np.array_equal(got["voxel"], ref["voxel"])
        lst = sim.download(order="list")
        assert np.array_equal(lst["ids"], ref["order"])
        # the handle refuses to step on until the error is cleared
        with pytest.raises(N.CrgError):
            sim.step(1)
        code, s = sim.clear_error()
        assert code == N.CRG_EBOUNDARY and s == 0
        again = sim.download(order="id")
        assert np.array_equal(again["pos"], got["pos"])


def test_boundary_error_in_batch_member(gpu, oracle):
    """Simulation 1 of a batch of three fails at step 3 of a 64-step call: it keeps its state
    after step 2 while simulations 0 and 2 run all 64 steps, bit for bit as alone."""
    a = W.spheres(400, 120.0, seed=3, dim=3)
    b = colliding_pair()
    c = W.spheres(300, 100.0, seed=4, dim=3)
    ws = [a, b, c]
    solo = [E.run(x, 64) for x in (a, c)]
    ref_b = oracle.run(b.model, b.pos, b.vel, 2)
    with E.Simulation([x.model for x in ws], [x.n for x in ws]) as sim:
        sim.upload(np.concatenate([x.pos for x in ws]), np.concatenate([x.vel for x in ws]),
                   counts=[x.n for x in ws])
        with pytest.raises(N.CrgError) as e:
            sim.step(64)
        assert e.value.code == N.CRG_EBOUNDARY and e.value.step == 3
        code, s = sim.clear_error()
        assert code == N.CRG_EBOUNDARY and s == 1
        got = sim.download(order="id")
    off = np.cumsum([0] + [x.n for x in ws])
    assert np.array_equal(got["pos"][off[0]:off[1]], solo[0]["pos"])
    assert np.array_equal(got["pos"][off[2]:off[3]], solo[1]["pos"])
    assert rel(got["pos"][off[1]:off[2]], ref_b["pos"]) <= TOL


def forces_ref(oracle, w):
    return oracle.run(w.model, w.pos, np.zeros_like(w.vel), 1, debug=True)["force"]


@pytest.mark.parametrize("n_sub", [1, 16])
def test_forces_spheres(gpu, oracle, n_sub):
    w = W.spheres_3d(seed=71, n_subdomains=n_sub)
    with E.Simulation.single(w.model, w.n) as sim:
        f = sim.forces(w.pos)
    assert rel(f, forces_ref(oracle, w)) <= TOL


@pytest.mark.parametrize("n_sub", [1, 16])
def test_forces_rods(gpu, oracle, n_sub):
    w = W.rods_2d(seed=72, n=20_000, n_subdomains=n_sub)
    with E.Simulation.single(w.model, w.n) as sim:
        f = sim.forces(w.pos)
    assert rel(f, forces_ref(oracle, w)) <= TOL


def test_forces_rods_3d_and_caller_order(gpu, oracle):
    """Forces come back in the caller's order: a permuted input gives the permuted forces of
    the oracle run on the same permuted input (the order inside a voxel fixes the sums)."""
    w = W.rods(3000, 300.0, seed=73, n_vertices=4, dim=3, n_subdomains=3)
    perm = np.random.Generator(np.random.PCG64(5)).permutation(w.n)
    wp = W.Workload(w.name, w.model, w.pos[perm], w.vel[perm], 1)
    with E.Simulation.single(w.model, w.n) as sim:
        f = sim.forces(wp.pos)
    assert rel(f, forces_ref(oracle, wp)) <= TOL


def test_forces_then_step_matches_upload(gpu):
    """crg_forces leaves the handle holding the agents with zero velocity: stepping on from
    there equals uploading them with zero velocity, bit for bit."""
    w = W.rods_2d(seed=74, n=5000, n_subdomains=2)
    zero = np.zeros_like(w.vel)
    with E.Simulation.single(w.model, w.n) as sim:
        sim.forces(w.pos)
        sim.step(5)
        a = sim.download(order="id")
    b = E.run(W.Workload(w.name, w.model, w.pos, zero, 5), 5)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])


def test_forces_rejects_batches(gpu):
    ws = W.ensemble(seed=1, n_sims=2, n_lo=100, n_hi=200, precision="f64", n_steps=1)
    with E.Simulation([x.model for x in ws], [x.n for x in ws]) as sim:
        with pytest.raises(N.CrgError) as e:
            sim.forces(ws[0].pos)
        assert e.value.code == N.CRG_ENOTSUP
