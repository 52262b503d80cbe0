"""Mixed-precision rods (CRG_PREC_MIXED) against the FP64 path, through the C ABI.

The vertex/segment pair arithmetic runs in FP32 on hi/lo-split coordinates; which pairs
interact is decided as on the FP64 path; sums are FP32 with Kahan compensation; springs,
curvature, the solver and the state stay FP64.  Tolerances (normwise: max |a - b| over
max |b|):
* interaction force on the same positions, mixed against FP64: <= 1e-6;
* positions after two steps (the first moves the rods with their initial velocity, the
  second with the force): <= 1e-10 (the force error times dt^2 / mass, over the box);
* the pass kernel and the rod-level fallback (pass-list overflow) produce identical bits.
"""
import numpy as np
import pytest

from cellular_raza_gb300 import _native as N
from cellular_raza_gb300 import engine as E
from cellular_raza_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL_FORCE = 1e-6
TOL_TWO_STEPS = 1e-10


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def mixed(w):
    return W.Workload(w.name, w.model.replace(precision="mixed"), w.pos, w.vel, w.n_steps)


def forces(w):
    with E.Simulation.single(w.model, w.n) as sim:
        return sim.forces(w.pos)


@pytest.mark.parametrize("n_sub", [1, 16])
def test_mixed_rod_forces_match_f64(gpu, n_sub):
    w = W.rods_2d(seed=81, n=20_000, n_subdomains=n_sub)
    f64 = forces(w)
    fmx = forces(mixed(w))
    assert np.all(np.isfinite(fmx))
    assert rel(fmx, f64) <= TOL_FORCE


def test_mixed_rod_forces_dense_cutoff_with_force(gpu):
    """Dense rods and a cutoff (5) below twice the radius (6), so the Morse force is
    non-zero at the cutoff: a pair that switched on or off relative to FP64 would show up as
    an error of the size of that force, far above the tolerance."""
    w = W.rods(8000, 240.0, seed=82, n_vertices=5, cutoff=5.0)
    f64 = forces(w)
    fmx = forces(mixed(w))
    assert rel(fmx, f64) <= TOL_FORCE


def test_mixed_rod_forces_3d_far_from_origin(gpu):
    """3D rods in a box at 1e5 from the origin: the hi/lo split keeps the coordinate
    differences exact to FP32 relative precision however large the coordinates."""
    w = W.rods(3000, 200.0, seed=83, n_vertices=4, dim=3, n_subdomains=3)
    shift = 1.0e5
    m = w.model.replace(domain_min=tuple(x + shift for x in w.model.domain_min),
                        domain_max=tuple(x + shift for x in w.model.domain_max))
    ws = W.Workload(w.name, m, w.pos + shift, w.vel, 1)
    f64 = forces(ws)
    fmx = forces(mixed(ws))
    assert rel(fmx, f64) <= TOL_FORCE


def test_mixed_rod_two_steps(gpu):
    w = W.rods_2d(seed=84, n=20_000, n_subdomains=4)
    a = E.run(w, 2)
    b = E.run(mixed(w), 2)
    assert rel(b["pos"], a["pos"]) <= TOL_TWO_STEPS
    assert np.array_equal(a["voxel"], b["voxel"])


def test_mixed_rod_fallback_bitwise(gpu):
    """Pass list too small on every step: every step's forces come from the rod-level mixed
    kernel, which adds the same FP32 terms in the same order as the pass kernel and the
    update's fold: identical bits to the default run."""
    w = mixed(W.rods_2d(seed=85, n=20_000, n_subdomains=4))
    a = E.run(w, 12)
    with E.Simulation.single(w.model, w.n) as sim:
        sim.upload(w.pos, w.vel)
        for _ in range(12):
            sim.set_option(N.OPT_PASS_LIST, 64)
            sim.step(1)
        b = sim.download(order="id")
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])


def test_mixed_rod_passes_without_survivors(gpu):
    """Every pass of the list has zero survivors (the checkerboard of the FP64 test): each
    pass still stores its zero rows (the list starts NaN-filled)."""
    import dataclasses

    gap, length = 6.01, 3.0
    px, py = length + gap, gap
    pts = []
    for i in range(40):
        for j in range(40):
            if (i + j) % 2:
                continue
            x0, y = 5.0 + i * px, 5.0 + j * py
            pts.append([[x0, y], [x0 + length, y]])
    pos = np.array(pts, dtype=np.float64)
    side = 5.0 + 40 * px + 5.0
    r = W.rods(n=len(pts), side=side, seed=0, n_vertices=2, spring_length=length)
    r = dataclasses.replace(r, pos=pos, vel=np.zeros_like(pos))
    a = E.run(r, 3)
    b = E.run(mixed(r), 3)
    assert np.all(np.isfinite(b["pos"]))
    assert np.array_equal(a["pos"], b["pos"])


def test_mixed_rod_batch_equals_single(gpu):
    """Mixed rods packed in a batch: each simulation bit for bit as alone."""
    ws = [mixed(W.rods(n, s, seed=90 + k, n_vertices=6)) for k, (n, s) in
          enumerate([(3000, 400.0), (500, 150.0), (6000, 600.0)])]
    solo = [E.run(x, 20) for x in ws]
    with E.Simulation([x.model for x in ws], [x.n for x in ws]) as sim:
        sim.upload(np.concatenate([x.pos for x in ws]), np.concatenate([x.vel for x in ws]),
                   counts=[x.n for x in ws])
        sim.step(20)
        got = sim.download(order="id")
    off = np.cumsum([0] + [x.n for x in ws])
    for k in range(3):
        assert np.array_equal(got["pos"][off[k]:off[k + 1]], solo[k]["pos"])


def test_mixed_rods_refuse_cell_cycle(gpu):
    w = W.rod_colony(n=50)
    with pytest.raises(N.CrgError) as e:
        E.Simulation.single(w.model.replace(precision="mixed"), 100)
    assert e.value.code == N.CRG_ENOTSUP
