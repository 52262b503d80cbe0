"""Parity of the CUDA path (through the C ABI) with the oracle on the same seeded inputs.

Bars (written in each test):
  * voxel keys, candidate-partner sets and interacting-pair counts: bit-exact;
  * FP64 interaction forces and one-step positions/velocities: norm-wise relative error
    <= 1e-12 (max_i |x_gpu - x_ref| / max_i |x_ref|);
  * multi-step FP64 trajectories: stated per test.
"""
import dataclasses

import numpy as np
import pytest

from cellular_raza_gb300 import _native as N
from cellular_raza_gb300 import engine as E
from cellular_raza_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-12


def rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / den) if den > 0 else float(np.max(np.abs(a)))


def by_id(arr, ids):
    out = np.empty_like(arr)
    out[ids.astype(np.int64)] = arr
    return out


def gpu_one_step(gpu, w):
    sim = E.Simulation.single(w.model, w.n)
    sim.set_option(N.OPT_DEBUG_FORCES, 1)
    sim.upload(w.pos, w.vel)
    st0 = sim.download(order="id")
    stats = sim.neighbor_stats()
    sim.step(1)
    f = sim.debug_forces()
    lst = sim.download(order="list")
    st1 = sim.download(order="id")
    sim.close()
    st1["list_ids"] = lst["ids"]
    st1["list_voxel"] = lst["voxel"]
    return st0, stats, by_id(f["force"], f["ids"]), st1


def check_one_step(gpu, oracle, w):
    ref = oracle.run(w.model, w.pos, w.vel, 1, debug=True)
    init_vox = oracle.initial_voxels(w.model, w.pos)
    st0, stats, force, st1 = gpu_one_step(gpu, w)
    # insertion and re-sort keys: bit-exact
    assert np.array_equal(st0["voxel"], init_vox)
    assert np.array_equal(st1["voxel"], ref["voxel"])
    # cell list: sorted by voxel, and inside each voxel chili's Vec order (stayers, then
    # movers of the same subdomain, then movers of other subdomains, each by source order)
    assert np.all(np.diff(st1["list_voxel"].astype(np.int64)) >= 0)
    assert np.array_equal(st1["list_ids"], ref["order"])
    # neighbour sets visited in the step: bit-exact
    ids = stats["ids"].astype(np.int64)
    assert np.array_equal(by_id(stats["n_cand"], ids), ref["n_cand"])
    assert np.array_equal(by_id(stats["cand_hash"], ids), ref["cand_hash"])
    assert np.array_equal(by_id(stats["n_inter"], ids), ref["n_inter"])
    # forces and state after one step
    assert rel(force, ref["force"]) <= TOL_STEP
    assert rel(st1["pos"], ref["pos"]) <= TOL_STEP
    assert rel(st1["vel"], ref["vel"]) <= TOL_STEP
    return ref, st1


@pytest.mark.parametrize("n_sub", [1, 3, 16])
def test_spheres_3d_one_step(gpu, oracle, n_sub):
    w = W.spheres_3d(seed=11, n_subdomains=n_sub)
    check_one_step(gpu, oracle, w)


def test_spheres_2d_one_step(gpu, oracle):
    w = W.spheres(3000, 600.0, seed=5, dim=2)
    check_one_step(gpu, oracle, w)


def test_spheres_single_subdomain_matches_chili_sum_order(gpu, oracle):
    """With one subdomain the GPU adds the same half-forces in chili's order, so forces agree
    to the last bits except where exp() rounds differently on the two libms."""
    w = W.spheres_3d(seed=12)
    ref = oracle.run(w.model, w.pos, w.vel, 1, debug=True)
    _, _, force, _ = gpu_one_step(gpu, w)
    assert rel(force, ref["force"]) <= 1e-14


@pytest.mark.parametrize("n_sub", [1, 4])
def test_spheres_3d_trajectory(gpu, oracle, n_sub):
    """200 steps of the 4,096-sphere workload: positions within 1e-10 relative (norm-wise)
    and every agent in the same voxel."""
    w = W.spheres_3d(seed=13, n_subdomains=n_sub)
    ref = oracle.run(w.model, w.pos, w.vel, 200, debug=True)
    got = E.run(w, 200)
    assert rel(got["pos"], ref["pos"]) <= 1e-10
    assert rel(got["vel"], ref["vel"]) <= 1e-8
    assert np.array_equal(got["voxel"], ref["voxel"])


def test_prefilter_is_exact(gpu):
    """The FP32 candidate prefilter only skips pairs whose FP64 force is zero: results with
    and without it are bitwise identical."""
    w = W.spheres_3d(seed=14, n_subdomains=2)
    a = E.run(w, 100)
    b = E.run(w, 100, options={N.OPT_PREFILTER: 0})
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])
    r = W.rods_2d(seed=14, n=4000)
    a = E.run(r, 20)
    b = E.run(r, 20, options={N.OPT_PREFILTER: 0})
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])


def test_gpu_determinism(gpu):
    w = W.spheres_3d(seed=15, n_subdomains=3)
    a = E.run(w, 50)
    b = E.run(w, 50)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["ids"], b["ids"])


@pytest.mark.parametrize("n_sub", [1, 5])
def test_rods_2d_one_step(gpu, oracle, n_sub):
    w = W.rods_2d(seed=21, n=3000, n_subdomains=n_sub)
    check_one_step(gpu, oracle, w)


def test_rods_3d_one_step(gpu, oracle):
    w = W.rods(1500, 300.0, seed=22, n_vertices=4, dim=3)
    check_one_step(gpu, oracle, w)


def test_rods_2d_trajectory(gpu, oracle):
    w = W.rods_2d(seed=23, n=3000)
    ref = oracle.run(w.model, w.pos, w.vel, 50, debug=True)
    got = E.run(w, 50)
    assert rel(got["pos"], ref["pos"]) <= 1e-10
    assert np.array_equal(got["voxel"], ref["voxel"])


@pytest.mark.parametrize("order", [2, 3])
def test_adams_bashforth_parity(gpu, oracle, order):
    w = W.spheres_3d(seed=31, solver_order=order)
    ref = oracle.run(w.model, w.pos, w.vel, 30)
    got = E.run(w, 30)
    assert rel(got["pos"], ref["pos"]) <= 1e-11
    r = W.rods_2d(seed=32, n=2000, solver_order=order)
    ref = oracle.run(r.model, r.pos, r.vel, 10)
    got = E.run(r, 10)
    assert rel(got["pos"], ref["pos"]) <= 1e-11


def test_mixed_precision_error(gpu):
    """FP32 pair forces with Kahan sums, FP64 state: relative position error against the FP64
    GPU path after 200 steps stays below 1e-5 (max over agents of |dx| / |x|)."""
    w = W.spheres_3d(seed=41)
    a = E.run(w, 200)
    b = E.run(W.Workload(w.name, w.model.replace(precision="mixed"), w.pos, w.vel, 200))
    err = np.linalg.norm(b["pos"] - a["pos"], axis=-1) / np.linalg.norm(a["pos"], axis=-1)
    assert float(err.max()) <= 1e-5


@pytest.mark.parametrize("dim,n_sub", [(3, 1), (3, 5), (2, 4)])
def test_mixed_kernel_variants_bitwise_identical(gpu, dim, n_sub):
    """Mixed-precision sphere kernels -- thread per agent and lane per agent with warp-packed
    survivors -- add the same FP32 terms in the same order: identical bits, single
    simulations and a batch of several."""
    w = W.spheres(20_000, 300.0 if dim == 3 else 2000.0, 63, dim, n_subdomains=n_sub,
                  precision="mixed")
    a = E.run(w, 60, options={N.OPT_KERNEL_VARIANT: 1})
    b = E.run(w, 60, options={N.OPT_KERNEL_VARIANT: 3})
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])
    ws = W.ensemble(seed=64, n_sims=3, n_lo=500, n_hi=5000, precision="mixed", n_steps=30)
    outs = []
    for variant in (1, 3):
        sim = E.Simulation([x.model for x in ws], [x.n for x in ws])
        sim.set_option(N.OPT_KERNEL_VARIANT, variant)
        sim.upload(np.concatenate([x.pos for x in ws]), np.concatenate([x.vel for x in ws]),
                   counts=[x.n for x in ws])
        sim.step(30)
        outs.append(sim.download(order="id"))
        sim.close()
    assert np.array_equal(outs[0]["pos"], outs[1]["pos"])


def test_boundary_error_reported(gpu):
    w = W.spheres(10, 100.0, seed=1, dim=3, dt=1.0, damping=0.0, strength=0.0)
    vel = np.zeros_like(w.vel)
    vel[3, 0, 0] = -1e4
    sim = E.Simulation.single(w.model, w.n)
    sim.upload(w.pos, vel)
    with pytest.raises(N.CrgError) as e:
        sim.step(5)
    assert e.value.code == N.CRG_EBOUNDARY and e.value.agent == 3 and e.value.step == 1
    sim.close()


def test_insertion_errors(gpu):
    w = W.spheres(10, 100.0, seed=1, dim=3)
    pos = w.pos.copy()
    pos[2, 0, 1] = 0.0
    with E.Simulation.single(w.model, w.n) as sim:
        with pytest.raises(N.CrgError) as e:
            sim.upload(pos, w.vel)
        assert e.value.code == N.CRG_EBOUNDARY
    pos = w.pos.copy()
    pos[4, 0, 2] = 100.0
    with E.Simulation.single(w.model, w.n) as sim:
        with pytest.raises(N.CrgError) as e:
            sim.upload(pos, w.vel)
        assert e.value.code == N.CRG_EINDEX


def test_large_grids_many_scan_tiles(gpu, oracle):
    """Voxel grids spanning many 4,096-voxel scan tiles (the cell-list scan is tiled)."""
    w = W.spheres_3d(seed=51, n=40_000)  # 28^3 = 21,952 voxels
    ref, st1 = check_one_step(gpu, oracle, w)
    r = W.rods_2d(seed=52, n=30_000, n_subdomains=7)  # 136^2 = 18,496 voxels
    check_one_step(gpu, oracle, r)


@pytest.mark.parametrize("n_sub", [1, 16])
def test_rod_kernel_variants_bitwise_identical(gpu, n_sub):
    """The pass-list rod path (default) and the thread-per-rod kernel evaluate the same items
    and add them in the same order: identical bits after many steps (16 subdomains: terms
    of chili's steps 2 and 3, summed per voxel)."""
    r = W.rods_2d(seed=61, n=20_000, n_subdomains=n_sub)
    a = E.run(r, 150)
    b = E.run(r, 150, options={N.OPT_KERNEL_VARIANT: 1})
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])


def test_rod_pass_list_overflow_falls_back_and_grows(gpu):
    """A pass list far too small for a step: that step's forces come from the rod-level
    kernel (same bits), the list is grown at the end of crg_step, and the later steps run on
    the pass list again.  The trajectory equals the default run bit for bit."""
    r = W.rods_2d(seed=63, n=20_000, n_subdomains=4)
    a = E.run(r, 40)
    with E.Simulation.single(r.model, r.n) as sim:
        sim.set_option(N.OPT_PASS_LIST, 1024)
        sim.upload(r.pos, r.vel)
        sim.step(5)   # overflows: rod-level kernel; the list grows afterwards
        sim.step(35)  # fits
        b = sim.download(order="id")
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])
    assert np.array_equal(a["voxel"], b["voxel"])


def test_rod_passes_without_survivors(gpu):
    """Rods in a checkerboard whose diagonal neighbours pass the bounding-box test but have
    no vertex/segment pair within the cutoff: every pass of the list has zero survivors, so
    every round of the pass kernel has nothing to evaluate.  Each pass must still store its
    (zero) M / 2 -- the pass list is allocated NaN-filled, so a missed store shows up as NaN
    -- and the result equals the thread-per-rod kernel bit for bit."""
    import math

    gap, length = 6.01, 3.0  # cutoff 6, prefilter threshold ~6.02
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
    b = E.run(r, 3, options={N.OPT_KERNEL_VARIANT: 1})
    assert np.all(np.isfinite(a["pos"]))
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])
    assert not math.isnan(float(a["vel"].sum()))


@pytest.mark.parametrize("n_sub", [1, 5])
def test_sphere_kernel_variants_bitwise_identical(gpu, n_sub):
    """FP64 sphere kernels -- agent groups of 8 lanes (the default at this size), of 16 and
    of 32 lanes, thread per agent (one-shot and persistent) and lane per agent with
    warp-packed survivors: identical bits."""
    w = W.spheres_3d(seed=62, n=20_000, n_subdomains=n_sub)
    a = E.run(w, 100)
    for opts in ({N.OPT_KERNEL_VARIANT: 1}, {N.OPT_KERNEL_VARIANT: 2},
                 {N.OPT_KERNEL_VARIANT: 2, N.OPT_BLOCK: 16},
                 {N.OPT_KERNEL_VARIANT: 2, N.OPT_BLOCK: 32},
                 {N.OPT_KERNEL_VARIANT: 1, N.OPT_BLOCK: 128, N.OPT_TILE: 2},
                 {N.OPT_KERNEL_VARIANT: 3}, {N.OPT_KERNEL_VARIANT: 3, N.OPT_BLOCK: 64}):
        b = E.run(w, 100, options=opts)
        assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])


def test_cell_list_order_over_many_steps(gpu, oracle):
    """After many steps with agents crossing voxels and subdomains, the GPU cell list holds
    exactly chili's per-voxel order."""
    for n_sub in (1, 6):
        w = W.spheres_3d(seed=53, n=6000, n_subdomains=n_sub)
        ref = oracle.run(w.model, w.pos, w.vel, 60, debug=True)
        got = E.run(w, 60, order="list")
        assert np.array_equal(got["ids"], ref["order"])
