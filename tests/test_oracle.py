"""Pins the CPU oracle against the known answers the reference's own tests hold.

The reference (Rust) cannot be built here, so the oracle's restatement is checked against:
  * doc/unit-test values of the reference (voxel counts, decomposition invariants,
    nearest-point values, solver truncation bounds, constant-velocity mechanics),
  * hand calculations of the chili pair weights, reflection and error paths,
  * analytic cases (two-body Morse equilibrium) and run-to-run determinism.
"""
import math

import numpy as np
import pytest

from cellular_raza_gb300 import workloads as W


def sphere_model(**kw):
    m = dict(kind="sphere", dim=3, n_vertices=1, domain_min=(0.0, 0.0, 0.0),
             domain_max=(100.0, 100.0, 100.0), interaction_range=20.0, mass=1.0, damping=0.1,
             radius=3.0, stiffness=0.5, cutoff=4.0, strength=0.01, dt=0.01)
    m.update(kw)
    return W.Model(**m)


# ---- cellular_raza-building-blocks/src/domains/cartesian_cuboid_n.rs -----------------

def test_voxel_counts_doc_example(oracle):
    # from_boundaries_and_interaction_range doc test (cartesian_cuboid_n.rs:167-182)
    m = sphere_model(domain_min=(2.0, 3.0, 1.0), domain_max=(10.0, 10.0, 20.0),
                     interaction_range=2.0)
    nv, dx = oracle.domain_voxels(m)
    assert nv == [4, 3, 9]
    assert dx == [8.0 / 4.0, 7.0 / 3.0, 19.0 / 9.0]


def test_get_decomp_res_invariants(oracle):
    # test_get_demomp_res (cartesian_cuboid_n.rs:665-700), debug-build bounds
    for n_voxel in range(1, 500):
        for n_regions in range(1, 100):
            res = oracle.get_decomp_res(n_voxel, n_regions)
            assert res is not None, (n_voxel, n_regions)
            n, m, avg = res
            assert n + m == n_regions
            assert n * avg + m * (avg - 1) == n_voxel


def test_generate_subdomains(oracle):
    # generate_subdomains (cartesian_cuboid_n.rs:380-402): 5^3 voxels in 4 subdomains
    m = sphere_model(n_subdomains=4)
    sub = oracle.subdomain_map(m)
    assert len(sub) == 5 ** 3
    assert sorted(set(sub.tolist())) == [0, 1, 2, 3]
    # contiguous chunks of the lexicographic voxel order
    assert np.all(np.diff(sub.astype(np.int64)) >= 0)


def test_neighbors_are_clipped_box(oracle):
    m = sphere_model()
    assert oracle.voxel_neighbors(m, 0) == [1, 5, 6, 25, 26, 30, 31]
    centre = 2 * 25 + 2 * 5 + 2
    nb = oracle.voxel_neighbors(m, centre)
    assert len(nb) == 26 and nb == sorted(nb) and centre not in nb


def test_insertion_errors(oracle):
    m = sphere_model()
    ok = np.array([[[1.0, 2.0, 3.0]]])
    assert oracle.initial_voxels(m, ok).tolist() == [0]
    with pytest.raises(oracle.OracleError) as e:  # pos <= min: check_min_max (:149-162, 321)
        oracle.initial_voxels(m, np.array([[[0.0, 2.0, 3.0]]]))
    assert e.value.code == oracle.EBOUNDARY
    with pytest.raises(oracle.OracleError) as e:  # index == n_voxels: no voxel
        oracle.initial_voxels(m, np.array([[[100.0, 2.0, 3.0]]]))
    assert e.value.code == oracle.EINDEX


# ---- cellular_raza-building-blocks/src/cell_building_blocks/interaction.rs -----------

def test_nearest_point_doc_example(oracle):
    # nearest_point_from_point_to_line doc test (interaction.rs:478-496)
    dist, point, t = oracle.nearest_point([0.0, 0.0], [1.0, 0.0], [-1.0, 2.0])
    assert abs(dist - 1.0 / math.sqrt(2.0)) < 1e-10
    assert abs(t - 0.25) < 1e-10
    assert abs(point[0] - 0.5) < 1e-10 and abs(point[1] - 0.5) < 1e-10


def test_closest_points_exact(oracle):
    # test_closest_points (interaction.rs:820-851) asserts exact equality
    p1, p2 = [0.0, 0.0], [2.0, 0.0]
    cases = [([0.5, 1.0], [0.5, 0.0], 1.0), ([-1.0, 2.0], p1, math.sqrt(5.0)),
             ([3.0, -2.0], p2, math.sqrt(5.0))]
    for q, r, d in cases:
        dist, point, _ = oracle.nearest_point(q, p1, p2)
        assert dist == d
        assert point.tolist() == r


def test_morse_formula(oracle):
    # calculate_morse_interaction (interaction.rs:151-182) by hand
    own, ext = np.array([1.0, 2.0, 3.0]), np.array([4.0, 6.0, 3.0])
    f1, f2 = oracle.morse(own, ext, 5.0, 5.0, 15.0, 0.5, 0.4)
    z = own - ext
    d = math.sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2])
    e = math.exp(-0.4 * (d - 10.0))
    F = -2.0 * 0.5 * 0.4 * e * (1.0 - e)
    assert np.array_equal(f1, (z / d) * F)
    assert np.array_equal(f2, (-(z / d)) * F)
    # beyond the cutoff and at zero distance the force vanishes
    z1, z2 = oracle.morse(own, own + 20.0, 5.0, 5.0, 15.0, 0.5, 0.4)
    assert not z1.any() and not z2.any()
    z1, _ = oracle.morse(own, own, 5.0, 5.0, 15.0, 0.5, 0.4)
    assert not z1.any()


# ---- cellular_raza-core/src/backend/chili/solvers.rs --------------------------------

def test_euler_exp_decay(oracle):
    # euler_exp_decay (solvers.rs:588-617)
    y0, lam, dt = 27.0, 0.3, 0.001
    y, t = y0, 0.0
    for _ in range(100):
        y = oracle.euler(y, -lam * y, dt)
        t += dt
        bound = dt * y0 * lam ** 2 / (2 * lam) * (math.exp(lam * t) - 1.0)
        assert abs(y - y0 * math.exp(-lam * t)) < bound


def test_adams_bashforth_2_harmonic_oscillator(oracle):
    # adams_bashforth_2_harmonic_oscillator (solvers.rs:619-710)
    y0, omega, dt = np.array([2.8347, 0.0]), 0.319, 0.045
    rhs = lambda y: np.array([y[1], -omega ** 2 * y[0]])
    exact = lambda t: np.array([y0[0] * math.cos(omega * t), -y0[0] * omega * math.sin(omega * t)])
    third = np.array([y0[0] * omega ** 3] * 2)
    lip = np.array([1.0, omega])
    local = third * (5.0 / 12.0 * dt ** 2)
    glob = lambda t: (np.exp(lip * t) - 1.0) * local / dt / lip
    t, y = 0.0, y0.copy()
    store = [rhs(exact(t - dt)), rhs(exact(t - 2 * dt))]
    for i in range(100):
        dy = rhs(y)
        store[1] = store[0]
        store[0] = dy
        y = np.array([oracle.adams_bashforth_2(y[k], store[0][k], store[1][k], dt) for k in range(2)])
        t += dt
        if i > 0:
            assert np.all(np.abs(y - exact(t)) < glob(t))


# ---- chili run loop -----------------------------------------------------------------

def test_constant_velocity_mechanics(oracle):
    # chili doc test (cellular_raza-core/src/backend/chili/mod.rs:116-158): without forces
    # pos = x0 + iteration * dt * v within 1e-5.
    n = 10
    m = sphere_model(domain_max=(1000.0, 1000.0, 1000.0), interaction_range=50.0, damping=0.0,
                     strength=0.0, dt=0.1)
    pos = np.zeros((n, 1, 3)) + 500.0
    pos[:, 0, 0] = 100.0 + 60.0 * np.arange(n)
    vel = np.zeros_like(pos)
    vel[:, 0, 0] = 0.1
    for it in (1, 10, 200):
        r = oracle.run(m, pos, vel, it)
        assert np.all(np.abs(r["pos"][:, 0, 0] - (pos[:, 0, 0] + it * 0.1 * 0.1)) < 1e-5)


def test_determinism(oracle):
    # determinism_mechanics_interaction (cellular_raza/tests/determinism_mechanics_interaction.rs
    # :44-108): identical trajectories on repeated runs, here also with several subdomains.
    rng = np.random.Generator(np.random.PCG64(1))
    pos = rng.uniform(0.0, 100.0, size=(10, 1, 3))
    vel = np.zeros_like(pos)
    for ns in (1, 3):
        m = sphere_model(n_subdomains=ns)
        a = oracle.run(m, pos, vel, 100)
        for _ in range(3):
            b = oracle.run(m, pos, vel, 100)
            assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])


def _two(model, p0, p1):
    pos = np.array([[p0], [p1]], dtype=np.float64)
    return pos, np.zeros_like(pos)


def _morse_np(own, ext, R=5.0, a=0.4, s=0.5, cutoff=15.0):
    z = own - ext
    d = math.sqrt(float(z @ z))
    if d > cutoff or d == 0.0:
        return np.zeros_like(z)
    e = math.exp(-a * (d - 2 * R))
    return (z / d) * (-2.0 * s * a * e * (1.0 - e))


@pytest.mark.parametrize("case", ["same_voxel", "neighbor_same_sub", "neighbor_other_sub"])
def test_chili_pair_weights(oracle, case):
    """chili keeps a force that a cell receives from a neighbour voxel of its own subdomain
    only from one side (update_mechanics.rs:205-220 drops the returned half)."""
    m = sphere_model(domain_max=(40.0, 20.0, 20.0), interaction_range=20.0, radius=5.0,
                     stiffness=0.4, cutoff=15.0, strength=0.5, damping=1.5)
    if case == "same_voxel":
        p0, p1, ns, w = [5.0, 10.0, 10.0], [14.0, 10.0, 10.0], 1, 1.0
    elif case == "neighbor_same_sub":
        p0, p1, ns, w = [15.0, 10.0, 10.0], [24.0, 10.0, 10.0], 1, 0.5
    else:
        p0, p1, ns, w = [15.0, 10.0, 10.0], [24.0, 10.0, 10.0], 2, 1.0
    m = m.replace(n_subdomains=ns)
    pos, vel = _two(m, p0, p1)
    r = oracle.run(m, pos, vel, 1, debug=True)
    f = _morse_np(np.array(p0), np.array(p1))
    assert np.allclose(r["force"][0, 0], w * f, rtol=1e-14, atol=0)
    assert np.allclose(r["force"][1, 0], -w * f, rtol=1e-14, atol=0)
    assert r["n_cand"].tolist() == [1, 1]


def test_two_body_morse_equilibrium(oracle):
    # Two spheres attract beyond 2R and settle at the Morse minimum d = 2R.
    m = sphere_model(domain_max=(60.0, 60.0, 60.0), interaction_range=20.0, radius=5.0,
                     stiffness=0.4, cutoff=15.0, strength=0.5, damping=1.5, dt=0.01)
    pos, vel = _two(m, [24.0, 30.0, 30.0], [36.0, 30.0, 30.0])
    r = oracle.run(m, pos, vel, 8000)
    d = np.linalg.norm(r["pos"][0, 0] - r["pos"][1, 0])
    assert abs(d - 10.0) < 1e-6


def test_reflecting_boundary(oracle):
    # CartesianSubDomain::apply_boundary (cartesian_cuboid_n.rs:594-631)
    m = sphere_model(damping=0.0, strength=0.0, dt=0.1)
    pos = np.array([[[0.5, 50.0, 99.5]]])
    vel = np.array([[[-10.0, 0.0, 10.0]]])
    r = oracle.run(m, pos, vel, 1)
    assert np.allclose(r["pos"][0, 0], [2 * 0.0 - (0.5 - 1.0), 50.0, 2 * 100.0 - (99.5 + 1.0)])
    assert r["vel"][0, 0].tolist() == [10.0, 0.0, -10.0]


def test_boundary_error(oracle):
    m = sphere_model(damping=0.0, strength=0.0, dt=1.0)
    pos = np.array([[[1.0, 50.0, 50.0]]])
    vel = np.array([[[-500.0, 0.0, 0.0]]])
    with pytest.raises(oracle.OracleError) as e:
        oracle.run(m, pos, vel, 1)
    assert e.value.code == oracle.EBOUNDARY and e.value.step == 1


def test_ab_solvers_history_quirk(oracle):
    """The history is pushed before it is read, so AB2 reduces to dx*(3/2) + dx*(-1/2) and
    AB3 uses [dx, previous dx, dx] (solvers.rs:171-231, 262-299)."""
    m = sphere_model(domain_max=(1000.0, 1000.0, 1000.0), interaction_range=100.0, damping=0.5,
                     strength=0.0, dt=0.1)
    pos = np.array([[[500.0, 500.0, 500.0]]])
    vel = np.array([[[3.0, -2.0, 1.0]]])
    for order in (1, 2, 3):
        x, v = pos[0, 0].copy(), vel[0, 0].copy()
        prev = None
        for step in range(5):
            dx, dv = v.copy(), (0.0 / 1.0 - 0.5 * v)
            if order == 1:
                xn, vn = dx * 0.1 + x, dv * 0.1 + v
            elif order == 2 or prev is None:
                xn = (dx * 1.5 + dx * -0.5) * 0.1 + x
                vn = (dv * 1.5 + dv * -0.5) * 0.1 + v
            else:
                f0, f1, f2 = 23.0 / 12.0, -16.0 / 12.0, 5.0 / 12.0
                xn = (dx * f0 + (prev[0] * f1 + dx * f2)) * 0.1 + x
                vn = (dv * f0 + (prev[1] * f1 + dv * f2)) * 0.1 + v
            prev = (dx, dv)
            x, v = xn, vn
        r = oracle.run(m.replace(solver_order=order), pos, vel, 5)
        assert np.array_equal(r["pos"][0, 0], x), order
        assert np.array_equal(r["vel"][0, 0], v), order


def test_straight_rod_at_rest(oracle):
    # RodMechanics (bacterial_rods.rs:157-213): springs at rest length and zero curvature
    w = W.rods(1, 100.0, seed=3, n_vertices=5, spring_length=3.0)
    pos = w.pos.copy()
    pos[0] = np.array([[40.0 + 3.0 * k, 50.0] for k in range(5)])
    r = oracle.run(w.model, pos, np.zeros_like(pos), 10)
    assert np.allclose(r["pos"], pos, atol=1e-12) and np.allclose(r["vel"], 0.0, atol=1e-12)


def test_rod_pair_forces_by_hand(oracle):
    # RodInteraction (bacterial_rods.rs:292-336) for two 2-vertex rods in one voxel
    m = W.rods(1, 100.0, n_vertices=2, spring_length=3.0).model.replace(
        interaction_range=50.0, spring_tension=0.0, rigidity=0.0, damping=0.0)
    A = np.array([[40.0, 50.0], [43.0, 50.0]])
    B = np.array([[41.0, 54.0], [44.0, 55.0]])
    pos = np.stack([A, B])
    r = oracle.run(m, pos, np.zeros_like(pos), 1, debug=True)

    def morse(own, ext):
        return _morse_np(own, ext, R=3.0, a=0.5, s=0.1, cutoff=6.0)

    def near(p, l0, l1):
        ab, ap = l1 - l0, p - l0
        t = min(max((ab @ ap) / (ab @ ab), 0.0), 1.0)
        return l0 * (1 - t) + l1 * t, t

    def calc(own, ext):
        fo, fe = np.zeros_like(own), np.zeros_like(own)
        for i in range(2):
            q, t = near(own[i], ext[0], ext[1])
            f = morse(own[i], q)
            fo[i] += f
            fe[0] += -f * (1 - t)
            fe[1] += -f * t
        return fo, fe

    oa, ea = calc(A, B)  # a.calc(a, b): own of A, ext on B
    ob, eb = calc(B, A)  # b.calc(b, a): own of B, ext on A
    fa = (oa * 0.5) + (eb * 0.5)  # A is first in the voxel: own then ext
    fb = (ea * 0.5) + (ob * 0.5)  # B is second: ext (from call 1) then own (call 2)
    assert np.allclose(r["force"][0], fa, rtol=1e-13, atol=1e-15)
    assert np.allclose(r["force"][1], fb, rtol=1e-13, atol=1e-15)


# ---- stochastic mechanics (Brownian / Langevin / RodMechanics diffusion) ------------

def test_philox4x32_10_known_answers(oracle):
    """Philox4x32-10 against the known-answer vectors published with the algorithm
    (Random123): zero, all-ones and the pi-digit counter/key."""
    assert oracle.philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c,
                                                          0x9b00dbd8]
    assert oracle.philox4x32_10([0xffffffff] * 4, [0xffffffff] * 2) == [
        0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert oracle.philox4x32_10([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                                [0xa4093822, 0x299f31d0]) == [0xd16cfe09, 0x94fdcceb,
                                                              0x5001e420, 0x24126ea1]


def test_normal_stream_statistics(oracle):
    z = np.concatenate([oracle.normals(11, s, i, 3) for s in range(100) for i in range(300)])
    n = z.size
    assert abs(z.mean()) < 4.0 / math.sqrt(n)
    assert abs(z.var() - 1.0) < 4.0 * math.sqrt(2.0 / n)
    assert abs(np.mean(z ** 4) - 3.0) < 0.1  # Gaussian kurtosis
    # deterministic, and distinct across ids, steps and seeds
    assert np.array_equal(oracle.normals(11, 5, 7, 6), oracle.normals(11, 5, 7, 6))
    assert not np.array_equal(oracle.normals(11, 5, 7, 6), oracle.normals(11, 5, 8, 6))
    assert not np.array_equal(oracle.normals(11, 5, 7, 6), oracle.normals(11, 6, 7, 6))
    assert not np.array_equal(oracle.normals(11, 5, 7, 6), oracle.normals(12, 5, 7, 6))


def free_particles(kind, n=3000, dim=3, **kw):
    """n non-interacting point particles (strength 0) far from the walls."""
    side = 1000.0
    rng = np.random.Generator(np.random.PCG64(3))
    pos = rng.uniform(400.0, 600.0, size=(n, 1, dim))
    m = W.Model(kind=kind, dim=dim, n_vertices=1, domain_min=(0.0,) * dim,
                domain_max=(side,) * dim, interaction_range=50.0, strength=0.0, dt=0.01, **kw)
    return m, pos, np.zeros_like(pos)


def test_brownian_free_diffusion_msd(oracle):
    """Brownian3D without forces: <|dx|^2> per axis = 2 D t (mechanics.rs:228-374)."""
    m, pos, vel = free_particles("brownian", diffusion=0.5, kb_temperature=1.0, rng_seed=5)
    out = oracle.run(m, pos, vel, 100)
    msd = np.mean((out["pos"] - pos) ** 2)
    expect = 2.0 * 0.5 * 1.0  # 2 D t, t = 100 * 0.01
    assert abs(msd / expect - 1.0) < 0.06  # ~2 % statistical error at 9,000 coordinates
    assert np.all(out["vel"] == 0.0)  # Brownian velocity stays zero


def test_langevin_equipartition(oracle):
    """Langevin3D without forces relaxes to <v^2> = k_B T / M per axis
    (mechanics.rs:376-475)."""
    m, pos, vel = free_particles("langevin", mass=2.0, damping=2.0, kb_temperature=0.5,
                                 rng_seed=9)
    out = oracle.run(m, pos, vel, 600)  # t = 6 = 12 relaxation times 1 / gamma
    v2 = np.mean(out["vel"] ** 2)
    assert abs(v2 / (0.5 / 2.0) - 1.0) < 0.08  # Euler bias ~ gamma dt / 2 = 1 %


def test_rod_diffusion_random_term(oracle):
    """RodMechanics with diffusion: each vertex coordinate moves by 2^-2 D sqrt(dt) z per step
    (bacterial_rods.rs:215-240) on top of the deterministic forces; with springs at rest,
    no bending and damping 0, one step's displacement has that variance."""
    n = 2000
    rng = np.random.Generator(np.random.PCG64(4))
    cen = rng.uniform(100.0, 900.0, size=(n, 2))
    pos = np.stack([cen + [-1.5, 0.0], cen + [1.5, 0.0]], axis=1)
    m = W.Model(kind="rod", dim=2, n_vertices=2, domain_min=(0.0, 0.0),
                domain_max=(1000.0, 1000.0), interaction_range=12.0, spring_tension=1.0,
                rigidity=0.0, spring_length=3.0, damping=0.0, diffusion=0.8, radius=0.1,
                stiffness=0.5, cutoff=0.2, strength=0.0, dt=0.01, rng_seed=21)
    out = oracle.run(m, pos, np.zeros_like(pos), 1)
    d = (out["pos"] - pos).ravel()
    expect = (0.25 * 0.8) ** 2 * 0.01
    assert abs(d.var() / expect - 1.0) < 0.08
