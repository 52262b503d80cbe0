"""Known answers of the oracle's cell cycle (bacterial-rods agent: neighbour-limited growth and
RodMechanics::divide), worked out by hand from the reference's formulas
(cellular_raza-examples/bacterial_rods/src/main.rs:48-112,
cellular_raza-building-blocks/src/cell_building_blocks/bacterial_rods.rs:586-663,
cellular_raza-core/src/backend/chili/update_cycle.rs:10-69)."""
import numpy as np
import pytest

from cellular_raza_gb300 import workloads as W

DIV = 1 << 63


def colony_model(**kw):
    base = dict(kind="rod", dim=2, n_vertices=5, domain_min=(0.0, 0.0),
                domain_max=(200.0, 100.0), interaction_range=40.0, spring_tension=10.0,
                rigidity=1.0, spring_length=3.0, damping=1.5, radius=3.0, stiffness=0.5,
                cutoff=5.0, strength=0.1, dt=0.01, cycle=True, growth_rate=0.0,
                division_length=6.0, sense_range=6.0, sense_saturation=8.0)
    base.update(kw)
    return W.Model(**base)


def test_division_of_a_straight_rod(oracle):
    """A straight rod at rest with spring length 6.5 > 6 divides in its first step.  Length
    26 = 4 x 6.5, so the halves' vertices sit (26 - 2 x 3) / 4 / 2 = 2.5 apart: the first
    half from the first vertex on, the second back from the last; both get spring length
    (1/2 - 3 / (5 x 6.5)) x 6.5 = 2.65.  The voxel (plain index 1) held one initial agent,
    so the parent becomes Division(1, 2) and the daughter Division(1, 3), both with parent 0."""
    m = colony_model()
    x = 10.0 + 6.5 * np.arange(5)
    pos = np.stack([x, np.full(5, 50.0)], axis=1)[None]
    out = oracle.run_cycle(m, pos, np.zeros_like(pos), 1, spring_length=np.array([6.5]))
    assert list(out["ids"]) == [DIV | (1 << 32) | 2, DIV | (1 << 32) | 3]
    assert list(out["parent"]) == [0, 0]
    np.testing.assert_allclose(out["pos"][0, :, 0], 10.0 + 2.5 * np.arange(5), rtol=1e-14)
    np.testing.assert_allclose(out["pos"][1, :, 0], 26.0 + 2.5 * np.arange(5), rtol=1e-14)
    assert np.all(out["pos"][:, :, 1] == 50.0)
    np.testing.assert_allclose(out["spring_length"], [2.65, 2.65], rtol=1e-14)


def test_neighbour_limited_growth(oracle):
    """Two parallel rods 5.5 apart (vertices 3 apart): only facing vertices are closer than
    6 (sqrt(3^2 + 5.5^2) > 6), so each rod senses n = 5 and grows at 2 x (8 - 5) / 8."""
    m = colony_model(growth_rate=2.0, division_length=100.0)
    x = 50.0 + 3.0 * np.arange(5)
    a = np.stack([x, np.full(5, 50.0)], axis=1)
    b = np.stack([x, np.full(5, 55.5)], axis=1)
    pos = np.stack([a, b])
    out = oracle.run_cycle(m, pos, np.zeros_like(pos), 1)
    assert np.all(out["growth_rate"] == 2.0 * (8.0 - 5.0) / 8.0)
    assert np.all(out["spring_length"] == 3.0 + 0.75 * 0.01)
    # far apart: no neighbours, the base rate
    pos[1, :, 1] = 90.0
    out = oracle.run_cycle(m, pos, np.zeros_like(pos), 1)
    assert np.all(out["growth_rate"] == 2.0)


def test_crowded_rods_stop_growing(oracle):
    """Rods 4 apart share 13 close vertex pairs: 2 x (8 - 13) / 8 < 0 is clamped to 0."""
    m = colony_model(growth_rate=2.0, division_length=100.0)
    x = 50.0 + 3.0 * np.arange(5)
    pos = np.stack([np.stack([x, np.full(5, 50.0)], 1), np.stack([x, np.full(5, 54.0)], 1)])
    out = oracle.run_cycle(m, pos, np.zeros_like(pos), 1)
    assert np.all(out["growth_rate"] == 0.0)
    assert np.all(out["spring_length"] == 3.0)


@pytest.mark.parametrize("dim,n_sub", [(2, 1), (2, 4), (3, 2)])
def test_colony_grows_and_ids_are_unique(oracle, dim, n_sub):
    """A growing colony: agents are only added, identifiers stay unique, every Division
    identifier names a voxel of the domain, every parent is an identifier seen before."""
    w = W.rod_colony(n=120, side=300.0 if dim == 2 else 120.0, seed=4, dim=dim,
                     n_subdomains=n_sub)
    out = oracle.run_cycle(w.model, w.pos, w.vel, 200, spring_length=w.spring_length)
    n = len(out["ids"])
    assert n > 120
    assert len(set(out["ids"].tolist())) == n
    n_vox = int(np.prod(oracle.domain_voxels(w.model)[0][:dim]))

    def names_a_voxel(x):
        return (x >> np.uint64(63) == 1) & ((x >> np.uint64(32)) & np.uint64(0x7fffffff) < n_vox)

    div = out["ids"] >> np.uint64(63) == 1
    assert np.all(names_a_voxel(out["ids"][div]))
    assert np.all(out["ids"][~div] < 120)
    par = out["parent"][div]
    assert np.all((par < 120) | names_a_voxel(par))
    assert np.all(out["parent"][~div] == np.uint64((1 << 64) - 1))
    assert np.all(out["spring_length"] > 0.0)


@pytest.mark.parametrize("order", [1, 3])
def test_cycle_without_growth_equals_plain_rods(oracle, order):
    """Growth 0 and every spring length at the model's: no division, so the cycle run moves
    the rods exactly as the plain rod step does (same storage order, same bits)."""
    w = W.rod_colony(n=120, seed=8, growth_rate=0.0, n_subdomains=3, solver_order=order)
    cyc = oracle.run_cycle(w.model, w.pos, w.vel, 150)
    plain = oracle.run(w.model.replace(cycle=False), w.pos, w.vel, 150, debug=True)
    assert np.array_equal(cyc["ids"], plain["order"])
    ids = cyc["ids"].astype(np.int64)
    assert np.array_equal(cyc["pos"], plain["pos"][ids])
    assert np.array_equal(cyc["vel"], plain["vel"][ids])
    assert np.all(cyc["parent"] == np.uint64((1 << 64) - 1))


def test_two_divisions_in_one_voxel(oracle):
    """Two rods of one voxel (plain index 1, two initial agents: counter 2) divide in the same
    step.  chili renames the parents first, in storage order (Division(1, 3), (1, 4)), then
    appends the daughters (Division(1, 5), (1, 6)) in the same order
    (chili/update_cycle.rs:30-64)."""
    m = colony_model()
    x = 10.0 + 6.5 * np.arange(5)
    a = np.stack([x, np.full(5, 55.0)], axis=1)
    b = np.stack([x, np.full(5, 90.0)], axis=1)
    pos = np.stack([a, b])
    out = oracle.run_cycle(m, pos, np.zeros_like(pos), 1, spring_length=np.array([6.5, 6.5]))
    v = 1 << 32
    assert list(out["ids"]) == [DIV | v | 3, DIV | v | 4, DIV | v | 5, DIV | v | 6]
    assert list(out["parent"]) == [0, 1, 0, 1]
    assert list(out["voxel"]) == [1, 1, 1, 1]


def test_division_error_for_a_rod_shorter_than_two_radii(oracle):
    """RodMechanics::divide finds no segment when (length - 2 R) < 0: a DivisionError, which
    ends the run with an error (CalcError here)."""
    m = colony_model(division_length=1.0)
    x = 10.0 + 1.2 * np.arange(5)  # length 4.8 < 2 R = 6
    pos = np.stack([x, np.full(5, 50.0)], axis=1)[None]
    with pytest.raises(oracle.OracleError) as e:
        oracle.run_cycle(m, pos, np.zeros_like(pos), 1, spring_length=np.array([1.2]))
    assert e.value.code == oracle.ECALC
