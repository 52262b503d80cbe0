"""Batched form: many independent simulations (uneven sizes and parameters) advanced by the
same launches.  Each simulation's result must not depend on its batch neighbours: bitwise
equal to running it alone, and within the FP64 bars of the oracle."""
import numpy as np
import pytest

from cellular_raza_gb300 import _native as N
from cellular_raza_gb300 import engine as E
from cellular_raza_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def run_batch(ws, steps):
    sim = E.Simulation([w.model for w in ws], [w.n for w in ws])
    sim.upload(np.concatenate([w.pos for w in ws]), np.concatenate([w.vel for w in ws]),
               counts=[w.n for w in ws])
    sim.step(steps)
    out = sim.download(order="id")
    sim.close()
    res, off = [], 0
    for w in ws:
        res.append({k: v[off:off + w.n] for k, v in out.items()})
        off += w.n
    return res


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_batch_members_equal_single_runs(gpu, precision):
    ws = W.ensemble(seed=81, n_sims=7, n_lo=200, n_hi=6000, precision=precision, n_steps=60)
    got = run_batch(ws, 60)
    for w, g in zip(ws, got):
        alone = E.run(w, 60)
        assert np.array_equal(g["pos"], alone["pos"]) and np.array_equal(g["vel"], alone["vel"])
        assert np.array_equal(g["voxel"], alone["voxel"])


def test_batch_member_oracle_parity(gpu, oracle):
    ws = W.ensemble(seed=82, n_sims=4, n_lo=500, n_hi=3000, precision="f64", n_steps=40)
    got = run_batch(ws, 40)
    for w, g in zip(ws, got):
        ref = oracle.run(w.model, w.pos, w.vel, 40, debug=True)
        err = np.max(np.abs(g["pos"] - ref["pos"])) / np.max(np.abs(ref["pos"]))
        assert err <= 1e-10
        assert np.array_equal(g["voxel"], ref["voxel"])


def test_rod_batch_members_equal_single_runs(gpu):
    """Rods of different sizes and parameters in one pack (the queue-fed force kernel hands
    rods of several simulations to the same warp): each equals its run alone.  One member is
    frozen after 30 of the 60 steps and must equal a 30-step run alone."""
    import ctypes as C

    ws = [W.rods(n=3000, side=500.0, seed=91),
          W.rods(n=700, side=260.0, seed=92, strength=0.15, dt=0.004),
          W.rods(n=5200, side=700.0, seed=93, rigidity=1.5)]
    sim = E.Simulation([w.model for w in ws], [w.n for w in ws])
    sim.upload(np.concatenate([w.pos for w in ws]), np.concatenate([w.vel for w in ws]),
               counts=[w.n for w in ws])
    N.check(sim._L.crg_set_sim_stop(sim._h, C.c_int32(1), C.c_int64(30)), "crg_set_sim_stop")
    sim.step(60)
    out = sim.download(order="id")
    sim.close()
    off = 0
    for s, w in enumerate(ws):
        g = {k: v[off:off + w.n] for k, v in out.items()}
        off += w.n
        alone = E.run(w, 30 if s == 1 else 60)
        assert np.array_equal(g["pos"], alone["pos"]) and np.array_equal(g["vel"], alone["vel"])


def run_pack_shape(ws, steps, variant, block, tile):
    sim = E.Simulation([w.model for w in ws], [w.n for w in ws])
    sim.set_option(N.OPT_KERNEL_VARIANT, variant)
    sim.set_option(N.OPT_BLOCK, block)
    sim.set_option(N.OPT_TILE, tile)
    assert sim.get_option(N.OPT_TILE) == tile
    sim.upload(np.concatenate([w.pos for w in ws]), np.concatenate([w.vel for w in ws]),
               counts=[w.n for w in ws])
    sim.step(steps)
    out = sim.download(order="id")
    sim.close()
    return out


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_persistent_tiles_equal_one_shot_grid(gpu, precision):
    """The persistent tile kernel (blocks claiming tiles of block x k agents until none is
    left) does each agent's work exactly as the one-thread-per-agent grid does: bitwise equal
    for every block and tile size, on a pack of uneven simulations (3D and 2D)."""
    for dim in (3, 2):
        rng = np.random.Generator(np.random.PCG64(83 + dim))
        ns = np.exp(rng.uniform(np.log(150), np.log(9000), size=9)).astype(int)
        # 3D at the ensemble's density; 2D at one agent per 250 unit^2
        ws = [W.spheres(int(n), (n / 5.12e-4) ** (1 / 3) if dim == 3 else (n * 250.0) ** 0.5,
                        seed=900 + s, dim=dim, strength=float(rng.uniform(0.1, 1.0)),
                        damping=float(rng.uniform(0.5, 2.0)), precision=precision)
              for s, n in enumerate(ns)]
        ref = run_pack_shape(ws, 40, 1, 128, 0)
        for block, tile in [(64, 1), (128, 1), (128, 3), (256, 2), (256, 16)]:
            got = run_pack_shape(ws, 40, 1, block, tile)
            for k in ("pos", "vel", "voxel"):
                assert np.array_equal(got[k], ref[k]), (dim, block, tile, k)


def test_autotune_reports_tile_and_keeps_state(gpu):
    ws = W.ensemble(seed=86, n_sims=5, n_lo=300, n_hi=5000, precision="mixed", n_steps=20)
    sim = E.Simulation([w.model for w in ws], [w.n for w in ws])
    sim.upload(np.concatenate([w.pos for w in ws]), np.concatenate([w.vel for w in ws]),
               counts=[w.n for w in ws])
    sim.step(5)
    before = sim.download(order="id")
    tune = sim.autotune(2)
    assert tune["tile"] == sim.get_option(N.OPT_TILE)
    assert tune["block"] == sim.get_option(N.OPT_BLOCK)
    after = sim.download(order="id")
    assert np.array_equal(before["pos"], after["pos"])
    sim.step(10)
    got = sim.download(order="id")
    sim.close()
    ref = run_pack_shape(ws, 15, 1, 128, 0)
    assert np.array_equal(got["pos"], ref["pos"]) and np.array_equal(got["vel"], ref["vel"])
