"""Stochastic mechanics on the GPU: Brownian and Langevin point agents and RodMechanics with
diffusion.  The GPU and the oracle draw the same counter-based random stream (Philox4x32-10
keyed by the seed, counter (draw, step, agent id), Box-Muller normals), so their trajectories
agree to libm rounding; the statistics are checked against the analytic values."""
import numpy as np
import pytest

from cellular_raza_gb300 import engine as E
from cellular_raza_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("order", [1, 3])
def test_brownian_interacting_parity(gpu, oracle, order):
    """Brownian3D + Morse (crowded start) against the oracle."""
    w = W.spheres(3000, 150.0, 31, 3, kind="brownian", diffusion=0.5, kb_temperature=2.0,
                  rng_seed=77, solver_order=order, n_subdomains=3)
    ref = oracle.run(w.model, w.pos, w.vel, 30)
    got = E.run(w, 30)
    assert rel_err(got["pos"], ref["pos"]) <= 1e-10
    assert np.all(got["vel"] == 0.0)


def test_langevin_interacting_parity(gpu, oracle):
    w = W.spheres(3000, 150.0, 32, 3, kind="langevin", mass=1.5, damping=1.0,
                  kb_temperature=0.8, rng_seed=78)
    ref = oracle.run(w.model, w.pos, w.vel, 30)
    got = E.run(w, 30)
    assert rel_err(got["pos"], ref["pos"]) <= 1e-10
    assert rel_err(got["vel"], ref["vel"]) <= 1e-8


def test_rod_diffusion_parity(gpu, oracle):
    """RodMechanics with diffusion != 0 (random term per vertex) against the oracle, through
    the default pass-list kernels and the thread-per-rod variant."""
    from cellular_raza_gb300 import _native as N

    r = W.rods(n=3000, side=500.0, seed=33, diffusion=0.6, rng_seed=79)
    ref = oracle.run(r.model, r.pos, r.vel, 20)
    got = E.run(r, 20)
    assert rel_err(got["pos"], ref["pos"]) <= 1e-10
    alt = E.run(r, 20, options={N.OPT_KERNEL_VARIANT: 1})
    assert np.array_equal(got["pos"], alt["pos"])


def test_stochastic_batch_members_equal_single_runs(gpu):
    """The random stream is keyed by agent id and pack step, not by position in the pack."""
    ws = [W.spheres(n, 120.0, 40 + k, 3, kind="brownian", diffusion=0.3 + 0.1 * k,
                    kb_temperature=1.0, rng_seed=100 + k) for k, n in enumerate((800, 1500, 400))]
    sim = E.Simulation([w.model for w in ws], [w.n for w in ws])
    sim.upload(np.concatenate([w.pos for w in ws]), np.concatenate([w.vel for w in ws]),
               counts=[w.n for w in ws])
    sim.step(25)
    out = sim.download(order="id")
    sim.close()
    off = 0
    for w in ws:
        alone = E.run(w, 25)
        assert np.array_equal(out["pos"][off:off + w.n], alone["pos"])
        off += w.n


def test_gpu_brownian_diffusion_constant(gpu):
    """Free Brownian particles on the GPU: mean squared displacement 2 D t per axis."""
    n, D = 200_000, 0.5
    rng = np.random.Generator(np.random.PCG64(6))
    pos = rng.uniform(400.0, 600.0, size=(n, 1, 3))
    m = W.Model(kind="brownian", dim=3, n_vertices=1, domain_min=(0.0,) * 3,
                domain_max=(1000.0,) * 3, interaction_range=50.0, strength=0.0, dt=0.01,
                diffusion=D, kb_temperature=1.0, rng_seed=17)
    w = W.Workload("free_brownian", m, pos, np.zeros_like(pos), 200)
    out = E.run(w)
    msd = np.mean((out["pos"] - pos) ** 2)
    assert abs(msd / (2.0 * D * 2.0) - 1.0) < 0.01  # 6e5 coordinates: ~0.2 % error


def test_brownian_mixed_precision_close_to_f64(gpu):
    """Brownian agents on the mixed-precision path (FP32 pair forces, Kahan sums) draw the
    same random stream as the FP64 path, so their trajectories stay close."""
    w = W.spheres(4000, 150.0, 34, 3, kind="brownian", diffusion=0.5, kb_temperature=2.0,
                  rng_seed=80)
    a = E.run(w, 50)
    b = E.run(W.Workload(w.name, w.model.replace(precision="mixed"), w.pos, w.vel, 50), 50)
    assert rel_err(b["pos"], a["pos"]) < 1e-5
    assert np.all(b["vel"] == 0.0)
