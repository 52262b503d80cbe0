"""Save points exported from GPU states (crg_download) against the same export of the oracle's
states: the same files, the same records in the same order, the same identifiers and
parents; numbers within the trajectory tolerance, and byte-identical files wherever the two
states are bit for bit equal."""
import os

import numpy as np
import pytest

from cellular_raza_gb300 import engine as E
from cellular_raza_gb300 import storage as S
from cellular_raza_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def files(root):
    out = {}
    for dirpath, _, names in os.walk(root):
        for n in names:
            p = os.path.join(dirpath, n)
            with open(p, "rb") as f:
                out[os.path.relpath(p, root)] = f.read()
    return out


def compare(model, gpu_state, ref_state, tmp_path, it, kind, dim, tol):
    a, b = str(tmp_path / "gpu"), str(tmp_path / "oracle")
    S.export_cells(a, it, model, gpu_state)
    S.export_cells(b, it, model, ref_state)
    fa, fb = files(a), files(b)
    assert sorted(fa) == sorted(fb)
    ra, rb = S.load_cells(a, it), S.load_cells(b, it)
    assert [r["identifier"] for r in ra] == [r["identifier"] for r in rb]
    assert [r["parent"] for r in ra] == [r["parent"] for r in rb]
    pa, pb = S.positions_of(ra, kind, dim), S.positions_of(rb, kind, dim)
    assert np.max(np.abs(pa - pb)) <= tol * np.max(np.abs(pb))
    if all(np.array_equal(gpu_state[k], ref_state[k]) for k in ("pos", "vel")):
        assert fa == fb


@pytest.mark.parametrize("n_sub", [1, 4])
def test_sphere_save_point(gpu, oracle, tmp_path, n_sub):
    w = W.spheres(2000, 200.0, seed=11, dim=3, n_subdomains=n_sub)
    ref = oracle.run(w.model, w.pos, w.vel, 20, debug=True)
    order = ref["order"].astype(np.int64)
    ref_state = {"pos": ref["pos"][order], "vel": ref["vel"][order], "ids": ref["order"],
                 "voxel": ref["voxel"][order]}
    with E.Simulation.single(w.model, w.n) as sim:
        sim.upload(w.pos, w.vel)
        sim.step(20)
        got = sim.download(order="list")
    compare(w.model, got, ref_state, tmp_path, 20, "sphere", 3, 1e-12)


def test_rod_colony_save_point(gpu, oracle, tmp_path):
    w = W.rod_colony(n=120, seed=12, dim=2, n_subdomains=2)
    ref = oracle.run_cycle(w.model, w.pos, w.vel, 100, spring_length=w.spring_length)
    got = E.run(w, 100, order="list")
    compare(w.model, got, ref, tmp_path, 100, "rod", 2, 1e-9)


@pytest.mark.parametrize("kind", ["sphere", "rod"])
def test_resume_from_save_point(gpu, tmp_path, kind):
    """A run stopped at a save point and resumed from its SerdeJson files (a new handle,
    agents uploaded in the save point's storage order) equals the uninterrupted run bit for
    bit: the numbers round-trip exactly and the cell list is the saved one (Euler, no
    solver history to lose)."""
    if kind == "sphere":
        w = W.spheres(3000, 230.0, seed=21, dim=3, n_subdomains=4)
    else:
        w = W.rods(n=2500, side=400.0, seed=22, n_subdomains=4)
    with E.Simulation.single(w.model, w.n) as sim:
        sim.upload(w.pos, w.vel)
        sim.step(20)
        paths = sim.save_point(str(tmp_path), 20)
        assert paths and all(os.path.exists(p) for p in paths)
        sim.step(20)
        ref = sim.download(order="list")
    with E.resume_save_point(str(tmp_path), 20, w.model) as sim:
        sim.step(20)
        got = sim.download(order="list")
    for k in ("pos", "vel", "ids", "voxel"):
        assert np.array_equal(got[k], ref[k]), k
