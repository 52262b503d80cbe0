"""Export of save points in chili's SerdeJson layout (cellular_raza_gb300/storage.py), on the
CPU: serde_json's number and pretty-print format, chili's file names and subdomain split,
and records of oracle states read back the way the reference's own plotting scripts read
them (cellular_raza-examples/bacterial_rods/plotter.py:20-38, cell_sorting/src/plot.py:55,
getting-started/src/plotting.py:53)."""
import json
import os

import numpy as np
import pytest

from cellular_raza_gb300 import storage as S
from cellular_raza_gb300 import workloads as W


@pytest.mark.parametrize("x,text", [
    (1.0, "1.0"), (0.1, "0.1"), (-2.5, "-2.5"), (0.0, "0.0"), (-0.0, "-0.0"),
    (0.001, "0.001"), (0.0001, "0.0001"), (0.00001, "0.00001"), (1e-6, "1e-6"),
    (1e-7, "1e-7"), (1.5e-7, "1.5e-7"), (123456789.0, "123456789.0"),
    (1e15, "1000000000000000.0"), (1e16, "1e16"), (1.5e20, "1.5e20"),
    (1234.5678, "1234.5678"), (5e-324, "5e-324"),
    (1.7976931348623157e308, "1.7976931348623157e308"), (float("nan"), "null"),
    (float("inf"), "null"),
])
def test_numbers_as_serde_json_prints_them(x, text):
    assert S.format_f64(x) == text


def test_numbers_round_trip():
    rng = np.random.Generator(np.random.PCG64(3))
    xs = np.concatenate([rng.standard_normal(2000) * 10.0 ** rng.integers(-30, 30, 2000),
                         rng.uniform(0, 3000, 2000)])
    for x in xs:
        assert float(S.format_f64(x)) == x


def test_pretty_printer_layout():
    v = {"data": [{"identifier": {"Initial": 3}, "element": [{"a": [1.0, 2.5]}, None]}],
         "empty": [], "obj": {}}
    text = S.to_pretty_json(v)
    assert text == ('{\n  "data": [\n    {\n      "identifier": {\n        "Initial": 3\n'
                    '      },\n      "element": [\n        {\n          "a": [\n'
                    '            1.0,\n            2.5\n          ]\n        },\n'
                    '        null\n      ]\n    }\n  ],\n  "empty": [],\n  "obj": {}\n}')
    assert json.loads(text) == v


def test_identifiers():
    assert S.cell_identifier(7) == {"Initial": 7}
    assert S.cell_identifier(S.ID_DIVISION | (12 << 32) | 5) == {"Division": [12, 5]}


def test_subdomains_follow_get_decomp_res():
    """Contiguous voxel chunks, sizes avg and avg - 1, every subdomain non-empty."""
    for n_vox, n_sub in [(62500, 16), (100, 7), (27, 27), (1000, 3), (8, 5)]:
        model = W.Model(dim=2, domain_min=(0.0, 0.0),
                        domain_max=(float(n_vox), 1.0), interaction_range=1.0,
                        n_subdomains=n_sub)
        sub = S.subdomain_of(model, np.arange(n_vox))
        assert sub[0] == 0 and sub[-1] == n_sub - 1
        assert np.all(np.diff(sub) >= 0) and np.all(np.diff(sub) <= 1)
        sizes = np.bincount(sub)
        assert len(sizes) == n_sub and sizes.max() - sizes.min() <= 1


def list_order(res):
    order = res["order"].astype(np.int64)
    return {"pos": res["pos"][order], "vel": res["vel"][order],
            "ids": res["order"], "voxel": res["voxel"][order]}


@pytest.mark.parametrize("n_sub", [1, 4])
def test_sphere_save_point_from_oracle(oracle, tmp_path, n_sub):
    w = W.spheres(600, 150.0, seed=5, dim=3, n_subdomains=n_sub)
    res = oracle.run(w.model, w.pos, w.vel, 10, debug=True)
    state = list_order(res)
    paths = S.export_cells(str(tmp_path), 10, w.model, state)
    # one file per chili thread, named as its StorageManager instance names it
    subs = np.unique(S.subdomain_of(w.model, state["voxel"]))
    assert [os.path.basename(p) for p in paths] == [
        f"batch_{s:020d}_{0:020d}.json" for s in subs]
    assert all(os.path.dirname(p).endswith(os.path.join("cells", "json", f"{10:020d}"))
               for p in paths)
    recs = S.load_cells(str(tmp_path), 10)
    # records in chili's storage order, agents recovered bit for bit
    assert [r["identifier"]["Initial"] for r in recs] == [int(i) for i in state["ids"]]
    got = S.positions_of(recs, "sphere", 3)
    assert np.array_equal(got, state["pos"])
    vel = np.array([r["cell"]["mechanics"]["vel"] for r in recs])
    assert np.array_equal(vel.reshape(state["vel"].shape), state["vel"])
    # what cell_sorting / getting-started plots read
    r0 = recs[0]
    assert r0["parent"] is None
    assert set(r0["cell"]["mechanics"]) == {"pos", "vel", "damping_constant", "mass"}
    assert r0["cell"]["interaction"]["potential_stiffness"] == w.model.stiffness


def test_rod_colony_save_point_from_oracle(oracle, tmp_path):
    """Rods with divisions: Division identifiers and parents, the bacterial-rods agent's
    fields, and positions read back as the reference's bacterial-rods plotter reads them
    (pos[0] reshaped to (3, vertices))."""
    w = W.rod_colony(n=60, side=200.0, seed=7, dim=3, n_subdomains=2)
    res = oracle.run_cycle(w.model, w.pos, w.vel, 80, spring_length=w.spring_length)
    assert np.any(res["ids"] & np.uint64(S.ID_DIVISION))
    paths = S.export_cells(str(tmp_path), 80, w.model, res)
    assert len(paths) >= 1
    with open(paths[0]) as f:
        elements = [e["element"][0] for e in json.load(f)["data"]]
    p = np.array(elements[0]["cell"]["mechanics"]["pos"][0], dtype=float).reshape(3, -1)
    first = int(np.nonzero(S.subdomain_of(w.model, res["voxel"]) ==
                           S.subdomain_of(w.model, res["voxel"][:1])[0])[0][0])
    assert np.array_equal(p[:, 0], res["pos"][first, 0])
    recs = S.load_cells(str(tmp_path), 80)
    assert np.array_equal(S.positions_of(recs, "rod", 3), res["pos"])
    assert any("Division" in r["identifier"] for r in recs)
    assert any(r["parent"] is not None for r in recs)
    assert [r["cell"]["mechanics"]["spring_length"] for r in recs] == [
        float(x) for x in res["spring_length"]]
    assert recs[0]["cell"]["spring_length_threshold"] == w.model.division_length
    assert recs[0]["cell"]["mechanics"]["pos"][1] == w.model.n_vertices


def test_records_read_back_as_upload_arrays(oracle, tmp_path):
    """state_from_records inverts the export: positions, velocities, identifiers, parents,
    spring lengths and growth rates of oracle states come back bit for bit, in storage
    order (spheres over four subdomains; a dividing rod colony)."""
    w = W.spheres(500, 140.0, seed=6, dim=3, n_subdomains=4)
    st = list_order(oracle.run(w.model, w.pos, w.vel, 8, debug=True))
    S.export_cells(str(tmp_path / "s"), 8, w.model, st)
    got = S.state_from_records(S.load_cells(str(tmp_path / "s"), 8), "sphere", 3)
    assert np.array_equal(got["pos"], st["pos"]) and np.array_equal(got["vel"], st["vel"])
    assert np.array_equal(got["ids"], st["ids"].astype(np.uint64))
    assert np.all(got["parent"] == np.uint64(S.NO_PARENT))

    c = W.rod_colony(n=60, side=200.0, seed=7, dim=2, n_subdomains=2)
    res = oracle.run_cycle(c.model, c.pos, c.vel, 80, spring_length=c.spring_length)
    S.export_cells(str(tmp_path / "r"), 80, c.model, res)
    got = S.state_from_records(S.load_cells(str(tmp_path / "r"), 80), "rod", 2)
    for k in ("pos", "vel", "ids", "parent", "spring_length", "growth_rate"):
        assert np.array_equal(got[k], np.asarray(res[k]).astype(got[k].dtype)), k
    assert S.crg_id({"Division": [12, 5]}) == S.ID_DIVISION | (12 << 32) | 5
