"""Cell records in the layout chili's `save_cells` writes with `StorageOption::SerdeJson`.

At a save point every chili subdomain thread stores its cells in one batch file
(chili/datastructures.rs:373-396, storage/concepts.rs:700-742, 766-790):

    {location}/cells/json/{iteration:020}/batch_{subdomain:020}_{counter:020}.json

holding `BatchSaveFormat { data: Vec<CombinedSaveFormat { identifier, element }> }`
(storage/concepts.rs:156-170) written by `serde_json::to_writer_pretty`, with
`element = (CellBox<C>, AuxStorage)`.  The subdomain's cells come in its voxels' order
(BTreeMap by voxel plain index) and, inside a voxel, in the voxel's storage order: the cell
list order of a handle.  `export_cells` writes these files from a `crg_download` (or any
state in cell-list order).

What each part of a record is, with the serde derive it follows:

* `identifier` / `CellBox::identifier`: `CellIdentifier` (concepts/src/cell.rs:16-25),
  an externally tagged enum: `{"Initial": k}` or `{"Division": [voxel, counter]}`
  (`VoxelPlainIndex` is a newtype and serialises as its number);
* `CellBox::parent`: `Option<CellIdentifier>`, `null` for initial agents;
* `CellBox::cell`: the agent struct.  The in-scope agents are written as the reference's
  examples declare them, a struct with the fields `mechanics` and `interaction`
  (cellular_raza-examples/bacterial_rods/src/main.rs:11-20; the cell_sorting and
  getting-started plots read `cell.mechanics.pos` and `cell.interaction.*`), plus
  `growth_rate` and `spring_length_threshold` for the bacterial-rods cell cycle:
  - NewtonDamped{2,3}D: `pos`, `vel` (nalgebra `SVector`, a flat array), `damping_constant`,
    `mass` (building-blocks/.../mechanics.rs:54-65);
  - Brownian{2,3}D: `pos`, `diffusion_constant`, `kb_temperature` (:255-261);
  - Langevin{2,3}D: `pos`, `vel`, `mass`, `damping`, `kb_temperature` (:415-426);
  - RodMechanics<f64, D>: `pos`, `vel` as nalgebra `VecStorage` triples `[data, nrows,
    ncols]` with the data column-major (all x, then all y, ...; the bacterial-rods plotter
    reads `pos[0]` and reshapes it to (D, n)), `diffusion_constant`, `spring_tension`,
    `rigidity`, `spring_length`, `damping` (bacterial_rods.rs:82-108);
  - MorsePotential: `radius`, `potential_stiffness`, `cutoff`, `strength`
    (interaction.rs:215-224); `RodInteraction` is a newtype around it (serialised as it).
* the second half of `element`, chili's aux storage, holds solver history in
  `circ_buffer` 0.1.8 ring buffers; that crate is not part of the reference tree, so its
  serde encoding cannot be restated here.  It is written as `null` unless the caller
  passes `aux` (one JSON-ready object per agent).

Numbers are printed as serde_json prints them (shortest round-trip digits in ryu's
layout: `1.0`, `0.001`, `1e-7`, `1.5e20`), with serde_json's pretty-printer indentation,
so a file written here from a state equal to the oracle's is byte-identical to the file
written from the oracle's state.  Non-finite numbers become `null`, as serde_json writes
them.
"""
from __future__ import annotations

import json
import math
import os
from typing import Dict, List, Optional, Sequence

import numpy as np

ID_DIVISION = 1 << 63
NO_PARENT = (1 << 64) - 1


# -- serde_json formatting -----------------------------------------------------------------

def format_f64(x: float) -> str:
    """A finite f64 as serde_json prints it (ryu's shortest representation and layout)."""
    x = float(x)
    if not math.isfinite(x):
        return "null"
    if x == 0.0:
        return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
    sign = "-" if x < 0 else ""
    r = repr(abs(x))  # shortest round-trip digits
    mant, _, exp = r.partition("e")
    e10 = int(exp) if exp else 0
    if "." in mant:
        ip, fp = mant.split(".")
    else:
        ip, fp = mant, ""
    digits = (ip + fp).lstrip("0")
    # position of the decimal point relative to the first significant digit
    lead_zeros = len(ip + fp) - len((ip + fp).lstrip("0"))
    point = len(ip) + e10 - lead_zeros
    digits = digits.rstrip("0") or "0"
    n = len(digits)
    kk = point  # value = 0.d1d2... x 10^kk
    if 0 < kk <= 16:
        if n <= kk:
            return sign + digits + "0" * (kk - n) + ".0"
        return sign + digits[:kk] + "." + digits[kk:]
    if -5 < kk <= 0:
        return sign + "0." + "0" * (-kk) + digits
    e = kk - 1
    m = digits if n == 1 else digits[0] + "." + digits[1:]
    return sign + m + "e" + str(e)


def _dump(v, indent: int, out: List[str]):
    pad = "  " * indent
    if v is None:
        out.append("null")
    elif isinstance(v, bool):
        out.append("true" if v else "false")
    elif isinstance(v, (int, np.integer)):
        out.append(str(int(v)))
    elif isinstance(v, (float, np.floating)):
        out.append(format_f64(float(v)))
    elif isinstance(v, str):
        out.append(json.dumps(v))
    elif isinstance(v, (list, tuple)):
        if not v:
            out.append("[]")
            return
        out.append("[\n")
        for k, item in enumerate(v):
            out.append(pad + "  ")
            _dump(item, indent + 1, out)
            out.append(",\n" if k + 1 < len(v) else "\n")
        out.append(pad + "]")
    elif isinstance(v, dict):
        if not v:
            out.append("{}")
            return
        out.append("{\n")
        items = list(v.items())
        for k, (key, item) in enumerate(items):
            out.append(pad + "  " + json.dumps(key) + ": ")
            _dump(item, indent + 1, out)
            out.append(",\n" if k + 1 < len(items) else "\n")
        out.append(pad + "}")
    else:
        raise TypeError(f"cannot serialise {type(v).__name__}")


def to_pretty_json(v) -> str:
    """serde_json::to_writer_pretty's text of a JSON-ready value (two-space indent)."""
    out: List[str] = []
    _dump(v, 0, out)
    return "".join(out)


# -- records -------------------------------------------------------------------------------

def cell_identifier(ident: int):
    """CellIdentifier of a crg id: Division(voxel, counter) for ids with CRG_ID_DIVISION,
    else Initial(id)."""
    ident = int(ident)
    if ident & ID_DIVISION:
        return {"Division": [(ident >> 32) & 0x7FFFFFFF, ident & 0xFFFFFFFF]}
    return {"Initial": ident}


def _svec(x) -> list:
    return [float(c) for c in np.asarray(x, dtype=np.float64).ravel()]


def _rod_matrix(x) -> list:
    """nalgebra Matrix<f64, Dyn, Const<D>, VecStorage>: [column-major data, nrows, ncols]
    (ncols, a Const, serialises as a unit: null)."""
    x = np.asarray(x, dtype=np.float64)
    return [[float(c) for c in x.T.ravel()], int(x.shape[0]), None]


def agent_cell(model, pos, vel, spring_length: Optional[float] = None,
               growth_rate: Optional[float] = None) -> Dict:
    """The `cell` of one agent (see the module docstring for the layouts)."""
    inter = {"radius": float(model.radius), "potential_stiffness": float(model.stiffness),
             "cutoff": float(model.cutoff), "strength": float(model.strength)}
    kind = model.kind
    if kind == "rod":
        mech = {"pos": _rod_matrix(pos), "vel": _rod_matrix(vel),
                "diffusion_constant": float(model.diffusion),
                "spring_tension": float(model.spring_tension),
                "rigidity": float(model.rigidity),
                "spring_length": float(model.spring_length if spring_length is None
                                       else spring_length),
                "damping": float(model.damping)}
    elif kind == "sphere":
        mech = {"pos": _svec(pos), "vel": _svec(vel), "damping_constant": float(model.damping),
                "mass": float(model.mass)}
    elif kind == "brownian":
        mech = {"pos": _svec(pos), "diffusion_constant": float(model.diffusion),
                "kb_temperature": float(model.kb_temperature)}
    elif kind == "langevin":
        mech = {"pos": _svec(pos), "vel": _svec(vel), "mass": float(model.mass),
                "damping": float(model.damping), "kb_temperature": float(model.kb_temperature)}
    else:
        raise ValueError(f"unknown agent kind {kind!r}")
    cell = {"mechanics": mech, "interaction": inter}
    if getattr(model, "cycle", False):
        cell["growth_rate"] = float(model.growth_rate if growth_rate is None else growth_rate)
        cell["spring_length_threshold"] = float(model.division_length)
    return cell


# -- chili's subdomains --------------------------------------------------------------------

def voxel_counts(model) -> List[int]:
    """Voxels per axis of the model's CartesianCuboid (cartesian_cuboid_n.rs:183-256)."""
    out = []
    for i in range(model.dim):
        lo, hi = model.domain_min[i], model.domain_max[i]
        if model.n_voxels is not None:
            out.append(int(model.n_voxels[i]))
        else:
            n = math.floor((hi - lo) / model.interaction_range)
            out.append(max(int(n), 1))
    return out


def decomp_res(n_voxel: int, n_regions: int):
    """get_decomp_res (cartesian_cuboid_n.rs:19-59): n chunks of `avg` voxels followed by m
    chunks of avg - 1."""
    average_len = math.ceil(n_voxel / n_regions)
    n, m = n_regions, 0
    for _ in range(n_regions):
        r = n_voxel - average_len * n - (average_len - 1) * m
        if r == 0:
            return n, m, average_len
        if r > 0:
            if n == n_regions:
                average_len += 1
                n, m = n_regions, 0
        else:
            n -= 1
            m += 1
    raise ValueError("no decomposition of the voxels into the requested subdomains")


def subdomain_of(model, voxels: np.ndarray) -> np.ndarray:
    """Subdomain (chili's thread key) of every voxel plain index."""
    total = int(np.prod(voxel_counts(model)))
    n, _, avg = decomp_res(total, int(model.n_subdomains))
    v = np.asarray(voxels, dtype=np.int64)
    div2 = max(avg - 1, 1)
    return np.where(v < n * avg, v // avg, (v - n * avg) // div2 + n)


# -- files ---------------------------------------------------------------------------------

def batch_path(location: str, iteration: int, subdomain: int, counter: int = 0) -> str:
    return os.path.join(location, "cells", "json", f"{int(iteration):020d}",
                        f"batch_{int(subdomain):020d}_{int(counter):020d}.json")


def export_cells(location: str, iteration: int, model, state: Dict[str, np.ndarray],
                 aux: Optional[Sequence] = None) -> List[str]:
    """Write one save point of a single simulation as chili's SerdeJson storage does.

    ``state``: arrays in cell-list order, as ``Simulation.download(order="list")`` returns
    them (``pos``, ``vel``, ``ids``, ``voxel``; ``parent``, ``spring_length`` and
    ``growth_rate`` for the cell cycle).  One file per subdomain that holds cells, as each
    chili thread writes its own; returns the paths written."""
    pos, vel = np.asarray(state["pos"]), np.asarray(state["vel"])
    ids = np.asarray(state["ids"], dtype=np.uint64)
    vox = np.asarray(state["voxel"], dtype=np.int64)
    parent = state.get("parent")
    slen = state.get("spring_length")
    grate = state.get("growth_rate")
    if np.any(np.diff(vox) < 0):
        raise ValueError("state is not in cell-list order (voxels must not decrease)")
    sub = subdomain_of(model, vox)
    paths = []
    for s in np.unique(sub):
        rows = np.nonzero(sub == s)[0]
        data = []
        for r in rows:
            ident = cell_identifier(ids[r])
            p = None
            if parent is not None and int(parent[r]) != NO_PARENT:
                p = cell_identifier(parent[r])
            agent_pos = pos[r] if model.kind == "rod" else pos[r].reshape(-1)
            agent_vel = vel[r] if model.kind == "rod" else vel[r].reshape(-1)
            cell = agent_cell(model, agent_pos, agent_vel,
                              None if slen is None else float(slen[r]),
                              None if grate is None else float(grate[r]))
            box = {"identifier": ident, "parent": p, "cell": cell}
            data.append({"identifier": ident,
                         "element": [box, None if aux is None else aux[r]]})
        path = batch_path(location, iteration, int(s))
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            f.write(to_pretty_json({"data": data}))
        paths.append(path)
    return paths


def load_cells(location: str, iteration: int) -> List[Dict]:
    """The CellBox records of one save point (every batch file, in file-name order)."""
    folder = os.path.join(location, "cells", "json", f"{int(iteration):020d}")
    out = []
    for name in sorted(os.listdir(folder)):
        with open(os.path.join(folder, name)) as f:
            out.extend(e["element"][0] for e in json.load(f)["data"])
    return out


def crg_id(identifier: Dict) -> int:
    """The crg id of a CellIdentifier record (the inverse of `cell_identifier`)."""
    if "Initial" in identifier:
        return int(identifier["Initial"])
    voxel, counter = identifier["Division"]
    return ID_DIVISION | (int(voxel) << 32) | int(counter)


def _floats(x) -> np.ndarray:
    """Numbers of a record; serde_json writes non-finite numbers as null, read as NaN."""
    return np.asarray([math.nan if v is None else v for v in x], dtype=np.float64)


def state_from_records(records: List[Dict], kind: str, dim: int) -> Dict[str, np.ndarray]:
    """The arrays of loaded records, in their storage order, as `Simulation.upload` and
    `set_spring_lengths` take them: ``pos`` and ``vel`` (n, vertices, dim; zeros for
    Brownian agents, which have no velocity), ``ids`` and ``parent`` (uint64, NO_PARENT for
    none), and for rods ``spring_length``; with the cell cycle also ``growth_rate``."""
    n = len(records)
    pos, vel = [], []
    for rec in records:
        mech = rec["cell"]["mechanics"]
        if kind == "rod":
            p = _floats(mech["pos"][0]).reshape(dim, -1).T
            v = _floats(mech["vel"][0]).reshape(dim, -1).T
        else:
            p = _floats(mech["pos"]).reshape(1, dim)
            v = _floats(mech["vel"]).reshape(1, dim) if "vel" in mech else np.zeros((1, dim))
        pos.append(p)
        vel.append(v)
    out = {"pos": np.asarray(pos).reshape(n, -1, dim), "vel": np.asarray(vel).reshape(n, -1, dim),
           "ids": np.array([crg_id(r["identifier"]) for r in records], dtype=np.uint64),
           "parent": np.array([NO_PARENT if r["parent"] is None else crg_id(r["parent"])
                               for r in records], dtype=np.uint64)}
    if kind == "rod":
        out["spring_length"] = _floats([r["cell"]["mechanics"]["spring_length"]
                                        for r in records])
    if records and all("growth_rate" in r["cell"] for r in records):
        out["growth_rate"] = _floats([r["cell"]["growth_rate"] for r in records])
    return out


def positions_of(records: List[Dict], kind: str, dim: int) -> np.ndarray:
    """Positions of loaded records, (n, vertices, dim), as the reference's plotting scripts
    read them (`cell.mechanics.pos`, rods: `pos[0]` reshaped to (dim, vertices))."""
    out = []
    for rec in records:
        p = rec["cell"]["mechanics"]["pos"]
        if kind == "rod":
            out.append(np.asarray(p[0], dtype=np.float64).reshape(dim, -1).T)
        else:
            out.append(np.asarray(p, dtype=np.float64).reshape(1, dim))
    return np.asarray(out)
