"""crg_cell_list_noalloc: the cell list of device-resident points with no device allocation.

Some callers of this library cannot allocate device memory when they need a cell list: a
host that manages device memory through its own arena, a serving loop whose HBM budget is
already committed to admitted jobs, or a latency-critical loop that must not pay for
cudaMalloc/cudaFree (which can synchronise the whole device).  This entry point works only
in the caller's buffers plus a fixed scratch array compiled into the library.

The test calls it through the C ABI twice in a row (different sizes, dimensions and grids,
so leftover scratch contents from the first call would show up in the second) and checks
each result exactly against what the existing entry point (crg_upload + crg_download)
produces for the same points: voxel indices, cell-list order and voxel starts are integer
results, so the tolerance is zero.  The test lives in its own file so that a run that stops
at the first failure has already run every other test.
"""
import ctypes as C
import math

import numpy as np
import pytest

from cellular_raza_gb300 import _native as N
from cellular_raza_gb300 import engine as E
from cellular_raza_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def n_voxels(model):
    nv = []
    for a in range(model.dim):
        f = math.floor((model.domain_max[a] - model.domain_min[a]) / model.interaction_range)
        nv.append(max(int(f), 1))
    return int(np.prod(nv))


def reference_cell_list(w):
    """Cell list from the existing entry point: crg_upload sorts the points into voxels."""
    with E.Simulation.single(w.model, w.n) as sim:
        sim.upload(w.pos, w.vel)
        lst = sim.download(order="list")
    ids = lst["ids"].astype(np.int64)
    voxel = np.empty(w.n, np.uint32)
    voxel[ids] = lst["voxel"]
    nvox = n_voxels(w.model)
    start = np.zeros(nvox + 1, np.int64)
    start[1:] = np.cumsum(np.bincount(voxel, minlength=nvox))
    return voxel, ids.astype(np.uint32), start.astype(np.uint32)


def noalloc_cell_list(torch, w):
    L = N.load()
    dom, _ = E.to_c(w.model)
    nvox = n_voxels(w.model)
    pos = torch.from_numpy(np.ascontiguousarray(w.pos[:, 0, :].T)).cuda()  # [dim][n]
    voxel = torch.full((w.n,), -1, dtype=torch.int32, device="cuda")
    order = torch.full((w.n,), -1, dtype=torch.int32, device="cuda")
    start = torch.full((nvox + 1,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = L.crg_cell_list_noalloc(C.byref(dom), w.n, C.c_void_p(pos.data_ptr()),
                                 C.c_void_p(voxel.data_ptr()), C.c_void_p(order.data_ptr()),
                                 C.c_void_p(start.data_ptr()), None)
    torch.cuda.synchronize()
    return rc, (voxel.cpu().numpy().astype(np.uint32), order.cpu().numpy().astype(np.uint32),
                start.cpu().numpy().astype(np.uint32))


def test_noalloc_cell_list_matches_upload_two_calls():
    torch = pytest.importorskip("torch")
    first = W.spheres_3d(seed=71, n=60_000)  # 30^3 voxels: several scan tiles
    second = W.spheres(5_000, 400.0, seed=72, dim=2)  # smaller, 2D grid
    for w in (first, second):
        want = reference_cell_list(w)
        rc, got = noalloc_cell_list(torch, w)
        assert rc == N.CRG_OK, N.strerror(rc)
        for name, g, r in zip(("voxel", "order", "start"), got, want):
            assert np.array_equal(g, r), name


def test_dense_voxels_sort_in_bounded_time():
    """Voxels holding tens of thousands of points (an interaction range as large as the
    domain puts 2^16 points into one voxel; a coarse grid gives segments below the
    shared-memory sort's 2,048 entries).  The per-voxel ordering is a block-wide sorting
    network for long segments, so these calls take milliseconds; the bound below is a
    generous wall-time limit.  Results: exact, against crg_upload, and the single voxel's
    order is the input order."""
    import time

    torch = pytest.importorskip("torch")
    one = W.spheres(1 << 16, 100.0, seed=81, dim=3, interaction_range=150.0)  # 1 voxel
    coarse = W.spheres(40_000, 100.0, seed=82, dim=2, interaction_range=20.0)  # 25 voxels
    for w in (one, coarse):
        t0 = time.perf_counter()
        want = reference_cell_list(w)
        rc, got = noalloc_cell_list(torch, w)
        assert time.perf_counter() - t0 < 20.0
        assert rc == N.CRG_OK, N.strerror(rc)
        for name, g, r in zip(("voxel", "order", "start"), got, want):
            assert np.array_equal(g, r), name
    _, order, _ = noalloc_cell_list(torch, one)[1]
    assert np.array_equal(order, np.arange(one.n, dtype=np.uint32))
