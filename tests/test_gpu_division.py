"""The FP64 rod pass kernel divides t = dot / |ab|^2 from the segment's correctly rounded
reciprocal with FMA residual corrections (div_rn_recip).  It must give the IEEE quotient bit
for bit: checked on a billion generated operand pairs (rod-like values, random exponents
across the fast path's bounds, quotients next to rounding midpoints, all-ones and
power-of-two divisors), and through the kernels, which must agree bit for bit with the
rod-level kernel that divides with the IEEE division."""
import ctypes as C

import numpy as np
import pytest

from cellular_raza_gb300 import _native as N
from cellular_raza_gb300 import engine as E
from cellular_raza_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2])
def test_division_matches_ieee(gpu, seed):
    n = 1 << 29
    bad, fast = C.c_int64(-1), C.c_int64(-1)
    N.check(gpu.crg_check_division(n, seed, C.byref(bad), C.byref(fast)), "crg_check_division")
    assert bad.value == 0
    assert fast.value > n // 2  # most pairs take the reciprocal path


@pytest.mark.parametrize("dim,n_sub", [(2, 1), (2, 16), (3, 4)])
def test_pass_list_equals_rod_kernel(gpu, dim, n_sub):
    """Default pass list (reciprocal division) against the rod-level kernel (IEEE division),
    60 steps of a dense rod system: identical bits."""
    w = W.rods(n=4000, side=420.0 if dim == 2 else 90.0, seed=31 + dim, dim=dim,
               n_subdomains=n_sub)
    out = []
    for variant in (0, 1):
        with E.Simulation.single(w.model, w.n) as sim:
            sim.set_option(N.OPT_KERNEL_VARIANT, variant)
            sim.upload(w.pos, w.vel)
            sim.step(60)
            out.append(sim.download(order="id"))
    assert np.array_equal(out[0]["pos"], out[1]["pos"])
    assert np.array_equal(out[0]["vel"], out[1]["vel"])


@pytest.mark.parametrize("precision,dim", [("f64", 2), ("mixed", 2), ("f64", 3)])
def test_warp_walk_equals_thread_walk(gpu, precision, dim):
    """The pass list walked with a warp per rod (CRG_OPT_BLOCK 32, the default for small
    systems) and with a thread per rod (128): identical bits after 60 steps, 4 subdomains."""
    w = W.rods(n=3000, side=360.0 if dim == 2 else 80.0, seed=41 + dim, dim=dim,
               n_subdomains=4, precision=precision)
    out = []
    for block in (32, 128):
        out.append(E.run(w, 60, options={N.OPT_BLOCK: block}))
    for k in ("pos", "vel", "voxel"):
        assert np.array_equal(out[0][k], out[1][k]), k


def test_warp_walk_colony(gpu):
    """A dividing colony (agent count changing every few steps) walked both ways."""
    w = W.rod_colony(n=150, seed=9, n_subdomains=2)
    a = E.run(w, 150, order="list", options={N.OPT_BLOCK: 32})
    b = E.run(w, 150, order="list", options={N.OPT_BLOCK: 128})
    for k in ("ids", "parent", "pos", "vel", "spring_length"):
        assert np.array_equal(a[k], b[k]), k
