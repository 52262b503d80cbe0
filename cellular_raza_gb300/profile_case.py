"""Runs a named workload for a few steps through the C ABI (for profilers such as ncu).

    python -m cellular_raza_gb300.profile_case --workload rods_2d --steps 10

Uploads the seeded workload, runs `--steps` chili steps with direct launches (no CUDA
graphs, so every kernel is a separate launch) and prints the elapsed wall time.
"""
from __future__ import annotations

import argparse
import time

from . import _native as N
from . import engine as E
from . import workloads as W


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--workload", default="rods_2d",
                   choices=["rods_2d", "spheres_3d", "spheres_3d_large"])
    p.add_argument("--n", type=int, default=0, help="agents (0: the workload's size)")
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--n-subdomains", type=int, default=16)
    p.add_argument("--precision", default=None, choices=[None, "f64", "mixed"])
    p.add_argument("--variant", type=int, default=0, help="CRG_OPT_KERNEL_VARIANT")
    a = p.parse_args()
    kw = {"n_subdomains": a.n_subdomains}
    if a.n:
        kw["n"] = a.n
    if a.precision:
        kw["precision"] = a.precision
    w = getattr(W, a.workload)(seed=2024, **kw)
    with E.Simulation.single(w.model, w.n) as sim:
        sim.set_option(N.OPT_GRAPH_CHUNK, 0)
        sim.set_option(N.OPT_KERNEL_VARIANT, a.variant)
        sim.upload(w.pos, w.vel)
        t = time.perf_counter()
        sim.step(a.steps)
        sim.download()
        print(f"{w.name}: {w.n} agents x {a.steps} steps in {time.perf_counter() - t:.3f} s")


if __name__ == "__main__":
    main()
