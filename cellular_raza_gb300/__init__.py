"""GB300-native backend for cellular_raza's mechanics/interaction step.

The device path lives in libcrg.so (CUDA for sm_103a behind the C ABI in include/crg.h);
``engine.Simulation`` drives it, ``chili`` mirrors the reference-facing types
(CartesianCuboid, NewtonDamped, MorsePotential, RodMechanics, RodInteraction,
run_simulation) and ``workloads`` generates the seeded benchmark inputs.
"""
__all__ = ["engine", "workloads", "chili", "build"]
