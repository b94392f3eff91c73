"""exastamp_gb300 -- GB300-native (sm_103a) implementation of exaStamp's
per-timestep MD hot path: cell-grid neighbour list, Lennard-Jones and
eam_alloy force operators, velocity-Verlet push and thermodynamic reduction.

The compute path is libgbmd.so (CUDA, include/gbmd.h); this package holds
its build script, the ctypes binding, the host-side mirror of the reference
operators, setfl tools and seeded system generators.
"""
__all__ = ["build", "_capi", "operators", "setfl", "systems"]
