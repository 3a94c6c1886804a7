"""GB300-native SPH impact solver: the step loop of the reference's hydrocode
as hand-written sm_103a CUDA kernels behind a C ABI (include/deorbit_sph.h).

Modules: `sph` (ctypes front end, `System` / `Context`), `ic` (seeded
synthetic workloads), `build` (compiles the CUDA library in-tree).
"""
__all__ = ["sph", "ic", "build"]
