"""GB300-native SPH hydro package (sm_103a) for the Spheral ideal-gas path.

Modules:
  engine    -- device-resident engine over the C ABI (libsphgpu.so)
  spheral   -- Spheral-style scripting front end (SPH, TableKernel, boundaries,
               CheapSynchronousRK2Integrator, OctTreeGravity)
  problems  -- seeded synthetic problems
  build     -- in-tree nvcc build of libsphgpu.so
"""
__all__ = ["engine", "problems", "build"]
