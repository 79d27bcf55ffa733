"""GB300 (sm_103a) energy-representation hot path of ERmod behind a C ABI.

Modules
  _lib       ctypes binding of libermod_gb300.so (include/ermod_gpu.h)
  build      in-tree nvcc build of the library
  engproc    EnergyRepresentation: the engconst/update_histogram protocol on the GPU
  setconf    set-up semantics (LJ tables, charge scaling, energy coordinate, screening)
  insertion  reference-solvent placements (insertion.F90 semantics)
  synth      seeded synthetic workloads
  roofline   algorithmic bytes of the per-placement path
"""
