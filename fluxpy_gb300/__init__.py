"""fluxpy_gb300 — the radiosity / thermal hot path of fluxpy on one GB300.

Modules mirror the reference package ``flux``:
  shape                    triangle-mesh shape models, LBVH ray queries
  form_factors             form-factor assembly (fused pair kernel -> CSR)
  compressed_form_factors  hierarchical compressed operator (ACA) and its matvec
  solve                    radiosity solves (reference Jacobi / CG; batched BF16)
  model                    steady-state temperature, time-dependent model
  thermal                  per-facet 1-D conduction (Crank-Nicolson)
  adjoint                  hand-written adjoints of the solve and the conduction
                           step (torch.autograd.Function), coupled misfit gradient
  batch                    uneven batches of independent meshes in shared
                           launches; batched thermal model with CUDA graphs
  terrain                  synthetic meshes used by the benchmarks
All compute runs in libfluxgb.so (hand-written sm_103a CUDA, C ABI in
include/fluxgb.h); there is no CPU fallback.
"""
__version__ = "0.1.0"
