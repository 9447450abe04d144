"""GB300-native exterior Helmholtz BEM backend for Boundary Lab.

A drop-in for the reference's ``beat_cuda`` solver on exterior Burton-Miller
solves: hand-written sm_103a CUDA kernels (operator assembly, dense LU with FP64
iterative refinement, field evaluation) behind a C ABI (include/gb300_bem.h),
driven by a Python host layer that mirrors the reference's solver-backend
interface and NDJSON event contract.

The directory name is not a Python identifier; load it with
``importlib.import_module("boundary-lab_gb300")`` after putting the repository
root on ``sys.path``.  Submodules import lazily so that CPU-only uses (mesh
generation, request parsing) never need CUDA.
"""

__all__ = ["meshes", "native", "build", "engine", "request", "backend", "serving"]
