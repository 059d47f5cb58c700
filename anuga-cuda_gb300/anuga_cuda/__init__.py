"""anuga_cuda -- ANUGA's explicit shallow-water evolve step on one GB300.

Drop-in for the reference's ``anuga_cuda.GPU_domain`` path: a domain object
with ANUGA's method names whose per-step work runs as hand-written sm_103a
CUDA kernels in libswgpu.so (C ABI in include/swgpu.h), called through
ctypes.  There is no CPU implementation in this package.
"""
from ._build import build, library_path
from .boundaries import (Dirichlet_boundary, Inflow_hydrograph_boundary, Reflective_boundary,
                         Time_stage_fourier_boundary, Time_stage_sine_boundary,
                         Transmissive_boundary, Transmissive_stage_zero_momentum_boundary)
from .config import DEFAULT, Parameters
from .gpu_domain import GPU_domain, Quantity
from .io import SWWWriter, create_domain_from_file, read_sww, read_tsh
from .mesh import Mesh, morton_order, rectangular_cross

CUDA_advanced_domain = GPU_domain

__all__ = [
    "GPU_domain", "CUDA_advanced_domain", "Quantity", "Mesh", "rectangular_cross",
    "morton_order", "Parameters", "DEFAULT", "Reflective_boundary", "Dirichlet_boundary",
    "Time_stage_sine_boundary", "Time_stage_fourier_boundary", "Transmissive_boundary",
    "Transmissive_stage_zero_momentum_boundary", "Inflow_hydrograph_boundary", "build",
    "library_path", "read_tsh", "create_domain_from_file", "SWWWriter", "read_sww",
]
