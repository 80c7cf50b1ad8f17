"""GB300 FEM time-stepping library: Python front end of libfea_gb300.so.

`binding.CUDASolver` is the reference's Solver interface over the C ABI of
include/fea_gpu.h, `binding.BatchSolver` steps many Gray-Scott instances
together; `meshgen` makes the synthetic meshes of the workloads.
"""
from . import meshgen  # noqa: F401
from .binding import (  # noqa: F401
    ADVECTION, ADVECTION_DIFFUSION, CG_VARIANTS, DEFERRED_VARIANTS, DIRICHLET, FP32, FP64, HEAT, MASS, NEUMANN,
    REACTION_DIFFUSION, STIFFNESS, WAVE, BatchSolver, CUDASolver, FeaError, Params, default_params, load,
    triangulate_pslg,
)
