"""acvd_gb300 -- ACVD's discrete Voronoi clustering on GB300 (sm_103a).

The minimisation runs in hand-written CUDA kernels behind the C ABI of
include/acvd_gpu.h (libacvd_gb300.so, built in-tree by acvd_gb300.build).
"""
from .engine import AcvdError, Engine, build_topology, initial_sampling, load, vertex_weights  # noqa: F401
from .remesh import (AnisotropicDiscreteRemeshing, IsotropicDiscreteRemeshing,  # noqa: F401
                     QIsotropicDiscreteRemeshing, QuadricPostPlacement, Surface)

__all__ = ["AcvdError", "Engine", "Surface", "IsotropicDiscreteRemeshing", "QIsotropicDiscreteRemeshing",
           "AnisotropicDiscreteRemeshing", "QuadricPostPlacement", "build_topology", "initial_sampling", "vertex_weights", "load"]
