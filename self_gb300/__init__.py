"""self_gb300: GB300-native (sm_103a) spectral-element hot path of SELF behind its type-bound API.

The compute lives in libselfgpu.so (CUDA + C++, C ABI in include/self_gpu.h).  This package is the host
mirror of the reference's Fortran types for Python drivers, tests and benchmarks.
"""
from . import _native  # noqa: F401
from .dgsem import (Advection, Context, NodalStorage_2D, QuadMesh, ShallowWater, bathymetry_gradient,  # noqa: F401
                    read_ism_mesh)
from .cgsem import CGsemElliptic_2D  # noqa: F401
from .batch import CGBatch  # noqa: F401
from . import workloads  # noqa: F401
from . import serving  # noqa: F401

__all__ = ["Context", "NodalStorage_2D", "QuadMesh", "ShallowWater", "Advection", "bathymetry_gradient", "read_ism_mesh",
           "CGsemElliptic_2D", "CGBatch", "workloads"]
