"""GB300-native spectral-element time step of SEM2DPACK.

The compute path is the CUDA library ``_lib/libsem2d_gb300.so`` (sm_103a)
behind the C-ABI of include/sem2d_gpu.h; this package holds its Python
binding, the Par.inp-shaped deck and the host problem builder binding.
"""
from .abi import (FRICTION_RSF, FRICTION_SWF, PRECISION_FP64, PRECISION_MIXED,  # noqa: F401
                  TIME_LEAPFROG, TIME_NEWMARK)
from .api import BatchSolver, Grid, Problem, Sem2dError, Solver  # noqa: F401
from .deck import Fault, Material, ParDeck, Receivers, Sources, Time  # noqa: F401

__all__ = ["Grid", "Problem", "Solver", "BatchSolver", "Sem2dError", "ParDeck", "Material", "Fault", "Time",
           "Sources", "Receivers"]
