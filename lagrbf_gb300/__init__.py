"""GB300-native partition-of-unity RBF interpolation and Lagrangian advection.

A drop-in for LagRBF's interpolation/advection path: the same C-ABI (liblagrbf.so, declared in
include/lagrbf.h) and a Python mirror of lagrbfpy's classes (LagRBFCtx, LagRBFInterpolator,
AdvectionInterpolation, AdvectionAnalytical, PointContainer).  PETSc's options database is
replaced by an options store filled from the same keyword arguments.
"""
from ._lib import load_cfuncs, last_error, Stats  # noqa: F401
from .points import PointContainer, fill_datafields  # noqa: F401
from .context import LagRBFCtx, Options  # noqa: F401
from .interpolation import LagRBFInterpolator  # noqa: F401
from .advection import (Advection, AdvectionInterpolation, AdvectionAnalytical, FunctionData,  # noqa: F401
                        FunctionPointer)

__all__ = ["LagRBFCtx", "Options", "LagRBFInterpolator", "Advection", "AdvectionInterpolation",
           "AdvectionAnalytical", "PointContainer", "FunctionData", "FunctionPointer", "fill_datafields",
           "load_cfuncs", "last_error", "Stats"]
