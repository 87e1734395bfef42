"""Advection classes (mirror lagrbfpy/advection.py:35-496 without the VTP/PVD file output).

``advect_step`` returns after updating ``output`` in place; file writing is left to the caller.
"""
import ctypes

import numpy as np

from ._lib import VELOCITY_FN_BATCH
from .context import LagRBFCtx


class FunctionData(ctypes.Structure):
    """Default data structure handed to analytical velocity callbacks
    (lagrbfpy/interface/function_pointer.py)."""
    _fields_ = [("time", ctypes.c_double), ("step", ctypes.c_int32)]


class FunctionPointer:
    """A Python velocity callback and its data as the C function pointer that
    lagrbf_advection_function_batch takes (lagrbfpy/interface/function_pointer.py:42-120):
    func(npoints, dim, coords, velocity, data_ptr) -> int; ``cfunc`` is the C pointer, ``data`` the
    ctypes structure handed to it."""

    def __init__(self, func, data=None):
        if data is not None and not isinstance(data, ctypes.Structure):
            raise TypeError("data must be a subclass of ctypes.Structure or FunctionData.\n"
                            "Build your own class from the helper class FunctionData, e.g.:\n"
                            "class MyFunctionData(FunctionData):\n"
                            "    _fields_ = [('param1', ctypes.c_double), ('param2', ctypes.c_int32)]\n")
        if not callable(func):
            raise TypeError("func must be a callable function with the signature "
                            "myfunction(npoints, dim, coords, velocity, data_ptr)\n")
        self.func = func
        self.data = data
        self.cfunc = VELOCITY_FN_BATCH(func)


class Advection(LagRBFCtx):
    def __init__(self, petsc_options=None, **kwargs):
        kwargs["advection"] = True
        kwargs["advection_scheme"] = kwargs.get("advection_scheme", 2)
        kwargs["advection_cfl"] = kwargs.get("advection_cfl", 0.3)
        kwargs["dt"] = kwargs.get("dt", 1e-7)
        time_start = kwargs.pop("time_start", None)
        time_end = kwargs.pop("time_end", None)
        nsteps = kwargs.pop("nsteps", None)
        time_steps = kwargs.pop("time_steps", None)
        steps = kwargs.pop("steps", None)
        super().__init__(petsc_options=petsc_options, **kwargs)
        self.start_idx = 0
        if time_steps is None:
            if time_start is None or time_end is None or nsteps is None:
                raise ValueError("time_start, time_end and nsteps must be provided if time_steps is not provided.")
            self.time_steps = np.linspace(time_start, time_end, nsteps, dtype=np.float64)
            self.nsteps = nsteps
        else:
            self.time_steps = np.asarray(time_steps, dtype=np.float64)
            self.nsteps = self.time_steps.shape[0]
        if steps is None:
            self.steps = np.arange(self.nsteps, dtype=np.int32)
        else:
            self.steps = np.asarray(steps, dtype=np.int32)
            if self.steps.shape[0] != self.nsteps:
                raise ValueError("steps must have the same length as time_steps.")

    def advect(self, *args, **kwargs):
        raise NotImplementedError("The advect method must be implemented in a subclass.")


class AdvectionAnalytical(Advection):
    def advect_step(self, step, output):
        time, time_next = self.time_steps[step], self.time_steps[step + 1]
        func_data = self.get_ref("advection_data")
        if hasattr(func_data, "time"):
            func_data.time = float(time)
        if hasattr(func_data, "step"):
            func_data.step = int(self.steps[step])
        self.advect_analytical_c(time, time_next)
        self.output(coords=output.coords, fvals=output.values, pidx=output.pidx, fieldname="velocity")

    def advect(self, points, output):
        try:
            self.get_ref("advection_fn")
        except KeyError as e:
            raise RuntimeError("No advection function has been registered.") from e
        self.fill_points(coords=points.coords, values=points.values, pidx=points.pidx)
        for step in range(self.nsteps - 1):
            self.advect_step(step, output)


class AdvectionInterpolation(Advection):
    def advect_step(self, step, get_data, data_args, output):
        """fill data -> interpolate -> output -> advect to the next time (advection.py:322-424)."""
        if "step" in data_args:
            data_args["step"] = np.int32(self.steps[step])
        if "time" in data_args:
            data_args["time"] = np.float64(self.time_steps[step])
        if "rank" in data_args:
            data_args["rank"] = np.int32(0)
        data = get_data(**data_args)
        self.fill_data(coords=data.coords, values=data.values, pidx=data.pidx)
        self.interpolate_c()
        self.output(coords=output.coords, fvals=output.values, pidx=output.pidx, fieldname="fields")
        if step == self.nsteps - 1:
            return
        self.advect_interpolate_c(self.time_steps[step], self.time_steps[step + 1])

    def advect(self, get_data, data_args, points, output):
        if not callable(get_data):
            raise ValueError("get_data must be a callable function that returns a PointContainer.")
        self.fill_points(coords=points.coords, values=points.values, pidx=points.pidx)
        for step in range(self.start_idx, self.nsteps):
            self.advect_step(step, get_data, data_args, output)
