"""LagRBFCtx: Python mirror of lagrbfpy.interface.context.LagRBFCtx (context.py:39-681).

The keyword arguments, their defaults and the options they set are those of the reference
(context.py:113-201); they are written into the library's options store (which stands in for
PETSc's options database) before ``lagrbf_create()`` reads them.  Two GPU-only keywords are
added: ``eval_precision`` ("fp64" plain path, "fp32" FP32 evaluation) and ``use_cuda_graph``.
"""
import ctypes
import os

import numpy as np

from ._lib import load_cfuncs, last_error, Stats, STEP_REDUCE, VELOCITY_FN, VELOCITY_FN_BATCH


def _fmt(v):
    if isinstance(v, (bool, np.bool_)):
        return "true" if v else "false"
    if isinstance(v, (list, tuple, np.ndarray)):
        return ",".join(_fmt(x) for x in np.asarray(v).ravel().tolist())
    if isinstance(v, float):
        return repr(v)
    return str(v)


class Options(dict):
    """Dict of option values (keys without the leading dash), pushed to the options store."""

    def getInt(self, k, default):
        return int(self.get(k, default))

    def getReal(self, k, default):
        return float(self.get(k, default))

    def getBool(self, k, default):
        v = self.get(k, default)
        return v if isinstance(v, bool) else str(v).lower() in ("1", "true", "yes")

    def getString(self, k, default):
        return str(self.get(k, default))

    def getRealArray(self, k, default):
        return np.asarray(self.get(k, default), dtype=np.float64)

    def getIntArray(self, k, default):
        return np.asarray(self.get(k, default), dtype=np.int32)

    def push(self):
        cf = load_cfuncs()
        for k, v in self.items():
            cf["lagrbf_options_set_value"](k.encode(), _fmt(v).encode())


class LagRBFCtx:
    def __init__(self, petsc_options=None, **kwargs):
        self.data_filled = False
        self.interp_filled = False
        self.PetscReal = np.dtype(np.float64)
        self.PetscRealCtype = ctypes.c_double
        self.options = Options(petsc_options or {})
        o = self.options
        self.output_path = kwargs.get("output_path", o.getString("output_path", "output"))
        self.dim = kwargs.get("dim", o.getInt("pu_mesh_dim", 3))
        o["pu_mesh_dim"] = self.dim
        o["pu_mesh_O"] = kwargs.get("minCoords", o.getRealArray("pu_mesh_O", np.zeros(self.dim)))
        o["pu_mesh_L"] = kwargs.get("maxCoords", o.getRealArray("pu_mesh_L", np.ones(self.dim)))
        o["pu_mesh_n"] = kwargs.get("npartitions", o.getIntArray("pu_mesh_n", np.full(self.dim, 4, dtype=np.int32)))
        o["n_interpolation_fields"] = kwargs.get("nfields", o.getInt("n_interpolation_fields", 0))
        o["pu_mesh_overlap"] = kwargs.get("overlap", o.getReal("pu_mesh_overlap", 1.0))
        o["pu_mesh_shape_factor"] = kwargs.get("shape_factor", o.getReal("pu_mesh_shape_factor", 1.0))
        o["kernel_type"] = kwargs.get("kernel", o.getInt("kernel_type", 2))
        o["solve_method"] = kwargs.get("solve_method", o.getInt("solve_method", 2))
        o["partition_pc_type"] = kwargs.get("partition_pc_type", o.getString("partition_pc_type", "cholesky"))
        o["partition_ksp_type"] = kwargs.get("partition_ksp_type", o.getString("partition_ksp_type", "preonly"))
        o["partition_ksp_reuse_preconditioner"] = kwargs.get(
            "partition_ksp_reuse_preconditioner", o.getBool("partition_ksp_reuse_preconditioner", True))
        o["partition_pc_factor_shift_type"] = kwargs.get(
            "partition_pc_factor_shift_type", o.getString("partition_pc_factor_shift_type", "positive_definite"))
        o["advection"] = kwargs.get("advection", o.getBool("advection", False))
        o["advection_scheme"] = kwargs.get("advection_scheme", o.getInt("advection_scheme", 2))
        o["cfl_fac"] = kwargs.get("advection_cfl", o.getReal("cfl_fac", 0.3))
        o["dt"] = kwargs.get("dt", o.getReal("dt", 1e-4))
        o["rmin"] = kwargs.get("rmin", o.getReal("rmin", 0.0))
        o["rmax"] = kwargs.get("rmax", o.getReal("rmax", 1e132))
        o["eval_precision"] = kwargs.get("eval_precision", o.getString("eval_precision", "fp64"))
        o["use_cuda_graph"] = kwargs.get("use_cuda_graph", o.getBool("use_cuda_graph", True))
        o["device_loop"] = kwargs.get("device_loop", o.getBool("device_loop", True))
        o["output_direct"] = kwargs.get("output_direct", o.getBool("output_direct", True))
        if "cuda_device" in kwargs or "cuda_device" in o:
            o["cuda_device"] = int(kwargs.get("cuda_device", o.get("cuda_device", 0)))
        self.nfields = int(o["n_interpolation_fields"])
        self._cf = load_cfuncs()
        self._cf["lagrbf_options_clear"]()
        o.push()
        self.ctx = self._cf["lagrbf_create"]()
        if not self.ctx:
            raise RuntimeError("Failed to create LagRBF context: " + last_error())
        self.refs = {}

    # ------------------------------------------------------------------ reference API
    def get_ctx(self):
        if self.ctx is None:
            raise RuntimeError("LagRBF context has not been created or has been destroyed.")
        return self.ctx

    def get_stored_refs(self):
        return self.refs

    def get_ref(self, key):
        ref = self.refs.get(key, None)
        if ref is None:
            raise KeyError(f"No reference found for key '{key}'.")
        return ref

    def store_ref(self, **objs):
        self.refs.update(objs)

    def __index__(self):
        """The C context pointer (context.py:262-263 of lagrbfpy)."""
        return self.ctx

    def __bool__(self):
        return self.ctx is not None

    def __del__(self):
        if getattr(self, "ctx", None) is not None:
            self._cf["lagrbf_destroy"](self.ctx)
            self.ctx = None

    def close(self):
        self.__del__()

    def _begin_c(self, array, dtype):
        if array is None:
            raise ValueError("Input array cannot be None.\nConsider using an empty array instead: np.empty((0, dim))\n")
        a = np.ascontiguousarray(array, dtype=dtype)
        return a.reshape((a.size,))

    def _end_c(self, array, bs=1):
        """A flat C array back to rows of bs values (context.py:285-287 of lagrbfpy)."""
        return array.reshape((-1, bs), order="C")

    def _check(self, ierr, name):
        if ierr != 0:
            raise RuntimeError(f"{name} failed with error code {ierr}: {last_error()}")

    def fill_swarm(self, coords, values=None, pidx=None, is_data=False):
        if coords is None:
            coords = np.empty((0, self.dim), dtype=self.PetscReal)
        npoints = coords.shape[0]
        pcoords = self._begin_c(coords, self.PetscReal)
        pvals = None if values is None else self._begin_c(values, self.PetscReal)
        ppidx = None if pidx is None else self._begin_c(pidx, np.int64)
        ierr = self._cf["lagrbf_fill_swarm"](self.ctx, is_data, npoints, pcoords, pvals, ppidx)
        self._check(ierr, "lagrbf_fill_swarm")

    def fill_data(self, coords, values, pidx=None):
        self.fill_swarm(coords=coords, values=values, pidx=pidx, is_data=True)
        self.data_filled = True

    def fill_points(self, coords, values=None, pidx=None):
        self.fill_swarm(coords=coords, values=values, pidx=pidx, is_data=False)
        self.interp_filled = True

    def output(self, coords=None, fvals=None, pidx=None, fieldname="fields", is_data=False):
        """Fill the caller's arrays in place (by pid - 1), like context.py:375-455."""
        npoints = 0
        if coords is None and fvals is None and pidx is None:
            raise ValueError("At least one of coords, fvals, or pidx must be provided.")
        for a in (coords, fvals, pidx):
            if a is not None:
                if not a.flags.c_contiguous:
                    raise ValueError("output arrays must be C-contiguous")
                npoints = a.shape[0]
        if npoints == 0:
            raise ValueError("Number of points must be greater than zero.")
        c = None if coords is None else coords.reshape(-1)
        f = None if fvals is None else fvals.reshape(-1)
        ierr = self._cf["lagrbf_output"](self.ctx, is_data, npoints, c, f, pidx, fieldname.encode("utf-8"))
        self._check(ierr, "lagrbf_output")

    def save(self, fname, output_points, fieldname="fields", is_data=False):
        """Write coordinates, values and pids to a NumPy .npz file (VTP writing is not part of this
        package)."""
        self.output(coords=output_points.coords, fvals=output_points.values, pidx=output_points.pidx,
                    fieldname=fieldname, is_data=is_data)
        np.savez(fname, coords=output_points.coords, values=output_points.values, pidx=output_points.pidx)

    def interpolate_c(self):
        if not self.data_filled:
            raise RuntimeError("Data have not been provided, use fill_data() to provide data points")
        if not self.interp_filled:
            raise RuntimeError("Interpolation swarm has not been provided, use fill_points() to provide the points on which to interpolate")
        self._check(self._cf["lagrbf_interpolation"](self.ctx), "lagrbf_interpolation")

    def reset_coefficients(self):
        self._check(self._cf["lagrbf_reset_coefficients"](self.ctx), "lagrbf_reset_coefficients")

    def set_advection_function(self, func, func_data=None):
        if not callable(func):
            raise ValueError("Provided advection function is not callable.")
        if not isinstance(func, VELOCITY_FN_BATCH):
            func = VELOCITY_FN_BATCH(func)
        from .advection import FunctionData
        if func_data is None:
            func_data = FunctionData(time=0.0, step=0)
        elif not isinstance(func_data, ctypes.Structure):
            raise ValueError("Provided advection function data is not a ctypes.Structure.")
        self.store_ref(advection_fn=func, advection_data=func_data)
        ierr = self._cf["lagrbf_advection_function_batch"](self.ctx, func, ctypes.cast(ctypes.pointer(func_data), ctypes.c_void_p))
        self._check(ierr, "lagrbf_advection_function_batch")

    def advect_analytical_c(self, time_start, time_end):
        if not self.interp_filled:
            raise RuntimeError("Swarm to advect has not been provided, use fill_swarm() to provide the points to advect")
        self._check(self._cf["lagrbf_avect_analytical"](self.ctx, float(time_start), float(time_end)), "lagrbf_advect")

    def advect_interpolate_c(self, time_start, time_end):
        if not self.data_filled:
            raise RuntimeError("Data have not been provided, use fill_swarm() to provide data points")
        if not self.interp_filled:
            raise RuntimeError("Swarm to advect has not been provided, use fill_swarm() to provide the points to advect")
        self._check(self._cf["lagrbf_avect_interpolate"](self.ctx, float(time_start), float(time_end)), "lagrbf_advect")
        # the reference clears the data swarm at the end of the advection loop (time_loop.c:97-98)
        self.data_filled = False

    # ------------------------------------------------------------------ GPU extension
    def stats(self):
        s = Stats()
        self._check(self._cf["lagrbf_gpu_get_stats"](self.ctx, ctypes.byref(s)), "lagrbf_gpu_get_stats")
        return s.as_dict()

    def reset_stats(self):
        self._check(self._cf["lagrbf_gpu_reset_stats"](self.ctx), "lagrbf_gpu_reset_stats")

    def set_profiling(self, on):
        self._check(self._cf["lagrbf_gpu_set_profiling"](self.ctx, int(bool(on))), "lagrbf_gpu_set_profiling")

    def share_dataset(self, owner):
        """Use owner's resident dataset in place, read-only (lagrbf_gpu_share_dataset); owner needs
        setup_all_patches and a completed interpolation, and must outlive this context."""
        self._check(self._cf["lagrbf_gpu_share_dataset"](self.ctx, owner.ctx), "lagrbf_gpu_share_dataset")
        self._shared_owner = owner
        self.data_filled = True

    def set_step_reduce(self, fn):
        """Coupling of sharded runs (lagrbf_gpu_set_step_reduce): fn(vals) replaces the numpy array
        vals by its element-wise maximum over the ranks; None removes it."""
        if fn is None:
            self._step_reduce = None
            self._check(self._cf["lagrbf_gpu_set_step_reduce"](self.ctx, STEP_REDUCE(), None),
                        "lagrbf_gpu_set_step_reduce")
            return

        def cb(ptr, n, user):
            try:
                fn(np.ctypeslib.as_array(ptr, shape=(n,)))
                return 0
            except Exception:  # an error code, never an exception through the C frame
                return 1
        self._step_reduce = STEP_REDUCE(cb)
        self._check(self._cf["lagrbf_gpu_set_step_reduce"](self.ctx, self._step_reduce, None),
                    "lagrbf_gpu_set_step_reduce")

    def set_condition_estimates(self, on):
        """Per-patch 1-norm condition estimates at every factorisation (lagrbf_gpu_set_condition_estimates)."""
        self._check(self._cf["lagrbf_gpu_set_condition_estimates"](self.ctx, int(bool(on))),
                    "lagrbf_gpu_set_condition_estimates")

    def condition(self):
        """(kappa by patch node, {"max", "median", "count"}) of the estimates made so far."""
        ints, _ = self.geometry()
        k = np.zeros(int(ints[4]))
        sm = np.zeros(3)
        self._check(self._cf["lagrbf_gpu_get_condition"](self.ctx, k, sm), "lagrbf_gpu_get_condition")
        return k, {"max": float(sm[0]), "median": float(sm[1]), "count": int(sm[2])}

    def test_eval_wait(self, poll_limit, withhold_copies=False):
        """Test hook of the evaluation kernel's bounded waits (lagrbf_gpu_test_eval_wait)."""
        self._check(self._cf["lagrbf_gpu_test_eval_wait"](self.ctx, int(poll_limit), int(bool(withhold_copies))),
                    "lagrbf_gpu_test_eval_wait")

    def advect_resident(self, time_start, time_end):
        """The advection loop of advect_interpolate_c without its end-of-call reset (data, binning
        and patch set-ups stay resident)."""
        self._check(self._cf["lagrbf_gpu_advect_resident"](self.ctx, float(time_start), float(time_end)),
                    "lagrbf_gpu_advect_resident")

    def fill_from_files(self, coords_file, field_files=(), pid_file=None, is_data=False):
        """lagrbf_fill_swarm_from_files: a swarm from PETSc binary files (coordinates, fields stacked
        in file order, optional pid index set)."""
        arr = (ctypes.c_char_p * max(len(field_files), 1))(*[str(f).encode() for f in field_files])
        rc = self._cf["lagrbf_fill_swarm_from_files"](self.ctx, bool(is_data), str(coords_file).encode(), arr,
                                                      len(field_files),
                                                      None if pid_file is None else str(pid_file).encode())
        self._check(rc, "lagrbf_fill_swarm_from_files")
        if is_data:
            self.data_filled = True
        else:
            self.interp_filled = True

    def output_files(self, prefix, npoints, fieldname="fields", is_data=False):
        """lagrbf_output_files: <prefix>_coor.pbvec, <prefix>_<fieldname>.pbvec, <prefix>_pid.pbis."""
        rc = self._cf["lagrbf_output_files"](self.ctx, bool(is_data), int(npoints), str(prefix).encode(),
                                             fieldname.encode())
        self._check(rc, "lagrbf_output_files")

    VFIELD_NONE, VFIELD_ROTATION, VFIELD_CELLULAR, VFIELD_ABC, VFIELD_FOURIER = 0, 1, 2, 3, 4

    def set_velocity_field(self, kind, params=None):
        """Device-side analytical velocity for advect_analytical_c (lagrbf_gpu_set_velocity_field):
        ROTATION (omega, cx, cy), CELLULAR (a, k), ABC (A, B, C, scale), FOURIER (n, then n rows of
        k1, k2, k3, phase, a1, a2, a3); kind 0 removes it."""
        p = None if params is None else np.ascontiguousarray(np.ravel(params), dtype=np.float64)
        n = 0 if p is None else int(p.size)
        self._check(self._cf["lagrbf_gpu_set_velocity_field"](self.ctx, int(kind), p, n), "lagrbf_gpu_set_velocity_field")

    def set_precision(self, fp32):
        self._check(self._cf["lagrbf_gpu_set_precision"](self.ctx, int(bool(fp32))), "lagrbf_gpu_set_precision")

    def synchronize(self):
        self._check(self._cf["lagrbf_gpu_synchronize"](self.ctx), "lagrbf_gpu_synchronize")

    def cellids(self, is_data, n):
        out = np.empty(n, dtype=np.int32)
        self._check(self._cf["lagrbf_gpu_get_cellids"](self.ctx, is_data, out), "lagrbf_gpu_get_cellids")
        return out

    def geometry(self):
        ints = np.zeros(7, dtype=np.int32)
        reals = np.zeros(2)
        self._check(self._cf["lagrbf_gpu_get_geometry"](self.ctx, ints, reals), "lagrbf_gpu_get_geometry")
        return ints, reals

    def patch_csr(self):
        ints, _ = self.geometry()
        nn = int(ints[4])
        total = self._cf["lagrbf_gpu_get_patch_csr"](self.ctx, None, None)
        start = np.zeros(nn + 1, dtype=np.int32)
        pts = np.zeros(max(total, 1), dtype=np.int32)
        self._cf["lagrbf_gpu_get_patch_csr"](self.ctx, start, pts)
        return start, pts[:total]

    def block_csr(self):
        ints, _ = self.geometry()
        nc = int(ints[5])
        total = self._cf["lagrbf_gpu_get_block_csr"](self.ctx, None, None)
        start = np.zeros(nc + 1, dtype=np.int32)
        pts = np.zeros(max(total, 1), dtype=np.int32)
        self._cf["lagrbf_gpu_get_block_csr"](self.ctx, start, pts)
        return start, pts[:total]
