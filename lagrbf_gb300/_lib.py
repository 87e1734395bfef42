"""ctypes registration of liblagrbf.so (mirrors lagrbfpy/interface/register_cfunc.py:44-197).

PetscInt is int32, PetscReal float64 and PetscInt64 int64, as in the reference's 32-bit-index
PETSc build.  The library must have been built (``python -m lagrbf_gb300.build`` or
``__graft_entry__.build()``); importing without it raises ImportError -- there is no CPU fallback.
"""
import ctypes
import os

import numpy as np
from numpy.ctypeslib import ndpointer

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "liblagrbf.so")

PetscInt = ctypes.c_int32
PetscReal = ctypes.c_double
PetscInt64 = np.dtype(np.int64)
REAL = np.dtype(np.float64)


def wrap_ndpointer(dtype=None, ndim=None, shape=None, flags=None):
    """ndpointer that also accepts None (a NULL pointer), as register_cfunc.py:34-42."""
    base = ndpointer(dtype=dtype, ndim=ndim, shape=shape, flags=flags)

    class WrappedPointer(base):
        @classmethod
        def from_param(cls, obj):
            if obj is None:
                return obj
            return super().from_param(obj)

    return WrappedPointer


VELOCITY_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(PetscReal), ctypes.POINTER(PetscReal), ctypes.c_void_p)
VELOCITY_FN_BATCH = ctypes.CFUNCTYPE(ctypes.c_int, PetscInt, PetscInt, ctypes.POINTER(PetscReal),
                                     ctypes.POINTER(PetscReal), ctypes.c_void_p)


# int fn(double *vals, int32 n, void *user): element-wise max of vals over the ranks, in place
STEP_REDUCE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int32, ctypes.c_void_p)


class Stats(ctypes.Structure):
    _fields_ = [
        ("launches", ctypes.c_int64), ("eval_launches", ctypes.c_int64), ("eval_flops", ctypes.c_double),
        ("eval_bytes", ctypes.c_double), ("eval_ms", ctypes.c_double), ("particle_steps", ctypes.c_int64),
        ("steps", ctypes.c_int64), ("patches_factored", ctypes.c_int64), ("factor_ms", ctypes.c_double),
        ("factor_flops", ctypes.c_double), ("np_alive", ctypes.c_int32), ("nd", ctypes.c_int32),
        ("max_patch", ctypes.c_int32), ("npatch_setup", ctypes.c_int32), ("dt", ctypes.c_double),
        ("chunk_cap", ctypes.c_int32), ("records", ctypes.c_int32), ("kappa_max", ctypes.c_double),
        ("kappa_median", ctypes.c_double), ("device_loop", ctypes.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def load_shared_lib(path=LIBPATH):
    if not os.path.exists(path):
        raise ImportError("liblagrbf.so is not built (run __graft_entry__.build()); no CPU fallback exists")
    return ctypes.CDLL(path)


def register_functions(clib):
    real_p = ndpointer(REAL, flags="C_CONTIGUOUS")
    real_pn = wrap_ndpointer(REAL, flags="C_CONTIGUOUS")
    i64_pn = wrap_ndpointer(PetscInt64, flags="C_CONTIGUOUS")
    f = {}

    def reg(name, restype, argtypes, key=None):
        fn = getattr(clib, name)
        fn.restype = restype
        fn.argtypes = argtypes
        f[key or name] = fn

    reg("lagrbf_interpolate_driver", None,
        [PetscInt, real_p, real_p, PetscInt, real_p, real_p, PetscInt, ctypes.c_char_p])
    reg("lagrbf_create", ctypes.c_void_p, [])
    reg("lagrbf_destroy", None, [ctypes.c_void_p])
    reg("lagrbf_fill_swarm", ctypes.c_int, [ctypes.c_void_p, ctypes.c_bool, PetscInt, real_p, real_pn, i64_pn])
    reg("lagrbf_interpolation", ctypes.c_int, [ctypes.c_void_p])
    reg("lagrbf_output", ctypes.c_int,
        [ctypes.c_void_p, ctypes.c_bool, PetscInt, real_pn, real_pn, i64_pn, ctypes.c_char_p])
    reg("lagrbf_avect_analytical", ctypes.c_int, [ctypes.c_void_p, PetscReal, PetscReal])
    reg("lagrbf_advection_function", ctypes.c_int, [ctypes.c_void_p, VELOCITY_FN, ctypes.c_void_p])
    reg("lagrbf_advection_function_batch", ctypes.c_int, [ctypes.c_void_p, VELOCITY_FN_BATCH, ctypes.c_void_p])
    # registered under the reference's key (register_cfunc.py:178-185)
    reg("lagrbf_advect_interpolate", ctypes.c_int, [ctypes.c_void_p, PetscReal, PetscReal],
        key="lagrbf_avect_interpolate")
    reg("lagrbf_reset_coefficients", ctypes.c_int, [ctypes.c_void_p])
    # options store
    reg("lagrbf_options_set_value", ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p])
    reg("lagrbf_options_clear", ctypes.c_int, [])
    reg("lagrbf_options_insert_file", ctypes.c_int, [ctypes.c_char_p])
    reg("lagrbf_options_get_value", ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32])
    # GPU extension
    reg("lagrbf_gpu_set_profiling", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int])
    reg("lagrbf_gpu_share_dataset", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p])
    reg("lagrbf_gpu_set_step_reduce", ctypes.c_int, [ctypes.c_void_p, STEP_REDUCE, ctypes.c_void_p])
    reg("lagrbf_gpu_set_condition_estimates", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int])
    reg("lagrbf_gpu_get_condition", ctypes.c_int, [ctypes.c_void_p, real_pn, real_pn])
    reg("lagrbf_gpu_test_eval_wait", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32])
    reg("lagrbf_gpu_advect_resident", ctypes.c_int, [ctypes.c_void_p, PetscReal, PetscReal])
    reg("lagrbf_gpu_set_precision", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int])
    reg("lagrbf_gpu_set_velocity_field", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, real_pn, ctypes.c_int32])
    reg("lagrbf_fill_swarm_from_files", ctypes.c_int, [ctypes.c_void_p, ctypes.c_bool, ctypes.c_char_p,
                                                       ctypes.POINTER(ctypes.c_char_p), ctypes.c_int32,
                                                       ctypes.c_char_p])
    reg("lagrbf_output_files", ctypes.c_int, [ctypes.c_void_p, ctypes.c_bool, ctypes.c_int32, ctypes.c_char_p,
                                              ctypes.c_char_p])
    reg("lagrbf_gpu_fp32_peak_tflops", ctypes.c_double, [])
    reg("lagrbf_gpu_fp64_peak_tflops", ctypes.c_double, [])
    reg("lagrbf_gpu_get_stats", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats)])
    reg("lagrbf_gpu_reset_stats", ctypes.c_int, [ctypes.c_void_p])
    reg("lagrbf_gpu_synchronize", ctypes.c_int, [ctypes.c_void_p])
    reg("lagrbf_gpu_stream", ctypes.c_void_p, [ctypes.c_void_p])
    reg("lagrbf_gpu_last_error", ctypes.c_char_p, [])
    i32_p = wrap_ndpointer(np.int32, flags="C_CONTIGUOUS")
    reg("lagrbf_gpu_get_cellids", ctypes.c_int, [ctypes.c_void_p, ctypes.c_bool, i32_p])
    reg("lagrbf_gpu_get_patch_csr", ctypes.c_int64, [ctypes.c_void_p, i32_p, i32_p])
    reg("lagrbf_gpu_get_block_csr", ctypes.c_int64, [ctypes.c_void_p, i32_p, i32_p])
    reg("lagrbf_gpu_get_geometry", ctypes.c_int,
        [ctypes.c_void_p, ndpointer(np.int32, flags="C_CONTIGUOUS"), real_p])
    return f


_clib = None
_cfuncs = None


def load_cfuncs():
    global _clib, _cfuncs
    if _cfuncs is None:
        _clib = load_shared_lib()
        _cfuncs = register_functions(_clib)
    return _cfuncs


def last_error():
    msg = load_cfuncs()["lagrbf_gpu_last_error"]()
    return msg.decode() if msg else ""
