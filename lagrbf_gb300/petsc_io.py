"""PETSc binary Vec / IS files without PETSc (lagrbf_petsc_* of liblagrbf.so).

Format: big-endian, 32-bit PetscInt; Vec = class id 1211214, n, n doubles; IS = class id 1211218,
n, n int32.  A Vec's block size lives in "<path>.info" ("-vecload_block_size <bs>").  These are
the files LagRBF's loaders and writers exchange (src/io_utils.c:211-238,
src/readers/petsc_loader/petsc_loader.c:38-99, src/swarm/swarm_output.c:87-166).
"""
import ctypes

import numpy as np

from ._lib import load_shared_lib, last_error

_lib = None


def _L():
    global _lib
    if _lib is None:
        L = load_shared_lib()
        L.lagrbf_petsc_vec_write.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32]
        L.lagrbf_petsc_vec_read.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64,
                                           ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32)]
        L.lagrbf_petsc_is_write.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64]
        L.lagrbf_petsc_is_read.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.POINTER(ctypes.c_int64)]
        _lib = L
    return _lib


def _check(rc, what):
    if rc:
        raise RuntimeError("%s failed (%d): %s" % (what, rc, last_error()))


def write_vec(path, values):
    """values: 1D (block size 1) or 2D [n, bs]."""
    a = np.ascontiguousarray(values, dtype=np.float64)
    bs = 1 if a.ndim == 1 else a.shape[1]
    _check(_L().lagrbf_petsc_vec_write(str(path).encode(), a.ctypes.data, a.size, bs), "lagrbf_petsc_vec_write")


def read_vec(path):
    """[n // bs, bs] array (1D when the block size is 1)."""
    n, bs = ctypes.c_int64(), ctypes.c_int32()
    _check(_L().lagrbf_petsc_vec_read(str(path).encode(), None, 0, ctypes.byref(n), ctypes.byref(bs)),
           "lagrbf_petsc_vec_read")
    a = np.empty(n.value, dtype=np.float64)
    _check(_L().lagrbf_petsc_vec_read(str(path).encode(), a.ctypes.data, a.size, ctypes.byref(n), ctypes.byref(bs)),
           "lagrbf_petsc_vec_read")
    return a if bs.value == 1 else a.reshape(-1, bs.value)


def write_is(path, indices):
    a = np.ascontiguousarray(indices, dtype=np.int64).ravel()
    _check(_L().lagrbf_petsc_is_write(str(path).encode(), a.ctypes.data, a.size), "lagrbf_petsc_is_write")


def read_is(path):
    n = ctypes.c_int64()
    _check(_L().lagrbf_petsc_is_read(str(path).encode(), None, 0, ctypes.byref(n)), "lagrbf_petsc_is_read")
    a = np.empty(n.value, dtype=np.int64)
    _check(_L().lagrbf_petsc_is_read(str(path).encode(), a.ctypes.data, a.size, ctypes.byref(n)),
           "lagrbf_petsc_is_read")
    return a
