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


# ------------------------------------------------------------------------------------------------
# lagrbfpy's petsc_io names (python_api/lagrbfpy/petsc_io/petscvec_loader.py and
# petscvec_writer.py), with the same arguments and results, for callers that used them through
# PETSc's PetscBinaryIO.  Formats: big-endian; Vec = [1211214, n] + n doubles; IS = [1211218, n] +
# n int32; Mat (AIJ layout) = [1211216, M, N, nz] + M row lengths + nz column indices + nz values.
# ------------------------------------------------------------------------------------------------
VEC_CLASSID, MAT_CLASSID, IS_CLASSID = 1211214, 1211216, 1211218


def _read_header(fp, classid, count):
    h = np.fromfile(fp, dtype=">i4", count=count)
    if len(h) != count:
        raise ValueError("truncated PETSc binary file")
    if h[0] != classid:
        raise ValueError("unexpected PETSc binary class id %d (expected %d)" % (h[0], classid))
    return [int(v) for v in h[1:]]


def _read_exact(fp, dtype, count):
    a = np.fromfile(fp, dtype=dtype, count=count)
    if len(a) != count:
        raise ValueError("truncated PETSc binary file")
    return a


def PetscVecLoadFromFile(fname, **kwargs):
    """The values of a binary Vec file, flat (petscvec_loader.py:32-37)."""
    with open(fname, "rb") as fp:
        (n,) = _read_header(fp, VEC_CLASSID, 2)
        return _read_exact(fp, ">f8", n).astype(np.float64)


def PetscVecLoadBlockSizeFromFile(fname):
    """The block size of a Vec from its .info file (petscvec_loader.py:39-45)."""
    with open(fname) as fp:
        line = fp.readline()
    if not line.startswith("-vecload_block_size"):
        raise ValueError('Expected first line to be "-vecload_block_size <size>", got: %s' % line)
    return int(line.split()[1])


def PetscVecLoad(fname, order="C", **kwargs):
    """A Vec reshaped to (-1, bs) when "<fname>.info" exists, else flat (petscvec_loader.py:47-54)."""
    v = PetscVecLoadFromFile(fname, **kwargs)
    try:
        bs = PetscVecLoadBlockSizeFromFile(str(fname) + ".info")
    except FileNotFoundError:
        return v
    return np.reshape(v, (-1, bs), order=order)


def PetscISLoadFromFile(fname, **kwargs):
    """The indices of a binary IS file as int32 (petscvec_loader.py:56-61)."""
    with open(fname, "rb") as fp:
        (n,) = _read_header(fp, IS_CLASSID, 2)
        return _read_exact(fp, ">i4", n).astype(np.int32)


def PetscMatDenseLoadFromFile(fname, **kwargs):
    """A binary Mat file as a dense M x N array (petscvec_loader.py:63-68)."""
    with open(fname, "rb") as fp:
        M, N, nz = _read_header(fp, MAT_CLASSID, 4)
        if nz < 0:  # dense storage: M*N values row by row
            return _read_exact(fp, ">f8", M * N).astype(np.float64).reshape(M, N)
        rows = _read_exact(fp, ">i4", M).astype(np.int64)
        cols = _read_exact(fp, ">i4", nz).astype(np.int64)
        vals = _read_exact(fp, ">f8", nz).astype(np.float64)
    if rows.sum() != nz:
        raise ValueError("inconsistent row lengths in PETSc binary Mat file")
    out = np.zeros((M, N), dtype=np.float64)
    out[np.repeat(np.arange(M), rows), cols] = vals
    return out


def PetscVecWriteToFile(fname, v):
    """A flat binary Vec file of v's values (petscvec_writer.py:31-35)."""
    a = np.ascontiguousarray(v, dtype=np.float64).ravel()
    with open(fname, "wb") as fp:
        np.array([VEC_CLASSID, a.size], dtype=">i4").tofile(fp)
        a.astype(">f8").tofile(fp)


def PetscVecWriteBlockSizeToFile(fname, v):
    """Writes "-vecload_block_size <bs>" (bs = columns of v, 1 for 1D) to fname; returns bs
    (petscvec_writer.py:37-44)."""
    bs = v.shape[1] if np.ndim(v) > 1 else 1
    with open(fname, "w") as fp:
        fp.write("-vecload_block_size %d\n" % bs)
    return bs


def PetscVecWrite(fname, v):
    """The .info block size file and the flat Vec file (petscvec_writer.py:46-51)."""
    bs = PetscVecWriteBlockSizeToFile(str(fname) + ".info", v)
    if bs > 1:
        v = np.reshape(v, (v.shape[0] * bs))
    PetscVecWriteToFile(fname, v)


def PetscISWriteToFile(fname, iset):
    """A binary IS file of int32 indices (petscvec_writer.py:53-57)."""
    a = np.ascontiguousarray(iset).ravel()
    if a.size and (a.min() < -2**31 or a.max() >= 2**31):
        raise ValueError("index out of the 32-bit PetscInt range")
    with open(fname, "wb") as fp:
        np.array([IS_CLASSID, a.size], dtype=">i4").tofile(fp)
        a.astype(">i4").tofile(fp)
