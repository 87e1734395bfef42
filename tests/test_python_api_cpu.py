"""Host-side helpers of the lagrbfpy mirror: FunctionPointer (a Python velocity callback as the C
pointer lagrbf_advection_function_batch takes) and fill_datafields."""
import ctypes

import numpy as np
import pytest

import lagrbf_gb300 as L


class _Data(L.FunctionData):
    _fields_ = [("p1", ctypes.c_double), ("p2", ctypes.c_int32)]


def test_function_pointer_calls_back_with_data():
    def fn(npoints, dim, coords, velocity, data_ptr):
        d = ctypes.cast(data_ptr, ctypes.POINTER(_Data)).contents
        X = np.ctypeslib.as_array(coords, shape=(npoints, dim))
        V = np.ctypeslib.as_array(velocity, shape=(npoints, dim))
        V[:, :] = X * d.p1 + d.p2 + d.step
        return 0

    data = _Data(time=1.2, step=4, p1=2.0, p2=3)
    fp = L.FunctionPointer(fn, data)
    assert fp.func is fn and fp.data is data
    x = np.arange(6.0).reshape(3, 2)
    v = np.zeros_like(x)
    dp = ctypes.cast(ctypes.pointer(data), ctypes.c_void_p)
    rc = fp.cfunc(3, 2, x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                  v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), dp)
    assert rc == 0 and np.array_equal(v, x * 2.0 + 3 + 4)


def test_function_pointer_rejects_bad_arguments():
    with pytest.raises(TypeError):
        L.FunctionPointer(lambda *a: 0, data=3.0)
    with pytest.raises(TypeError):
        L.FunctionPointer(42)


def test_fill_datafields():
    pd = {"velocity": np.array([[1.0, np.nan], [3.0, 4.0]]), "T": np.array([5.0, 6.0])}
    out = L.fill_datafields(2, {"T": 1, "missing": 2, "velocity": 2}, pd, nan_replacement=-1.0)
    assert out.shape == (2, 5)
    assert np.array_equal(out[:, 0], [5.0, 6.0])
    assert np.array_equal(out[:, 1:3], [[1.0, -1.0], [3.0, 4.0]])
    assert not out[:, 3:].any()  # a missing field does not advance the column (as lagrbfpy)
