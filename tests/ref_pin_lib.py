"""ctypes access to LagRBF's own hot-loop units compiled against a PETSc stand-in
(oracle/_ref/liblagrbf_refpin.so, built by oracle/ref_pin/Makefile) -- test infrastructure.

Available only where the LagRBF source tree is present and the host has AVX-512F (the units are
AVX-512 / AVX-256 code); callers skip otherwise.
"""
import ctypes
import os
import platform
import subprocess

import numpy as np
from numpy.ctypeslib import ndpointer

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PIN_DIR = os.path.join(ROOT, "oracle", "ref_pin")
PIN_SO = os.path.join(ROOT, "oracle", "_ref", "liblagrbf_refpin.so")
# Location of a LagRBF checkout: required to (re)build the pin, no default.
REF = os.environ.get("LAGRBF_REFERENCE") or None

_lib = None
_why = None


def _has_avx512():
    if platform.machine() not in ("x86_64", "AMD64"):
        return False
    try:
        with open("/proc/cpuinfo") as f:
            return " avx512f" in f.read()
    except OSError:
        return False


def available():
    """(lib or None, reason)."""
    global _lib, _why
    if _lib is not None or _why is not None:
        return _lib, _why
    if not _has_avx512():
        _why = "host has no AVX-512F"
    elif not os.path.exists(PIN_SO) and not (REF and os.path.isdir(os.path.join(REF, "src"))):
        _why = ("no prebuilt pin library and no LagRBF source tree (set LAGRBF_REFERENCE to a LagRBF checkout)"
                if not REF else "LagRBF source tree not found at LAGRBF_REFERENCE=%s" % REF)
    else:
        if REF and os.path.isdir(os.path.join(REF, "src")):
            p = subprocess.run(["make", "-s", "-C", PIN_DIR, "REF=" + REF], capture_output=True, text=True)
            if p.returncode != 0:
                _why = "pin build failed: " + p.stdout[-300:] + p.stderr[-300:]
                return None, _why
        L = ctypes.CDLL(PIN_SO)
        d = ndpointer(np.float64, flags="C_CONTIGUOUS")
        i = ndpointer(np.int32, flags="C_CONTIGUOUS")
        l64 = ndpointer(np.int64, flags="C_CONTIGUOUS")
        i3 = ctypes.POINTER(ctypes.c_int)
        d3 = ctypes.POINTER(ctypes.c_double)
        L.rp_last_error.restype = ctypes.c_char_p
        L.rp_phi.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, d, ctypes.c_double, d]
        L.rp_weights.argtypes = [ctypes.c_int, i3, d3, d3, ctypes.c_double, ctypes.c_int, d, i, d]
        L.rp_assemble.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, i, d, d]
        L.rp_interpolate.argtypes = [ctypes.c_int, ctypes.c_int, i3, d3, d3, ctypes.c_double, ctypes.c_int,
                                     ctypes.c_int, d, i, i, i, i, d, l64, ctypes.c_int, ctypes.c_int, i, d, d, d]
        _lib = L
    return _lib, _why


def _geom(pc):
    pu = pc.pu
    n = (ctypes.c_int * 3)(*pu.n)
    O = (ctypes.c_double * 3)(*pu.O)
    L = (ctypes.c_double * 3)(*pu.L)
    return n, O, L


def _check(rc):
    if rc:
        raise RuntimeError("reference unit failed (%d): %s" % (rc, _lib.rp_last_error().decode()))


def phi(kernel, lanes, r, eps):
    r = np.ascontiguousarray(r, dtype=np.float64)
    out = np.zeros_like(r)
    _check(_lib.rp_phi(kernel, lanes, len(r), r, eps, out))
    return out


def weights(pc, x, cellid):
    n, O, L = _geom(pc)
    x = np.ascontiguousarray(x, dtype=np.float64)
    w = np.zeros(len(x) * pc.nen)
    _check(_lib.rp_weights(pc.dim, n, O, L, pc.pu.eps_w, len(x), x.reshape(-1), cellid, w))
    return w.reshape(len(x), pc.nen)


def assemble(pc, kernel, idx, xd):
    m = len(idx)
    A = np.zeros(m * m)
    _check(_lib.rp_assemble(pc.dim, kernel, pc.pu.eps_r, m, np.ascontiguousarray(idx, dtype=np.int32),
                            np.ascontiguousarray(xd, dtype=np.float64).reshape(-1), A))
    return A.reshape(m, m)


def interpolate(pc, lanes, kernel, xd, bs, bp, ps, pp, coeffs, coff, nf, xp, cellid, w):
    n, O, L = _geom(pc)
    out = np.zeros(len(xp) * nf)
    _check(_lib.rp_interpolate(lanes, pc.dim, n, O, L, pc.pu.eps_r, kernel, len(xd),
                               np.ascontiguousarray(xd, dtype=np.float64).reshape(-1), bs, bp, ps, pp, coeffs,
                               np.ascontiguousarray(coff, dtype=np.int64), nf, len(xp), cellid,
                               np.ascontiguousarray(xp, dtype=np.float64).reshape(-1),
                               np.ascontiguousarray(w).reshape(-1), out))
    return out.reshape(len(xp), nf)
