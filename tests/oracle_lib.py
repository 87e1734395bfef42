"""ctypes access to the CPU oracle (oracle/_build/liblagrbf_oracle.so) -- test infrastructure.

The oracle is the checker: tests compare the GPU library against it, never the other way round.
"""
import ctypes
import os
import subprocess

import numpy as np
from numpy.ctypeslib import ndpointer

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "liblagrbf_oracle.so")


class OrcConfig(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("n", ctypes.c_int * 3), ("O", ctypes.c_double * 3), ("L", ctypes.c_double * 3),
        ("overlap", ctypes.c_double), ("shape_factor", ctypes.c_double), ("kernel", ctypes.c_int),
        ("solve_method", ctypes.c_int), ("nfields", ctypes.c_int), ("advection", ctypes.c_int),
        ("scheme", ctypes.c_int), ("cfl_fac", ctypes.c_double), ("dt", ctypes.c_double),
        ("rmin", ctypes.c_double), ("rmax", ctypes.c_double), ("dopri_dt_fac", ctypes.c_double),
        ("dopri_dt_fac_min", ctypes.c_double), ("dopri_dt_fac_max", ctypes.c_double),
        ("dopri_atol", ctypes.c_double), ("dopri_rtol", ctypes.c_double), ("dopri_per_particle", ctypes.c_int),
        ("setup_all", ctypes.c_int),
    ]


class OrcPU(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("n", ctypes.c_int * 3), ("nnodes", ctypes.c_int), ("ncells", ctypes.c_int),
        ("nen", ctypes.c_int), ("O", ctypes.c_double * 3), ("L", ctypes.c_double * 3), ("h", ctypes.c_double * 3),
        ("eps_w", ctypes.c_double), ("eps_r", ctypes.c_double),
    ]


STEP_REDUCE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int32, ctypes.c_void_p)
VFN_BATCH = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                             ctypes.POINTER(ctypes.c_double), ctypes.c_void_p)

_lib = None


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(
                os.path.join(ORACLE_DIR, "lagrbf_oracle.c")):
            build_oracle()
        L = ctypes.CDLL(ORACLE_SO)
        d = ndpointer(np.float64, flags="C_CONTIGUOUS")
        i = ndpointer(np.int32, flags="C_CONTIGUOUS")

        class DN(d):
            @classmethod
            def from_param(cls, o):
                return o if o is None else super().from_param(o)

        class IN(i):
            @classmethod
            def from_param(cls, o):
                return o if o is None else super().from_param(o)

        class LN(ndpointer(np.int64, flags="C_CONTIGUOUS")):
            @classmethod
            def from_param(cls, o):
                return o if o is None else super().from_param(o)

        L.orc_config_default.argtypes = [ctypes.POINTER(OrcConfig)]
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.POINTER(OrcConfig)]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_fill_swarm.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, d, DN, LN]
        L.orc_interpolation.argtypes = [ctypes.c_void_p]
        L.orc_output.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, DN, DN, LN, ctypes.c_char_p]
        L.orc_reset_coefficients.argtypes = [ctypes.c_void_p]
        L.orc_advect_interpolate.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
        L.orc_advect_analytical.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
        L.orc_set_velocity_batch_fn.argtypes = [ctypes.c_void_p, VFN_BATCH, ctypes.c_void_p]
        L.orc_get_counts.argtypes = [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_int)] * 4
        L.orc_set_step_reduce.argtypes = [ctypes.c_void_p, STEP_REDUCE, ctypes.c_void_p]
        L.orc_get_accepted.restype = ctypes.c_longlong
        L.orc_get_accepted.argtypes = [ctypes.c_void_p]
        L.orc_get_dt.restype = ctypes.c_double
        L.orc_get_dt.argtypes = [ctypes.c_void_p]
        L.orc_get_cellids.argtypes = [ctypes.c_void_p, ctypes.c_int, i]
        L.orc_get_patch_csr.restype = ctypes.c_long
        L.orc_get_patch_csr.argtypes = [ctypes.c_void_p, IN, IN]
        L.orc_get_block_csr.restype = ctypes.c_long
        L.orc_get_block_csr.argtypes = [ctypes.c_void_p, IN, IN]
        L.orc_get_weights.argtypes = [ctypes.c_void_p, d]
        L.orc_time_baseline.argtypes = [ctypes.POINTER(OrcConfig), ctypes.c_int, d, d, ctypes.c_int, d, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double)]
        pu = ctypes.POINTER(OrcPU)
        L.orc_pu_setup.argtypes = [pu, ctypes.POINTER(OrcConfig)]
        L.orc_phi_scalar.restype = ctypes.c_double
        L.orc_phi_scalar.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_phi_lane.restype = ctypes.c_double
        L.orc_phi_lane.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_locate.argtypes = [pu, ctypes.c_int, d, i]
        L.orc_cell_csr.argtypes = [pu, ctypes.c_int, i, i, i]
        L.orc_patch_csr.restype = ctypes.c_long
        L.orc_patch_csr.argtypes = [pu, i, i, IN, IN]
        L.orc_block_csr.restype = ctypes.c_long
        L.orc_block_csr.argtypes = [pu, i, i, IN, IN]
        L.orc_weights.argtypes = [pu, ctypes.c_int, d, i, IN, d]
        L.orc_assemble.argtypes = [pu, ctypes.c_int, ctypes.c_int, i, d, d]
        L.orc_patch_solve.argtypes = [pu, ctypes.c_int, ctypes.c_int, i, d, ctypes.c_int, d, d]
        L.orc_eval.argtypes = [pu, ctypes.c_int, ctypes.c_int, d, i, IN, d, d, i, i, i, i, IN,
                               ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), ctypes.c_int, d]
        _lib = L
    return _lib


def make_config(dim, npartitions, nfields, kernel=2, overlap=1.0, shape_factor=1.0, minCoords=None,
                maxCoords=None, solve_method=2, advection=False, advection_scheme=2, advection_cfl=0.3,
                dt=1e-4, rmin=0.0, rmax=1e132, dopri_per_particle=False, dopri_rtol=None, dopri_atol=None,
                setup_all_patches=False, **_):
    """Config with the lagrbfpy keyword defaults (context.py:113-201)."""
    c = OrcConfig()
    lib().orc_config_default(ctypes.byref(c))
    c.dim = dim
    for k in range(dim):
        c.n[k] = int(npartitions[k])
        c.O[k] = 0.0 if minCoords is None else minCoords[k]
        c.L[k] = 1.0 if maxCoords is None else maxCoords[k]
    c.overlap, c.shape_factor, c.kernel, c.solve_method, c.nfields = overlap, shape_factor, kernel, solve_method, nfields
    c.advection, c.scheme, c.cfl_fac, c.dt, c.rmin, c.rmax = int(advection), advection_scheme, advection_cfl, dt, rmin, rmax
    c.dopri_per_particle = int(bool(dopri_per_particle))
    c.setup_all = int(bool(setup_all_patches))
    if dopri_rtol is not None:
        c.dopri_rtol = dopri_rtol
    if dopri_atol is not None:
        c.dopri_atol = dopri_atol
    return c


class Oracle:
    """The reference API (lagrbf_* semantics) on the CPU oracle."""

    def __init__(self, **kw):
        self.cfg = make_config(**kw)
        self.dim = self.cfg.dim
        self.nfields = self.cfg.nfields
        self.h = lib().orc_create(ctypes.byref(self.cfg))
        if not self.h:
            raise RuntimeError("orc_create failed")
        self._keep = []

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def fill(self, is_data, coords, values=None, pidx=None):
        coords = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1)
        v = None if values is None else np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        p = None if pidx is None else np.ascontiguousarray(pidx, dtype=np.int64)
        return lib().orc_fill_swarm(self.h, int(is_data), coords.size // self.dim, coords, v, p)

    def interpolate(self):
        return lib().orc_interpolation(self.h)

    def output(self, n, fieldname="fields", is_data=False):
        nf = {"fields": self.nfields, "velocity": self.dim, "weights": 1 << self.dim}[fieldname]
        x = np.zeros(n * self.dim)
        f = np.zeros(n * nf)
        pid = np.zeros(n, dtype=np.int64)
        rc = lib().orc_output(self.h, int(is_data), n, x, f, pid, fieldname.encode())
        if rc:
            raise RuntimeError("orc_output failed %d" % rc)
        return x.reshape(n, self.dim), f.reshape(n, nf), pid

    def reset(self):
        return lib().orc_reset_coefficients(self.h)

    def advect(self, t, tn):
        return lib().orc_advect_interpolate(self.h, t, tn)

    def advect_analytical(self, t, tn):
        return lib().orc_advect_analytical(self.h, t, tn)

    def set_velocity_batch(self, fn):
        cb = VFN_BATCH(fn)
        self._keep.append(cb)
        return lib().orc_set_velocity_batch_fn(self.h, cb, None)

    def set_step_reduce(self, fn):
        """fn(vals: numpy view of n doubles) reduces them in place (element-wise max over ranks)."""
        def cb(ptr, n, user):
            fn(np.ctypeslib.as_array(ptr, shape=(n,)))
            return 0
        c = STEP_REDUCE(cb)
        self._keep.append(c)
        return lib().orc_set_step_reduce(self.h, c, None)

    def counts(self):
        v = [ctypes.c_int() for _ in range(4)]
        lib().orc_get_counts(self.h, *[ctypes.byref(x) for x in v])
        return [x.value for x in v]

    def dt(self):
        return lib().orc_get_dt(self.h)

    def accepted(self):
        return lib().orc_get_accepted(self.h)

    def cellids(self, is_data, n):
        out = np.zeros(n, dtype=np.int32)
        lib().orc_get_cellids(self.h, int(is_data), out)
        return out

    def patch_csr(self, nnodes):
        tot = lib().orc_get_patch_csr(self.h, None, None)
        s = np.zeros(nnodes + 1, dtype=np.int32)
        p = np.zeros(max(tot, 1), dtype=np.int32)
        lib().orc_get_patch_csr(self.h, s, p)
        return s, p[:tot]

    def block_csr(self, ncells):
        tot = lib().orc_get_block_csr(self.h, None, None)
        s = np.zeros(ncells + 1, dtype=np.int32)
        p = np.zeros(max(tot, 1), dtype=np.int32)
        lib().orc_get_block_csr(self.h, s, p)
        return s, p[:tot]


class Pieces:
    """The oracle's building blocks on one mesh (geometry, binning, membership, weights, patch
    solves and evaluation), for comparisons below the lagrbf_* API."""

    def __init__(self, **kw):
        self.cfg = make_config(**kw)
        self.pu = OrcPU()
        lib().orc_pu_setup(ctypes.byref(self.pu), ctypes.byref(self.cfg))
        self.dim, self.nen = self.pu.dim, self.pu.nen
        self.nnodes, self.ncells = self.pu.nnodes, self.pu.ncells

    def locate(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        c = np.zeros(len(x), dtype=np.int32)
        lib().orc_locate(ctypes.byref(self.pu), len(x), x.reshape(-1), c)
        return c

    def csr(self, cellid):
        cs = np.zeros(self.ncells + 1, dtype=np.int32)
        cp = np.zeros(max(len(cellid), 1), dtype=np.int32)
        lib().orc_cell_csr(ctypes.byref(self.pu), len(cellid), cellid, cs, cp)
        tot = lib().orc_patch_csr(ctypes.byref(self.pu), cs, cp, None, None)
        ps = np.zeros(self.nnodes + 1, dtype=np.int32)
        pp = np.zeros(max(tot, 1), dtype=np.int32)
        lib().orc_patch_csr(ctypes.byref(self.pu), cs, cp, ps, pp)
        tot = lib().orc_block_csr(ctypes.byref(self.pu), cs, cp, None, None)
        bs = np.zeros(self.ncells + 1, dtype=np.int32)
        bp = np.zeros(max(tot, 1), dtype=np.int32)
        lib().orc_block_csr(ctypes.byref(self.pu), cs, cp, bs, bp)
        return (cs, cp), (ps, pp), (bs, bp)

    def weights(self, x, cellid):
        x = np.ascontiguousarray(x, dtype=np.float64)
        w = np.zeros(len(x) * self.nen)
        lib().orc_weights(ctypes.byref(self.pu), len(x), x.reshape(-1), cellid, None, w)
        return w.reshape(len(x), self.nen)

    def assemble(self, kernel, idx, xd):
        m = len(idx)
        A = np.zeros(m * m)
        lib().orc_assemble(ctypes.byref(self.pu), kernel, m, np.ascontiguousarray(idx, dtype=np.int32),
                           np.ascontiguousarray(xd, dtype=np.float64).reshape(-1), A)
        return A.reshape(m, m)

    def solve_all(self, kernel, xd, fd, ps, pp):
        """Coefficients of every patch, packed column-major per patch; offsets coff[nnodes+1]."""
        nf = fd.shape[1]
        sizes = np.diff(ps).astype(np.int64)
        coff = np.concatenate([[0], np.cumsum(sizes * nf)]).astype(np.int64)
        coeffs = np.zeros(max(int(coff[-1]), 1))
        xdf = np.ascontiguousarray(xd, dtype=np.float64).reshape(-1)
        fdf = np.ascontiguousarray(fd, dtype=np.float64).reshape(-1)
        for k in range(self.nnodes):
            m = int(sizes[k])
            if m == 0:
                continue
            out = np.zeros(m * nf)
            rc = lib().orc_patch_solve(ctypes.byref(self.pu), kernel, m, np.ascontiguousarray(pp[ps[k]:ps[k + 1]]),
                                       xdf, nf, fdf, out)
            if rc:
                raise RuntimeError("patch %d: non-positive pivot at row %d" % (k, rc))
            coeffs[coff[k]:coff[k + 1]] = out
        return coeffs, coff

    def eval(self, kernel, xp, cellid, w, xd, bs, bp, ps, pp, coeffs, coff, nf_total, nf):
        n = len(xp)
        ptrs = (ctypes.POINTER(ctypes.c_double) * self.nnodes)()
        base = coeffs.ctypes.data
        for k in range(self.nnodes):
            ptrs[k] = ctypes.cast(base + 8 * int(coff[k]), ctypes.POINTER(ctypes.c_double))
        setup = np.ones(self.nnodes, dtype=np.int32)
        out = np.zeros(n * nf)
        lib().orc_eval(ctypes.byref(self.pu), kernel, n, np.ascontiguousarray(xp, dtype=np.float64).reshape(-1),
                       cellid, None, np.ascontiguousarray(w).reshape(-1),
                       np.ascontiguousarray(xd, dtype=np.float64).reshape(-1), bs, bp, ps, pp, setup, ptrs, nf, out)
        return out.reshape(n, nf)
