"""Serving loop (lagrbf_server_* of liblagrbf.so): advection jobs admitted by a device-memory
budget and run concurrently, one context and CUDA stream per running job, datasets kept resident
by id for later jobs.  p50/p99 latency is measured from submission to completion."""
import ctypes

import numpy as np

from ._lib import load_shared_lib, last_error


class Job(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32), ("nodes", ctypes.c_int32 * 3), ("O", ctypes.c_double * 3),
        ("L", ctypes.c_double * 3), ("overlap", ctypes.c_double), ("shape_factor", ctypes.c_double),
        ("kernel", ctypes.c_int32), ("nfields", ctypes.c_int32), ("dataset_id", ctypes.c_int64),
        ("nd", ctypes.c_int32), ("data_coords", ctypes.c_void_p), ("data_values", ctypes.c_void_p),
        ("np", ctypes.c_int32), ("particles", ctypes.c_void_p), ("scheme", ctypes.c_int32),
        ("nsteps", ctypes.c_int32), ("dt", ctypes.c_double), ("cfl", ctypes.c_double), ("fp32", ctypes.c_int32),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("failed", ctypes.c_int64),
        ("queued", ctypes.c_int64), ("running", ctypes.c_int64), ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
        ("particle_steps", ctypes.c_double), ("elapsed_s", ctypes.c_double), ("bytes_in_use", ctypes.c_double),
        ("datasets_resident", ctypes.c_int32), ("queue_p50_ms", ctypes.c_double), ("queue_p99_ms", ctypes.c_double),
        ("service_p50_ms", ctypes.c_double), ("service_p99_ms", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _lib():
    L = load_shared_lib()
    L.lagrbf_server_create.restype = ctypes.c_void_p
    L.lagrbf_server_create.argtypes = [ctypes.c_double, ctypes.c_int32]
    L.lagrbf_server_submit.argtypes = [ctypes.c_void_p, ctypes.POINTER(Job), ctypes.POINTER(ctypes.c_int64)]
    L.lagrbf_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    L.lagrbf_server_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ServerStats)]
    L.lagrbf_server_reset_stats.argtypes = [ctypes.c_void_p]
    L.lagrbf_server_destroy.argtypes = [ctypes.c_void_p]
    return L


class Server:
    def __init__(self, hbm_budget_bytes=150e9, nworkers=8):
        self._L = _lib()
        self.h = self._L.lagrbf_server_create(float(hbm_budget_bytes), int(nworkers))
        if not self.h:
            raise RuntimeError("lagrbf_server_create failed: " + last_error())
        self._np = {}

    def submit(self, *, npartitions, particles, dt, nsteps, scheme=2, data_coords=None, data_values=None,
               dataset_id=0, overlap=None, shape_factor=1.0, kernel=2, nfields=None, minCoords=None,
               maxCoords=None, cfl=0.3, fp32=True):
        particles = np.ascontiguousarray(particles, dtype=np.float64)
        dim = particles.shape[1]
        j = Job()
        j.dim = dim
        for d in range(dim):
            j.nodes[d] = int(npartitions[d])
            j.O[d] = 0.0 if minCoords is None else minCoords[d]
            j.L[d] = 1.0 if maxCoords is None else maxCoords[d]
        n = int(npartitions[0])
        j.overlap = 1.5 * n / (n - 1) if overlap is None else overlap
        j.shape_factor, j.kernel = shape_factor, kernel
        keep = [particles]
        if data_values is not None:
            data_coords = np.ascontiguousarray(data_coords, dtype=np.float64)
            data_values = np.ascontiguousarray(data_values, dtype=np.float64)
            keep += [data_coords, data_values]
            j.nd = len(data_coords)
            j.data_coords, j.data_values = data_coords.ctypes.data, data_values.ctypes.data
            j.nfields = data_values.shape[1]
        else:
            j.nfields = dim if nfields is None else nfields
        j.dataset_id = int(dataset_id)
        j.np = len(particles)
        j.particles = particles.ctypes.data
        j.scheme, j.nsteps, j.dt, j.cfl, j.fp32 = scheme, nsteps, dt, cfl, int(bool(fp32))
        jid = ctypes.c_int64()
        rc = self._L.lagrbf_server_submit(self.h, ctypes.byref(j), ctypes.byref(jid))
        if rc:
            raise RuntimeError("lagrbf_server_submit failed (%d): %s" % (rc, last_error()))
        self._np[jid.value] = (len(particles), dim)
        return jid.value

    def wait(self, job_id):
        """(positions [np, dim], latency_ms)."""
        n, dim = self._np[job_id]
        out = np.zeros((n, dim))
        lat = ctypes.c_double()
        rc = self._L.lagrbf_server_wait(self.h, job_id, out.ctypes.data, ctypes.byref(lat))
        if rc:
            raise RuntimeError("job %d failed (%d): %s" % (job_id, rc, last_error()))
        return out, lat.value

    def stats(self):
        st = ServerStats()
        self._L.lagrbf_server_stats(self.h, ctypes.byref(st))
        return st.as_dict()

    def reset_stats(self):
        self._L.lagrbf_server_reset_stats(self.h)

    def close(self):
        if self.h:
            self._L.lagrbf_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
