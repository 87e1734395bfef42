"""PointContainer: coordinates, values and unique point indices of a point set
(mirrors lagrbfpy/utils/points_container.py)."""
import numpy as np


class PointContainer:
    def __init__(self, coords=None, values=None, pidx=None):
        self.coords = None if coords is None else np.ascontiguousarray(coords, dtype=np.float64)
        self.values = None if values is None else np.ascontiguousarray(values, dtype=np.float64)
        self.pidx = None if pidx is None else np.ascontiguousarray(pidx, dtype=np.int64)

    @classmethod
    def empty(cls, npoints, dim, nfields):
        return cls(np.zeros((npoints, dim)), np.zeros((npoints, nfields)), np.zeros(npoints, dtype=np.int64))
