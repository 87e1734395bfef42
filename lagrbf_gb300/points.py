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


def fill_datafields(npoints, fields, point_data, nan_replacement=0.0):
    """[npoints, sum of components] array of the named fields of point_data, in the order of
    `fields` (name -> components), NaNs replaced; fields missing from point_data are skipped
    (lagrbfpy/utils/points_container.py:49-77)."""
    nfields = sum(fields.values())
    fvals = np.zeros((npoints, nfields), dtype=np.float64)
    idx = 0
    for name, ncomp in fields.items():
        if name in point_data:
            fvals[:, idx:idx + ncomp] = np.nan_to_num(np.asarray(point_data[name]).reshape((npoints, ncomp)),
                                                      nan=nan_replacement)
            idx += ncomp
    return fvals
