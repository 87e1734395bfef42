"""LagRBFInterpolator (mirrors lagrbfpy/interpolation.py:35-115)."""
from .context import LagRBFCtx


class LagRBFInterpolator(LagRBFCtx):
    """RBF partition-of-unity interpolation (no polynomial augmentation)."""

    def __init__(self, petsc_options=None, **kwargs):
        super().__init__(petsc_options=petsc_options, **kwargs)

    def interpolate(self, data, points, output, fieldname="fields"):
        """fill data -> fill points -> interpolate -> output -> reset (interpolation.py:64-115)."""
        self.fill_data(coords=data.coords, values=data.values, pidx=data.pidx)
        self.fill_points(coords=points.coords, values=points.values, pidx=points.pidx)
        self.interpolate_c()
        self.output(coords=output.coords, fvals=output.values, pidx=output.pidx, fieldname=fieldname, is_data=False)
        self.reset_coefficients()
