"""The CUDA path (through the C-ABI) against the golden fixtures of tests/golden/, i.e. against the
outputs of LagRBF's own weights and evaluation units.  FP64 path: PU weights within 1e-13 (absolute;
weights lie in [0, 1]) and interpolated values within 1e-10 max-normalised relative error (the
patch coefficients come from the GPU's own Cholesky, the fixtures' from the oracle's)."""
import glob
import os

import numpy as np
import pytest

import lagrbf_gb300 as L

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz")))


def _rel(a, b):
    den = np.abs(b).max(axis=0)
    den[den == 0] = 1.0
    return float((np.abs(a - b).max(axis=0) / den).max())


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_matches_reference_units(path, precision):
    g = np.load(path)
    dim, npu, kernel = int(g["dim"]), int(g["npu"]), int(g["kernel"])
    nf = g["fd"].shape[1]
    c = L.LagRBFCtx(dim=dim, npartitions=[npu] * dim, nfields=nf, overlap=float(g["overlap"]), kernel=kernel,
                    shape_factor=float(g["shape_factor"]))
    if precision == "fp32":
        c.set_precision(True)
    c.fill_data(g["xd"], g["fd"])
    c.fill_points(g["xp"])
    c.interpolate_c()
    n = len(g["xp"])
    x = np.zeros((n, dim)); f = np.zeros((n, nf)); p = np.zeros(n, dtype=np.int64)
    c.output(coords=x, fvals=f, pidx=p, fieldname="fields")
    assert np.array_equal(p, np.arange(1, n + 1))
    assert np.array_equal(x, g["xp"])
    w = np.zeros((n, 1 << dim))
    c.output(coords=np.zeros((n, dim)), fvals=w, pidx=np.zeros(n, dtype=np.int64), fieldname="weights")
    assert np.abs(w - g["weights_ref"]).max() <= 1e-13
    tol = 1e-10 if precision == "fp64" else 1e-6
    assert _rel(f, g["values_ref"]) <= tol
