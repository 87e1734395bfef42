"""GPU test of the evaluation kernel's bounded waits: with the staging copies withheld (the barriers
are armed but nothing completes them) every wait runs out after a short poll limit, the kernel sets
its error flag and returns, and the call reports LAGRBF_ERR_TIMEOUT (200).  The context stays usable:
with the default limit restored the same evaluation gives the same values as before, bit for bit.
No copy is ever issued in the withheld mode, so nothing is in flight when the blocks exit.
"""
import numpy as np
import pytest

import lagrbf_gb300 as L
from lagrbf_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _ctx():
    rng = np.random.default_rng(21)
    xd = W.jittered_lattice(12, 3, rng)
    fd = W.abc_flow(xd)
    xp = W.uniform_points(800, 3, np.random.default_rng(22))
    c = L.LagRBFCtx(dim=3, npartitions=[4, 4, 4], overlap=W.pu_overlap(4), shape_factor=1.0, kernel=2, nfields=3,
                    advection=True, advection_scheme=2, advection_cfl=0.3, dt=1e-3, eval_precision="fp32")
    c.fill_data(xd, fd)
    c.fill_points(xp)
    return c, xp


def _fields(c, n):
    f = np.zeros((n, 3))
    c.output(fvals=f)
    return f


def test_withheld_copies_time_out_and_context_recovers():
    c, xp = _ctx()
    n = len(xp)
    assert c.stats()["records"] == 1  # the record-streamed kernel is the one under test
    c.interpolate_c()
    ref = _fields(c, n)
    c.test_eval_wait(2000, withhold_copies=True)
    with pytest.raises(RuntimeError, match="error code 200"):
        c.interpolate_c()
    with pytest.raises(RuntimeError, match="error code 200"):
        c.advect_resident(0.0, 1e-3)
    c.test_eval_wait(0, withhold_copies=False)
    c.fill_points(xp, pidx=np.arange(1, n + 1, dtype=np.int64))
    c.interpolate_c()
    assert np.array_equal(_fields(c, n), ref)
    c.advect_resident(0.0, 1e-3)  # the flag was cleared: stepping works again
