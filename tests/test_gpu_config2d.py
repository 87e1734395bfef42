"""The 2D CPU-runnable configuration: 64x64 jittered lattice (4,096 nodes) carrying the cellular
flow, 8x8 PU nodes with an overlap of 1.5 spacings, 10,000 particles, Gaussian kernel with
eps = 3/h, RK4 with dt = 1e-3, through the reference's call sequence (fill data, interpolate,
advect over [t, t + dt], repeated).  The GPU's FP64 trajectories are compared with the CPU
oracle's after all 100 steps."""
import numpy as np
import pytest

from oracle_lib import Oracle
import lagrbf_gb300 as L
from lagrbf_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_cellular_2d_rk4_steps(nsteps=100):
    xd, fd, xp, opts = W.config_cellular_2d(np_=10000, seed=1, kernel=6)
    adv = dict(advection=True, advection_scheme=2, advection_cfl=0.3, dt=1e-3, solve_method=1)
    c = L.LagRBFCtx(**opts, **adv)
    o = Oracle(**opts, **adv)
    c.fill_points(xp)
    assert o.fill(False, xp) == 0
    dt = 1e-3
    for s in range(nsteps):
        c.fill_data(xd, fd)
        assert o.fill(True, xd, fd) == 0
        c.interpolate_c()
        assert o.interpolate() == 0
        c.advect_interpolate_c(s * dt, (s + 1) * dt)
        assert o.advect(s * dt, (s + 1) * dt) == 0
    n = len(xp)
    x1 = np.zeros((n, 2)); f1 = np.zeros((n, 2)); p1 = np.zeros(n, dtype=np.int64)
    c.output(coords=x1, fvals=f1, pidx=p1)
    x2, f2, p2 = o.output(n)
    assert np.array_equal(p1, p2)
    alive = p1 > 0
    assert alive.mean() > 0.95
    assert np.abs(x1 - x2).max() <= 1e-10
    # the interpolated field follows the cellular flow: stream function preserved along paths
    psi0 = np.sin(np.pi * xp[:, 0]) * np.sin(np.pi * xp[:, 1])
    psi1 = np.sin(np.pi * x1[:, 0]) * np.sin(np.pi * x1[:, 1])
    assert np.abs(psi1[alive] - psi0[alive]).max() < 5e-3
