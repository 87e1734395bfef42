"""Known-answer tests of the CPU oracle (no GPU): binning and membership against plain numpy
restatements, PU weights against brute force, node reproduction of the PU interpolant, and the
convergence order of the RK1/RK2/RK4/Dormand-Prince drivers on a rigid rotation (the scenario of
the reference's src/tests/test_advection.c:43-155)."""
import numpy as np
import pytest

import oracle_lib as O
from oracle_lib import Oracle
from lagrbf_gb300 import workloads as W


def _pieces(dim, npu, overlap=None, kernel=2, nfields=1):
    return O.Pieces(dim=dim, npartitions=[npu] * dim, nfields=nfields,
                    overlap=W.pu_overlap(npu) if overlap is None else overlap, kernel=kernel)


@pytest.mark.parametrize("dim,npu", [(2, 7), (3, 5)])
def test_locate_convention(dim, npu):
    pc = _pieces(dim, npu)
    rng = np.random.default_rng(0)
    x = rng.uniform(-0.1, 1.1, size=(5000, dim))
    h = 1.0 / (npu - 1)
    planes = np.arange(npu) * h  # points on node planes, the box faces and corners
    x = np.concatenate([x, np.stack([planes] * dim, 1), [[np.nan] * dim]])
    c = pc.locate(x)
    with np.errstate(invalid="ignore"):
        inside = np.all((x >= 0.0) & (x <= 1.0), axis=1)
        t = np.clip(np.floor(x / h), 0, npu - 2).astype(np.int64)
    nc = npu - 1
    exp = t[:, 0] + nc * t[:, 1] + (nc * nc * t[:, 2] if dim == 3 else 0)
    exp = np.where(inside, exp, -1)
    assert np.array_equal(c, exp)


@pytest.mark.parametrize("dim,npu,nlat", [(2, 7, 30), (3, 5, 14)])
def test_membership_csrs(dim, npu, nlat):
    pc = _pieces(dim, npu)
    xd = W.jittered_lattice(nlat, dim, np.random.default_rng(1))
    cd = pc.locate(xd)
    (cs, cp), (ps, pp), (bs, bp) = pc.csr(cd)
    nc = npu - 1
    ncell = nc ** dim
    # cell CSR: stable counting sort
    assert np.array_equal(cs, np.concatenate([[0], np.cumsum(np.bincount(cd, minlength=ncell))]))
    assert np.array_equal(cp[:cs[-1]], np.argsort(cd, kind="stable"))

    def cell_ijk(c):
        return (c % nc, (c // nc) % nc, c // (nc * nc))

    # patch k = node k: its <= 2^dim adjacent cells in ascending order, points in cell order
    for k in range(npu ** dim):
        i, j, l = k % npu, (k // npu) % npu, k // (npu * npu)
        cells = sorted(ci + nc * cj + nc * nc * cl
                       for cl in ((l - 1, l) if dim == 3 else (0,)) for cj in (j - 1, j) for ci in (i - 1, i)
                       if 0 <= ci < nc and 0 <= cj < nc and 0 <= cl < (nc if dim == 3 else 1))
        exp = np.concatenate([cp[cs[c]:cs[c + 1]] for c in cells]) if cells else np.zeros(0, np.int32)
        assert np.array_equal(pp[ps[k]:ps[k + 1]], exp)
    # block of cell c: the points of its 3^dim neighbourhood (order inside is immaterial for values)
    for c in range(ncell):
        ci, cj, cl = cell_ijk(c)
        nb = [a + nc * b + nc * nc * e
              for e in ((cl - 1, cl, cl + 1) if dim == 3 else (0,)) for b in (cj - 1, cj, cj + 1)
              for a in (ci - 1, ci, ci + 1)
              if 0 <= a < nc and 0 <= b < nc and 0 <= e < (nc if dim == 3 else 1)]
        exp = np.concatenate([cp[cs[q]:cs[q + 1]] for q in nb])
        got = bp[bs[c]:bs[c + 1]]
        assert len(got) == len(exp) and np.array_equal(np.sort(got), np.sort(exp))


@pytest.mark.parametrize("dim,npu,overlap", [(2, 8, None), (3, 5, None), (3, 5, 2.7)])
def test_weights_brute_force(dim, npu, overlap):
    pc = _pieces(dim, npu, overlap)
    xp = W.uniform_points(400, dim, np.random.default_rng(2))
    cp = pc.locate(xp)
    w = pc.weights(xp, cp)
    h = 1.0 / (npu - 1)
    g = np.stack(np.meshgrid(*[np.arange(npu) * h] * dim, indexing="ij"), -1)
    nodes = g.transpose(list(range(dim))[::-1] + [dim]).reshape(-1, dim)  # x fastest
    eps = pc.pu.eps_w
    r = np.sqrt(((xp[:, None, :] - nodes[None]) ** 2).sum(-1))
    u = np.maximum(1.0 - eps * r, 0.0)
    phi = u ** 4 * (5.0 - 4.0 * u)
    tot = phi.sum(1)
    nc = npu - 1
    for p in range(len(xp)):
        c = cp[p]
        ci, cj, cl = c % nc, (c // nc) % nc, c // (nc * nc)
        for k in range(1 << dim):
            q = k & 3
            ox, oy, oz = int(q in (1, 2)), int(q >= 2), k >> 2
            node = (ci + ox) + npu * (cj + oy) + npu * npu * (cl + oz)
            assert abs(w[p, k] - phi[p, node] / tot[p]) <= 1e-14


@pytest.mark.parametrize("dim,npu,nlat", [(2, 6, 24), (3, 4, 10)])
def test_node_reproduction(dim, npu, nlat):
    """Support radius = one node spacing: only the cell's corners carry weight, and every corner
    patch holds the data of the cell, so the PU interpolant reproduces the data at data points."""
    xd = W.jittered_lattice(nlat, dim, np.random.default_rng(3))
    fd = W.cellular_flow(xd) if dim == 2 else W.abc_flow(xd)
    o = Oracle(dim=dim, npartitions=[npu] * dim, nfields=dim, overlap=npu / (npu - 1), kernel=2)
    assert o.fill(True, xd, fd) == 0 and o.fill(False, xd) == 0 and o.interpolate() == 0
    _, f, pid = o.output(len(xd))
    assert np.array_equal(pid, np.arange(1, len(xd) + 1))
    assert np.abs(f - fd).max() <= 1e-9


def _rotation_batch(npts, dim, coords, vel, user):
    for p in range(npts):
        x, y = coords[dim * p] - 0.5, coords[dim * p + 1] - 0.5
        vel[dim * p], vel[dim * p + 1] = -y, x
        if dim == 3:
            vel[dim * p + 2] = 0.0
    return 0


def _rotation_error(scheme, cfl, t_end=1.2, dim=2):
    """Max position error after t_end; the CFL step is cfl * 1.5 here (support radius 0.375,
    max speed 0.25), so cfl = 0.2 gives four equal steps of 0.3."""
    xp = 0.5 + 0.25 * np.stack([np.cos(np.linspace(0, 2 * np.pi, 16, endpoint=False)),
                                np.sin(np.linspace(0, 2 * np.pi, 16, endpoint=False))], 1)
    o = Oracle(dim=dim, npartitions=[5] * dim, nfields=dim, overlap=W.pu_overlap(5), kernel=2, advection=True,
               advection_scheme=scheme, advection_cfl=cfl)
    assert o.set_velocity_batch(_rotation_batch) == 0
    assert o.fill(False, xp) == 0
    assert o.advect_analytical(0.0, t_end) == 0
    x, _, _ = o.output(len(xp), fieldname="velocity")
    c, s = np.cos(t_end), np.sin(t_end)
    exact = 0.5 + np.stack([c * (xp[:, 0] - 0.5) - s * (xp[:, 1] - 0.5), s * (xp[:, 0] - 0.5) + c * (xp[:, 1] - 0.5)], 1)
    return np.abs(x - exact).max()


@pytest.mark.parametrize("scheme,order", [(0, 1), (1, 2), (2, 4)])
def test_rk_convergence_order(scheme, order):
    cfl = 0.1 if order < 4 else 0.2
    e1, e2 = _rotation_error(scheme, cfl), _rotation_error(scheme, cfl / 2)
    observed = np.log2(e1 / e2)
    assert abs(observed - order) < 0.35, (e1, e2, observed)


def test_dopri_meets_tolerance():
    assert _rotation_error(3, 0.1) <= 1e-6


def test_analytical_advection_without_fields():
    """n_interpolation_fields = 0 is a valid configuration for analytical advection."""
    xp = np.array([[0.3, 0.5], [0.6, 0.4]])
    o = Oracle(dim=2, npartitions=[5, 5], nfields=0, overlap=W.pu_overlap(5), kernel=2, advection=True,
               advection_scheme=2, advection_cfl=0.2)
    assert o.set_velocity_batch(_rotation_batch) == 0
    assert o.fill(False, xp) == 0
    assert o.advect_analytical(0.0, 0.3) == 0
    x, _, _ = o.output(len(xp), fieldname="velocity")
    assert np.all(np.isfinite(x)) and np.abs(x - xp).max() > 0.0


def _rotation_radii(per_particle, cfl=0.1, t_end=1.2):
    """Rigid rotation of particles at radii 0.02-0.4 (speeds 0.02-0.4): returns the max position
    error, internal steps (sweeps) and accepted particle steps."""
    r = np.linspace(0.02, 0.4, 24)
    a = np.linspace(0, 2 * np.pi, 24, endpoint=False)
    xp = 0.5 + np.stack([r * np.cos(a), r * np.sin(a)], 1)
    o = Oracle(dim=2, npartitions=[5, 5], nfields=2, overlap=W.pu_overlap(5), kernel=2, advection=True,
               advection_scheme=3, advection_cfl=cfl, dopri_per_particle=per_particle, dopri_rtol=1e-8,
               dopri_atol=1e-10)
    assert o.set_velocity_batch(_rotation_batch) == 0
    assert o.fill(False, xp) == 0
    assert o.advect_analytical(0.0, t_end) == 0
    x, _, _ = o.output(len(xp), fieldname="velocity")
    c, s = np.cos(t_end), np.sin(t_end)
    exact = 0.5 + np.stack([c * (xp[:, 0] - 0.5) - s * (xp[:, 1] - 0.5), s * (xp[:, 0] - 0.5) + c * (xp[:, 1] - 0.5)], 1)
    return np.abs(x - exact).max(), o.counts()[3], o.accepted()


def test_dopri_per_particle_meets_tolerance_with_fewer_particle_steps():
    """Per-particle adaptive Dormand-Prince (extension): every particle reaches t_end within the
    tolerance, and slow particles take fewer, longer steps than the global step imposes."""
    e_pp, sweeps, accepted = _rotation_radii(True)
    e_gl, steps, _ = _rotation_radii(False)
    assert e_pp <= 1e-6 and e_gl <= 1e-6, (e_pp, e_gl)
    assert accepted < 24 * steps, (accepted, steps)
    assert sweeps >= steps  # the fastest particle needs as many steps as the global scheme
