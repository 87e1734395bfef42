"""The oracle against LagRBF's own hot-loop units (compiled unmodified against a PETSc stand-in,
oracle/ref_pin/) on the same inputs.  Bit-exact wherever both sides use IEEE operations in the
same order: scalar kernels, the vector Linear / Wendland C0 / Wendland C2 kernels, PU weights
(SwarmInterpSetWeights_AVX256), patch assembly (PartitionAssembleRBFMatrix_AVX512) and evaluation
(PointwiseInterpolation_AVX512).  The reference's vector exp (exp_avx.h) is its own polynomial, so
the bump and Gaussian vector kernels agree to within a few ulp there.  Skipped where the LagRBF
source tree or AVX-512F is missing.
"""
import numpy as np
import pytest

import oracle_lib as O
import ref_pin_lib as R
from lagrbf_gb300 import workloads as W

_lib, _why = R.available()
pytestmark = pytest.mark.skipif(_lib is None, reason=str(_why))

ULP = 2.220446049250313e-16


def _radii(n=8000, seed=0):
    rng = np.random.default_rng(seed)
    return np.concatenate([np.linspace(0.0, 2.0, n // 2), rng.uniform(0.0, 2.0, n // 2)])


@pytest.mark.parametrize("kernel", range(7))
def test_scalar_kernels_bit_exact(kernel):
    r = _radii()
    o = np.array([O.lib().orc_phi_scalar(kernel, x, 1.3) for x in r])
    assert np.array_equal(o, R.phi(kernel, 1, r, 1.3))


@pytest.mark.parametrize("kernel", [0, 1, 2, 3, 6])
def test_vector_kernels(kernel):
    r = _radii()
    o = np.array([O.lib().orc_phi_lane(kernel, x, 1.3) for x in r])
    p = R.phi(kernel, 8, r, 1.3)
    if kernel in (0, 1, 2):
        assert np.array_equal(o, p)
        assert np.array_equal(o, R.phi(kernel, 4, r, 1.3))
    else:  # reference Exp_AVX512 polynomial vs libm exp (it flushes subnormal results to zero)
        assert (np.abs(o - p) <= 2 * ULP * np.abs(p) + 1e-300).all()


def test_reference_avx256_exp_quirk():
    """Exp_AVX256 (exp_avx.h:34-102) returns 2*exp(x) for x <= -ln(2)/2 -- a reference defect that
    reaches the Gaussian and bump kernels only through the AVX-256 interpolation/assembly units
    (hosts without AVX-512F).  The oracle and the GPU path follow exp(), like the scalar and
    AVX-512 units."""
    u = np.linspace(0.0, 3.0, 3001)[:3000]
    g4 = R.phi(6, 4, u, 1.0)
    ex = np.exp(-(u * u))
    x = -(u * u)
    hit = x <= -np.log(2.0) / 2 - 1e-9
    assert np.allclose(g4[hit] / ex[hit], 2.0, rtol=1e-13, atol=0)
    assert np.allclose(g4[~hit] / ex[~hit], 1.0, rtol=1e-13, atol=0)
    assert np.allclose(R.phi(6, 8, u, 1.0), ex, rtol=4 * ULP, atol=0)


def _case(dim, npu, nlat, overlap, kernel=2, seed=1, np_=2000):
    rng = np.random.default_rng(seed)
    xd = W.jittered_lattice(nlat, dim, rng)
    fd = W.cellular_flow(xd) if dim == 2 else W.abc_flow(xd)
    xp = W.uniform_points(np_, dim, np.random.default_rng(seed + 1))
    # points on faces, interior node planes and the upper corner
    xp = np.concatenate([xp, [[1.0] * dim, [0.0] * dim, [1.0 / (npu - 1)] * dim, [0.5] * dim]])
    pc = O.Pieces(dim=dim, npartitions=[npu] * dim, nfields=fd.shape[1], overlap=overlap, kernel=kernel)
    return pc, xd, fd, xp


@pytest.mark.parametrize("dim,npu,nlat", [(2, 8, 40), (3, 5, 16), (3, 6, 12)])
@pytest.mark.parametrize("overlap", ["pu", 1.0, 2.5])
def test_weights_bit_exact(dim, npu, nlat, overlap):
    ov = W.pu_overlap(npu) if overlap == "pu" else overlap
    pc, xd, fd, xp = _case(dim, npu, nlat, ov)
    cp = pc.locate(xp)
    assert (cp >= 0).all()
    assert np.array_equal(pc.weights(xp, cp), R.weights(pc, xp, cp))


@pytest.mark.parametrize("dim,npu,nlat", [(2, 8, 40), (3, 5, 16)])
@pytest.mark.parametrize("kernel", [0, 1, 2, 3, 6])
def test_assembly(dim, npu, nlat, kernel):
    pc, xd, fd, xp = _case(dim, npu, nlat, W.pu_overlap(npu), kernel=kernel)
    (cs, cpts), (ps, pp), (bs, bp) = pc.csr(pc.locate(xd))
    for k in (0, pc.nnodes // 2 + 1, pc.nnodes - 1):  # corner, interior, corner patch
        idx = pp[ps[k]:ps[k + 1]]
        a, b = pc.assemble(kernel, idx, xd), R.assemble(pc, kernel, idx, xd)
        if kernel in (0, 1, 2):
            assert np.array_equal(a, b)
        else:
            assert (np.abs(a - b) <= 2 * ULP * np.abs(b) + 1e-300).all()


@pytest.mark.parametrize("dim,npu,nlat", [(2, 8, 40), (3, 5, 16)])
def test_interpolation_bit_exact(dim, npu, nlat):
    pc, xd, fd, xp = _case(dim, npu, nlat, W.pu_overlap(npu))
    cd, cp = pc.locate(xd), pc.locate(xp)
    (cs, cpts), (ps, pp), (bs, bp) = pc.csr(cd)
    w = pc.weights(xp, cp)
    coeffs, coff = pc.solve_all(2, xd, fd, ps, pp)
    nf = fd.shape[1]
    mine = pc.eval(2, xp, cp, w, xd, bs, bp, ps, pp, coeffs, coff, nf, nf)
    ref = R.interpolate(pc, 8, 2, xd, bs, bp, ps, pp, coeffs, coff, nf, xp, cp, w)
    assert np.array_equal(mine, ref)


def test_interpolation_gaussian_within_ulps():
    """Gaussian kernel (eps = 3/h): only the reference's vector exp differs, so the values agree
    to rounding level."""
    dim, npu, nlat = 2, 8, 40
    rng = np.random.default_rng(3)
    xd = W.jittered_lattice(nlat, dim, rng)
    fd = W.cellular_flow(xd)
    xp = W.uniform_points(1500, dim, np.random.default_rng(4))
    pc0 = O.Pieces(dim=dim, npartitions=[npu] * dim, nfields=2, overlap=W.pu_overlap(npu), kernel=6)
    shape = (3.0 * nlat) / pc0.pu.eps_w
    pc = O.Pieces(dim=dim, npartitions=[npu] * dim, nfields=2, overlap=W.pu_overlap(npu), kernel=6,
                  shape_factor=shape)
    cd, cp = pc.locate(xd), pc.locate(xp)
    (cs, cpts), (ps, pp), (bs, bp) = pc.csr(cd)
    w = pc.weights(xp, cp)
    coeffs, coff = pc.solve_all(6, xd, fd, ps, pp)
    mine = pc.eval(6, xp, cp, w, xd, bs, bp, ps, pp, coeffs, coff, 2, 2)
    ref = R.interpolate(pc, 8, 6, xd, bs, bp, ps, pp, coeffs, coff, 2, xp, cp, w)
    assert np.abs(mine - ref).max() / np.abs(ref).max() <= 1e-13
