"""Generates the golden fixtures of this folder from LagRBF's own hot-loop units (compiled unmodified
against the PETSc stand-in of oracle/ref_pin/; needs the LagRBF source tree, named by the
LAGRBF_REFERENCE environment variable, and an AVX-512F host).

Each case stores its seeded inputs and what the reference units return for them:
  weights_ref  SwarmInterpSetWeights_AVX256 (src/swarm/weights_avx.c:97-243), [np, 2^dim]
  A_ref        PartitionAssembleRBFMatrix_AVX512 (src/partitions/partition_asmb_avx512.c:119-198)
               of patch `a_patch` (data indices a_idx), row-major
  values_ref   PointwiseInterpolation_AVX512 (src/interpolation/interpolation_avx512.c:121-291) of
               every field at the particles, from the coefficients of the oracle's patch solves
               (the reference factorises with LAPACK through PETSc, which is not part of its tree)
Membership and cell ids are the oracle's (PETSc's DMLocatePoints / DMSwarmSort are not vendored).

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle_lib as O  # noqa: E402
import ref_pin_lib as R  # noqa: E402
from lagrbf_gb300 import workloads as W  # noqa: E402

CASES = {
    # name: dim, nodes per axis, lattice points per axis, particles, kernel, eps_r*h (None: shape 1)
    "pin_2d_c2": (2, 6, 32, 1000, 2, None),
    "pin_2d_gauss": (2, 6, 32, 1000, 6, 3.0),
    "pin_3d_c2": (3, 4, 12, 800, 2, None),
}


def make(name, dim, npu, nlat, np_, kernel, eps_h, seed=11):
    rng = np.random.default_rng(seed)
    xd = W.jittered_lattice(nlat, dim, rng)
    fd = W.cellular_flow(xd) if dim == 2 else W.abc_flow(xd)
    xp = W.uniform_points(np_, dim, np.random.default_rng(seed + 1))
    xp = np.concatenate([xp, [[1.0] * dim, [0.0] * dim, [1.0 / (npu - 1)] * dim]])
    overlap = W.pu_overlap(npu)
    shape = 1.0
    if eps_h is not None:
        pc0 = O.Pieces(dim=dim, npartitions=[npu] * dim, nfields=fd.shape[1], overlap=overlap, kernel=kernel)
        shape = eps_h * nlat / pc0.pu.eps_w
    pc = O.Pieces(dim=dim, npartitions=[npu] * dim, nfields=fd.shape[1], overlap=overlap, kernel=kernel,
                  shape_factor=shape)
    cd, cp = pc.locate(xd), pc.locate(xp)
    (cs, cpts), (ps, pp), (bs, bp) = pc.csr(cd)
    w = R.weights(pc, xp, cp)
    a_patch = 0
    a_idx = pp[ps[a_patch]:ps[a_patch + 1]].copy()
    A = R.assemble(pc, kernel, a_idx, xd)
    coeffs, coff = pc.solve_all(kernel, xd, fd, ps, pp)
    vals = R.interpolate(pc, 8, kernel, xd, bs, bp, ps, pp, coeffs, coff, fd.shape[1], xp, cp, w)
    out = os.path.join(HERE, name + ".npz")
    np.savez_compressed(out, dim=dim, npu=npu, nlat=nlat, kernel=kernel, overlap=overlap, shape_factor=shape,
                        xd=xd, fd=fd, xp=xp, cellid_p=cp, weights_ref=w, a_patch=a_patch, a_idx=a_idx, A_ref=A,
                        values_ref=vals)
    print("%s: %d data, %d particles, patch %d of %d points -> %s (%d bytes)"
          % (name, len(xd), len(xp), a_patch, len(a_idx), out, os.path.getsize(out)))


if __name__ == "__main__":
    lib, why = R.available()
    if lib is None:
        sys.exit("reference pin unavailable: %s" % why)
    for name, args in CASES.items():
        make(name, *args)
