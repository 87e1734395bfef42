"""Times the oracle port (the build the CPU baseline runs) against LagRBF's own hot-loop units on
the same inputs -- test infrastructure, x86-64 hosts with AVX-512F and the LagRBF source tree only.

Case: 45^3 jittered lattice (91,125 points, ABC flow), 12^3 patches, Wendland C2, 3 fields,
4,000 uniform particles.  Printed: best-of-5 wall time of one call of
  - PU weights: SwarmInterpSetWeights_AVX256 (weights_avx.c) vs orc_weights,
  - evaluation: PointwiseInterpolation_AVX512 (interpolation_avx512.c) vs orc_eval,
for the strict parity build and the fast build of the oracle.

    LAGRBF_REFERENCE=<LagRBF checkout> python oracle/ref_pin/time_units.py
"""
import ctypes
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, ROOT)

import oracle_lib as O  # noqa: E402
import ref_pin_lib as R  # noqa: E402
from lagrbf_gb300 import workloads as W  # noqa: E402


def best(f, n=5):
    t_min = 1e9
    for _ in range(n):
        t = time.perf_counter()
        f()
        t_min = min(t_min, time.perf_counter() - t)
    return t_min


def main():
    pin, why = R.available()
    if pin is None:
        print("reference units unavailable:", why)
        return 0
    strict = O.lib()
    fast = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "liblagrbf_oracle_fast.so"))
    for name in ("orc_weights", "orc_eval"):
        getattr(fast, name).argtypes = getattr(strict, name).argtypes
        getattr(fast, name).restype = getattr(strict, name).restype

    dim, npu, nlat, npart = 3, 12, 45, 4000
    xd = W.jittered_lattice(nlat, dim, np.random.default_rng(1))
    fd = W.abc_flow(xd)
    xp = W.uniform_points(npart, dim, np.random.default_rng(2))
    pc = O.Pieces(dim=dim, npartitions=[npu] * dim, nfields=3, overlap=W.pu_overlap(npu), kernel=2)
    cd, cp = pc.locate(xd), pc.locate(xp)
    _, (ps, pp), (bs, bp) = pc.csr(cd)
    coeffs, coff = pc.solve_all(2, xd, fd, ps, pp)
    w = pc.weights(xp, cp)
    xflat = np.ascontiguousarray(xp).reshape(-1)

    def weights_with(lib):
        out = np.zeros(npart * 8)
        lib.orc_weights(ctypes.byref(pc.pu), npart, xflat, cp, None, out)

    def eval_with(lib):
        O._lib = lib
        try:
            pc.eval(2, xp, cp, w, xd, bs, bp, ps, pp, coeffs, coff, 3, 3)
        finally:
            O._lib = strict

    print("case: %d^3 lattice (%d points), %d^3 patches, Wendland C2, 3 fields, %d particles"
          % (nlat, len(xd), npu, npart))
    print("weights    : reference AVX-256 unit %.4f s | oracle strict %.4f s | oracle fast %.4f s"
          % (best(lambda: R.weights(pc, xp, cp)), best(lambda: weights_with(strict)), best(lambda: weights_with(fast))))
    print("evaluation : reference AVX-512 unit %.4f s | oracle strict %.4f s | oracle fast %.4f s"
          % (best(lambda: R.interpolate(pc, 8, 2, xd, bs, bp, ps, pp, coeffs, coff, 3, xp, cp, w)),
             best(lambda: eval_with(strict)), best(lambda: eval_with(fast))))
    return 0


if __name__ == "__main__":
    sys.exit(main())
