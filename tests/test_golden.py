"""The oracle against the golden fixtures of tests/golden/ (outputs of LagRBF's own hot-loop units,
generated by tests/golden/make_golden.py).  Runs anywhere: the fixtures carry the reference's
results, so neither the LagRBF tree nor AVX-512 is needed here."""
import glob
import os

import numpy as np
import pytest

import oracle_lib as O

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz")))


def _load(path):
    g = np.load(path)
    dim, npu, kernel = int(g["dim"]), int(g["npu"]), int(g["kernel"])
    pc = O.Pieces(dim=dim, npartitions=[npu] * dim, nfields=g["fd"].shape[1], overlap=float(g["overlap"]),
                  kernel=kernel, shape_factor=float(g["shape_factor"]))
    return g, pc, kernel


def test_fixtures_present():
    assert len(GOLDEN) >= 3


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_matches_reference_units(path):
    g, pc, kernel = _load(path)
    xd, fd, xp = g["xd"], g["fd"], g["xp"]
    cp = pc.locate(xp)
    assert np.array_equal(cp, g["cellid_p"])
    w = pc.weights(xp, cp)
    assert np.array_equal(w, g["weights_ref"])
    A = pc.assemble(kernel, g["a_idx"], xd)
    (cs, cpts), (ps, pp), (bs, bp) = pc.csr(pc.locate(xd))
    k = int(g["a_patch"])
    assert np.array_equal(pp[ps[k]:ps[k + 1]], g["a_idx"])
    coeffs, coff = pc.solve_all(kernel, xd, fd, ps, pp)
    v = pc.eval(kernel, xp, cp, w, xd, bs, bp, ps, pp, coeffs, coff, fd.shape[1], fd.shape[1])
    if kernel == 6:  # the reference's vector exp differs from exp() by an ulp or two
        assert np.abs(A - g["A_ref"]).max() <= 4.5e-16
        assert np.abs(v - g["values_ref"]).max() / np.abs(g["values_ref"]).max() <= 1e-13
    else:
        assert np.array_equal(A, g["A_ref"])
        assert np.array_equal(v, g["values_ref"])
