"""The GPU's arithmetic schemes that depart from a textbook operation order, restated in numpy and
checked on the CPU (the CUDA code itself is checked against the oracle by the GPU parity tests):

- the triangular solves of lgb_factor.cu on the "prepared" factor: 32 x 32 diagonal blocks holding
  1/L(j,j) on the diagonal and M(i,j) = L(i,j)/L(j,j) below it, FMA-only substitution inside a
  block, rows below the block updated in the forward sweep and rows above it in the backward sweep;
- the CFL step of lgb_step.cu: min_p c / (sqrt(|v_p|^2) + 1e-16) evaluated once at max_p |v_p|^2,
  bit for bit, because every step of the expression is a correctly rounded monotone function.
"""
import numpy as np
import pytest


def prepared(L):
    m = L.shape[0]
    P = L.copy()
    for j in range(m):
        iend = min((j // 32 + 1) * 32, m)
        P[j + 1:iend, j] /= L[j, j]
    P[np.arange(m), np.arange(m)] = 1.0 / np.diag(L)
    return P


def solve_prepared(P, B):
    """chol_solve_group: B is (FC, m); lanes of a warp are the 32 rows of a block."""
    B = B.copy()
    m = P.shape[0]
    nblk = (m + 31) // 32
    for kb in range(nblk):
        j0, nb = 32 * kb, min(32, m - 32 * kb)
        u = B[:, j0:j0 + nb].copy()
        for jj in range(nb - 1):
            mcol = np.where(np.arange(nb) > jj, P[j0:j0 + nb, j0 + jj], 0.0)
            u = u - mcol[None, :] * u[:, jj:jj + 1]
        y = u * np.diag(P)[j0:j0 + nb][None, :]
        B[:, j0:j0 + nb] = y
        B[:, j0 + nb:] -= y @ P[j0 + nb:, j0:j0 + nb].T
    for kb in range(nblk - 1, -1, -1):
        i0, nb = 32 * kb, min(32, m - 32 * kb)
        w = B[:, i0:i0 + nb] * np.diag(P)[i0:i0 + nb][None, :]
        for ii in range(nb - 1, 0, -1):
            mrow = np.where(np.arange(nb) < ii, P[i0 + ii, i0:i0 + nb], 0.0)
            w = w - mrow[None, :] * w[:, ii:ii + 1]
        B[:, i0:i0 + nb] = w
        B[:, :i0] -= w @ P[i0:i0 + nb, :i0]
    return B


@pytest.mark.parametrize("m", [1, 5, 31, 32, 33, 64, 97, 200])
@pytest.mark.parametrize("fc", [1, 3, 4])
def test_prepared_factor_solve(m, fc):
    rng = np.random.default_rng(m * 10 + fc)
    A = rng.standard_normal((m, m))
    A = A @ A.T + m * np.eye(m)
    B = rng.standard_normal((fc, m))
    X = solve_prepared(prepared(np.linalg.cholesky(A)), B)
    ref = np.linalg.solve(A, B.T).T
    assert np.abs(X - ref).max() <= 1e-12 * np.abs(ref).max()


def test_prepared_factor_solve_rbf_system():
    """A Wendland C2 collocation matrix of a jittered 3D lattice patch (the shape the GPU solves)."""
    rng = np.random.default_rng(7)
    g = np.stack(np.meshgrid(*[np.arange(7)] * 3, indexing="ij"), -1).reshape(-1, 3) / 6.0
    x = g + rng.uniform(-0.04, 0.04, g.shape)
    r = np.linalg.norm(x[:, None, :] - x[None, :, :], axis=-1)
    u = np.maximum(1.0 - 2.5 * r, 0.0)
    A = u ** 4 * (4.0 * (1.0 - u) + 1.0)
    F = np.sin(3 * x).T
    X = solve_prepared(prepared(np.linalg.cholesky(A)), F)
    ref = np.linalg.solve(A, F.T).T
    assert np.abs(A @ X.T - F.T).max() <= 1e-10 * np.abs(F).max()
    assert np.abs(X - ref).max() <= 1e-8 * np.abs(ref).max()


def test_cfl_step_from_largest_squared_speed():
    rng = np.random.default_rng(3)
    c = 0.3 * (1.0 / 21.3)
    for scale in (1e-3, 1.0, 1e3):
        v = rng.standard_normal((20000, 3)) * scale
        v[:5] = 0.0
        n2 = np.zeros(len(v))
        for d in range(3):
            n2 = n2 + v[:, d] * v[:, d]
        per_particle = c / (np.sqrt(n2) + 1e-16)
        once = c / (np.sqrt(n2.max()) + 1e-16)
        assert per_particle.min() == once
