"""The cell-location scheme of the GPU path, restated on the CPU: the cell index
clamp(floor((x - O) / h), 0, n - 2) per axis equals the number of cell faces at or below x, with
doubles compared through order-preserving integer keys and each face the smallest x whose
floor((x - O) / h) reaches k, found by bisection over the keys (stepping one ulp at a time from
O + k h does not end when a face lies at 0, where the doubles are dense).  The CUDA code builds
the same table in lgb_host.c (build_face_keys) and searches it in lgb_common.cuh (lgb_locate);
the GPU parity test test_locate_at_cell_faces checks that code against the oracle.
"""
import numpy as np
import pytest


def key(v):
    b = np.array([v], dtype=np.float64).view(np.int64)[0]
    if b == np.int64(-2**63):
        b = np.int64(0)
    return int(b) if b >= 0 else int(b ^ np.int64(0x7FFFFFFFFFFFFFFF))


def key_double(k):
    if k < 0:
        k ^= 0x7FFFFFFFFFFFFFFF
    return float(np.array([k], dtype=np.int64).view(np.float64)[0])


def faces(O, L, n):
    """Smallest x in [O, L] with floor((x - O) / h) >= k, k = 1 .. n-2: bisection over the keys."""
    h = (L - O) / (n - 1)
    out = []
    for k in range(1, n - 1):
        lo, hi = key(O), key(L)
        assert np.floor((key_double(hi) - O) / h) >= k
        while hi - lo > 1:
            mid = lo + (hi - lo) // 2
            if np.floor((key_double(mid) - O) / h) >= k:
                hi = mid
            else:
                lo = mid
        out.append(hi)
    return out, h


def locate_keys(x, O, L, n, fk):
    k = key(x)
    if k < key(O) or k > key(L):
        return -1
    return int(np.searchsorted(np.array(fk, dtype=np.int64), k, side="right"))


def locate_fp64(x, O, L, h, n):
    if not (O <= x <= L):
        return -1
    return int(min(max(np.floor((x - O) / h), 0), n - 2))


def test_keys_order_like_doubles():
    vals = [-np.inf, -1e300, -2.0, -1.0, -1e-300, -5e-324, 0.0, 5e-324, 1e-300, 0.5, 1.0, 2.0, 1e300, np.inf]
    ks = [key(v) for v in vals]
    assert ks == sorted(ks) and len(set(ks)) == len(ks)
    assert key(-0.0) == key(0.0)
    assert key(np.nan) > key(np.inf) and key(-np.nan) < key(-np.inf)


@pytest.mark.parametrize("O,L,n", [(0.0, 1.0, 32), (-0.3, 1.7, 7), (-2.0, -0.5, 13), (0.0, 1.0, 160),
                                   (1e-3, 3.0, 1000), (-1e5, 1e5, 97), (-1.0, 1.0, 9)])
def test_face_count_equals_floor(O, L, n):
    fk, h = faces(O, L, n)
    assert all(a <= b for a, b in zip(fk, fk[1:]))
    rng = np.random.default_rng(n)
    pts = list(rng.uniform(O, L, 3000))
    for k in range(n):
        x = O + k * h
        lo = hi = x
        for _ in range(3):
            lo, hi = np.nextafter(lo, -np.inf), np.nextafter(hi, np.inf)
            pts += [x, lo, hi]
    pts += [O, L, np.nextafter(O, -np.inf), np.nextafter(L, np.inf), -0.0, np.nan]
    for x in pts:
        assert locate_keys(x, O, L, n, fk) == locate_fp64(x, O, L, h, n), x
