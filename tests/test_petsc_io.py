"""PETSc binary Vec / IS files (lagrbf_petsc_*): byte layout of the PETSc binary viewer format
(big-endian class id, 32-bit length, big-endian payload), block size in the .info side file,
round trips, and the errors of bad or truncated files.  Host only."""
import struct

import numpy as np
import pytest

from lagrbf_gb300 import petsc_io as P

VEC, IS = 1211214, 1211218


def test_vec_bytes_and_info(tmp_path):
    f = tmp_path / "v.pbvec"
    a = np.array([[1.5, -2.0, 3.25], [0.0, 1e-300, -7.0]])
    P.write_vec(f, a)
    raw = f.read_bytes()
    assert struct.unpack(">ii", raw[:8]) == (VEC, 6)
    assert np.array_equal(np.frombuffer(raw[8:], dtype=">f8"), a.ravel())
    assert (tmp_path / "v.pbvec.info").read_text().split() == ["-vecload_block_size", "3"]
    assert np.array_equal(P.read_vec(f), a)


def test_vec_written_elsewhere_is_read(tmp_path):
    """A file laid out by hand the way PETSc's VecView writes it."""
    f = tmp_path / "w.pbvec"
    vals = np.linspace(-1, 1, 8)
    f.write_bytes(struct.pack(">ii", VEC, 8) + vals.astype(">f8").tobytes())
    (tmp_path / "w.pbvec.info").write_text("-vecload_block_size 2\n")
    assert np.array_equal(P.read_vec(f), vals.reshape(4, 2))
    (tmp_path / "w.pbvec.info").unlink()
    assert np.array_equal(P.read_vec(f), vals)


def test_is_roundtrip_and_range(tmp_path):
    f = tmp_path / "p.pbis"
    idx = np.array([5, 1, 2**31 - 1, -3, 0])
    P.write_is(f, idx)
    raw = f.read_bytes()
    assert struct.unpack(">ii", raw[:8]) == (IS, 5)
    assert np.array_equal(np.frombuffer(raw[8:], dtype=">i4"), idx)
    assert np.array_equal(P.read_is(f), idx)
    with pytest.raises(RuntimeError, match="32-bit"):
        P.write_is(f, [2**31])


def test_bad_files(tmp_path):
    f = tmp_path / "bad.pbvec"
    f.write_bytes(struct.pack(">ii", IS, 2) + b"\0" * 8)
    with pytest.raises(RuntimeError, match="not a PETSc binary Vec"):
        P.read_vec(f)
    f.write_bytes(struct.pack(">ii", VEC, 4) + b"\0" * 8)
    with pytest.raises(RuntimeError, match="truncated"):
        P.read_vec(f)
    with pytest.raises(RuntimeError, match="cannot open"):
        P.read_vec(tmp_path / "missing.pbvec")


def test_large_vector_roundtrip(tmp_path):
    a = np.random.default_rng(0).standard_normal((100_003, 3))
    P.write_vec(tmp_path / "big.pbvec", a)
    assert np.array_equal(P.read_vec(tmp_path / "big.pbvec"), a)
