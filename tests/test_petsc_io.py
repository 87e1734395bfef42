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


def test_lagrbfpy_named_vec_functions(tmp_path):
    """PetscVecWrite / PetscVecLoad (lagrbfpy's names): .info always written, 2D reshaped, files
    interchangeable with the library's own reader and writer."""
    a = np.random.default_rng(1).standard_normal((50, 3))
    f = tmp_path / "v.pbvec"
    P.PetscVecWrite(f, a)
    assert (tmp_path / "v.pbvec.info").read_text() == "-vecload_block_size 3\n"
    assert np.array_equal(P.PetscVecLoad(f), a)
    assert np.array_equal(P.PetscVecLoadFromFile(f), a.ravel())
    assert np.array_equal(P.read_vec(f), a)
    g = tmp_path / "w.pbvec"
    P.write_vec(g, a)
    assert np.array_equal(P.PetscVecLoad(g), a)
    b = np.arange(7.0)
    P.PetscVecWrite(tmp_path / "b.pbvec", b)
    assert (tmp_path / "b.pbvec.info").read_text() == "-vecload_block_size 1\n"
    assert np.array_equal(P.PetscVecLoad(tmp_path / "b.pbvec"), b.reshape(-1, 1))
    P.PetscVecWriteToFile(tmp_path / "c.pbvec", b)
    assert np.array_equal(P.PetscVecLoad(tmp_path / "c.pbvec"), b)  # no .info: flat
    (tmp_path / "bad.info").write_text("-other 3\n")
    with pytest.raises(ValueError):
        P.PetscVecLoadBlockSizeFromFile(tmp_path / "bad.info")


def test_lagrbfpy_named_is_and_mat_functions(tmp_path):
    idx = np.array([5, 0, 2**31 - 1, 7])
    P.PetscISWriteToFile(tmp_path / "i.pbis", idx)
    r = P.PetscISLoadFromFile(tmp_path / "i.pbis")
    assert r.dtype == np.int32 and np.array_equal(r, idx)
    assert np.array_equal(P.read_is(tmp_path / "i.pbis"), idx)
    with pytest.raises(ValueError):
        P.PetscISWriteToFile(tmp_path / "j.pbis", [2**31])
    # AIJ layout: 2 x 3 with entries (0,1)=1.5, (1,0)=-2, (1,2)=4
    m = tmp_path / "m.pbmat"
    with open(m, "wb") as fp:
        np.array([1211216, 2, 3, 3], dtype=">i4").tofile(fp)
        np.array([1, 2], dtype=">i4").tofile(fp)
        np.array([1, 0, 2], dtype=">i4").tofile(fp)
        np.array([1.5, -2.0, 4.0], dtype=">f8").tofile(fp)
    assert np.array_equal(P.PetscMatDenseLoadFromFile(m), np.array([[0, 1.5, 0], [-2.0, 0, 4.0]]))
    d = tmp_path / "d.pbmat"
    with open(d, "wb") as fp:
        np.array([1211216, 2, 2, -1], dtype=">i4").tofile(fp)
        np.array([1.0, 2.0, 3.0, 4.0], dtype=">f8").tofile(fp)
    assert np.array_equal(P.PetscMatDenseLoadFromFile(d), np.array([[1.0, 2.0], [3.0, 4.0]]))
    with pytest.raises(ValueError):
        P.PetscMatDenseLoadFromFile(tmp_path / "i.pbis")
