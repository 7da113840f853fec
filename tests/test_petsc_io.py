"""PETSc binary format (the reference's file interface): the tutorial
operator A_GL with its trailing objects, round trips, index widths, dense
matrices in AIJ layout, vectors, and corrupt files."""
import os
import struct

import numpy as np
import pytest
import scipy.sparse as sp

from rsvdt import petsc_io, synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_reads_tutorial_operator_and_ignores_trailing_objects():
    path = os.path.join(GOLDEN, "A_GL")
    raw = open(path, "rb").read()
    assert struct.unpack(">4q", raw[:32]) == (1211216, 500, 500, 2000)
    A = petsc_io.read_mat(path)
    assert A.shape == (500, 500) and A.nnz == 2000
    assert (np.diff(A.indptr) == 4).all()
    body = 32 + 8 * 500 + 8 * 2000 + 16 * 2000
    assert len(raw) - body == 384  # four trailing Vec objects from MATLAB
    vals = np.frombuffer(raw, ">c16", 2000, 32 + 8 * 2500)
    assert np.array_equal(A.data, vals.astype(complex))


@pytest.mark.parametrize("index_bytes", [4, 8])
def test_sparse_round_trip(tmp_path, index_bytes):
    A = synth.gl_operator(50) + sp.random(50, 50, density=0.05, random_state=1)
    p = tmp_path / "A"
    petsc_io.write_mat(str(p), A, index_bytes=index_bytes)
    B = petsc_io.read_mat(str(p))
    assert (abs(A - B) > 0).nnz == 0


def test_dense_matrix_is_written_as_full_aij(tmp_path):
    # MatView of a dense matrix writes every entry in AIJ layout.
    M = synth.complex_normal(7, 3, 1)
    p = tmp_path / "S"
    petsc_io.write_mat(str(p), M)
    raw = open(p, "rb").read()
    assert struct.unpack(">4q", raw[:32]) == (1211216, 7, 3, 21)
    assert np.allclose(petsc_io.read_mat(str(p)).toarray(), M)


def test_vector_round_trip(tmp_path):
    v = synth.complex_normal(11, 1, 2)[:, 0]
    p = tmp_path / "v"
    petsc_io.write_vec(str(p), v)
    assert np.array_equal(petsc_io.read_vec(str(p)), v)


def test_corrupt_files_are_rejected(tmp_path):
    A = synth.gl_operator(20)
    p = tmp_path / "A"
    petsc_io.write_mat(str(p), A)
    raw = open(p, "rb").read()
    (tmp_path / "trunc").write_bytes(raw[:-40])
    with pytest.raises(petsc_io.PetscFormatError):
        petsc_io.read_mat(str(tmp_path / "trunc"))
    (tmp_path / "bad").write_bytes(b"\x00" * 64)
    with pytest.raises(petsc_io.PetscFormatError):
        petsc_io.read_mat(str(tmp_path / "bad"))
