"""The drop-in driver's C PETSc-binary layer (host/petsc_bin.c) against the Python
reader/writer: both index widths, the tutorial operator with its trailing
objects, the dense-as-AIJ output of MatView, vectors, and a throughput
figure for a matrix of 5M nonzeros (printed; the parallel byte swap and
block writes should keep it well above 500 MB/s here)."""
import os
import subprocess
import time

import numpy as np
import pytest
import scipy.sparse as sp

from rsvdt import petsc_io, synth

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HOST = os.path.join(ROOT, "rsvd-delta-t_gb300", "host")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("bin") / "petsc_bin_check")
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-fopenmp", "-I", HOST, os.path.join(HERE, "petsc_bin_check.c"),
                    os.path.join(HOST, "petsc_bin.c"), "-o", exe], check=True)
    return exe


def run(checker, *args):
    r = subprocess.run([checker, *args], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return r.stdout.split()


@pytest.mark.parametrize("index_bytes", [4, 8])
def test_sparse_read_then_dense_write(checker, tmp_path, index_bytes):
    A = (synth.gl_operator(40) + sp.random(40, 40, density=0.1, random_state=3)).tocsr()
    src, dst = str(tmp_path / "A"), str(tmp_path / "D")
    petsc_io.write_mat(src, A, index_bytes=index_bytes)
    rows, cols, nnz = map(int, run(checker, "mat", src, dst)[:3])
    assert (rows, cols, nnz) == (40, 40, A.nnz)
    D = petsc_io.read_mat(dst)
    assert D.nnz == 1600  # every entry present, as MatView writes a dense matrix
    assert np.array_equal(D.toarray(), A.toarray())


def test_tutorial_operator_with_trailing_objects(checker, tmp_path):
    src = os.path.join(HERE, "golden", "A_GL")
    dst = str(tmp_path / "D")
    rows, cols, nnz = map(int, run(checker, "mat", src, dst)[:3])
    assert (rows, cols, nnz) == (500, 500, 2000)
    assert np.array_equal(petsc_io.read_mat(dst).toarray(), petsc_io.read_mat(src).toarray())


def test_vector_round_trip_and_truncation(checker, tmp_path):
    v = synth.complex_normal(1001, 1, 4)[:, 0]
    src, dst = str(tmp_path / "v"), str(tmp_path / "w")
    petsc_io.write_vec(src, v)
    assert int(run(checker, "vec", src, dst)[0]) == 1001
    assert np.array_equal(petsc_io.read_vec(dst), v)
    raw = open(src, "rb").read()
    open(src, "wb").write(raw[:-8])
    r = subprocess.run([checker, "vec", src, dst], capture_output=True, text=True)
    assert r.returncode != 0 and "truncated" in r.stderr


def test_read_and_write_throughput(checker, tmp_path):
    """200,000 x 25 matrix with every entry stored (5M nonzeros, 120 MB of
    file): the C reader and the dense writer against the Python reader."""
    M = sp.random(200_000, 25, density=1.0, random_state=2, format="csr").astype(np.complex128)
    src, dst = str(tmp_path / "tall"), str(tmp_path / "tall_d")
    petsc_io.write_mat(src, M, index_bytes=8)
    mb = os.path.getsize(src) / 1e6
    t0 = time.perf_counter()
    petsc_io.read_mat(src)
    t_py = time.perf_counter() - t0
    out = run(checker, "mat", src, dst)
    t_read, t_write = float(out[3]), float(out[4])
    print(f"C reader {mb / t_read:.0f} MB/s, C dense writer {os.path.getsize(dst) / 1e6 / t_write:.0f} MB/s, "
          f"Python reader {mb / t_py:.0f} MB/s")
    assert np.array_equal(petsc_io.read_mat(dst).toarray(), M.toarray())
    assert mb / t_read > 200
