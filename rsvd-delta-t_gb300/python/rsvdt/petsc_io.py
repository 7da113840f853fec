"""PETSc binary matrix / vector files (the reference's input and output
format: MatLoad/MatView/VecLoad through PetscViewerBinary, e.g.
SourceCode/LNSStructure.c:23-26, SourceCode/SaveResults.c:32-85).

Layout (big-endian): a Mat starts with [classid 1211216, M, N, nz] as
PetscInt (int32, or int64 in a --with-64-bit-indices build), then M row
lengths, nz column indices and nz scalars. A dense matrix viewed by MatView
is written in the same AIJ layout with every entry present. A Vec is
[classid 1211214, n] followed by n scalars. Scalars are complex128 in the
reference's complex build. Only the first object of a file is read: files
written from MATLAB carry trailing objects (the tutorial's A_GL has 384
trailing bytes), which MatLoad ignores as well.
"""
from __future__ import annotations

import struct

import numpy as np
import scipy.sparse as sp

MAT_CLASSID = 1211216
VEC_CLASSID = 1211214


class PetscFormatError(ValueError):
    pass


def _int_width(buf: bytes, classid: int) -> int:
    if len(buf) >= 4 and struct.unpack(">i", buf[:4])[0] == classid:
        return 4
    if len(buf) >= 8 and struct.unpack(">q", buf[:8])[0] == classid:
        return 8
    raise PetscFormatError("not a PETSc binary object of the expected class")


def _ints(buf, off, n, w):
    dt = ">i4" if w == 4 else ">i8"
    need = off + n * w
    if need > len(buf):
        raise PetscFormatError("file truncated")
    return np.frombuffer(buf, dtype=dt, count=n, offset=off).astype(np.int64), need


def _scalars(buf, off, n, complex_scalars=True):
    dt = ">c16" if complex_scalars else ">f8"
    size = 16 if complex_scalars else 8
    need = off + n * size
    if need > len(buf):
        raise PetscFormatError("file truncated")
    return np.frombuffer(buf, dtype=dt, count=n, offset=off).astype(np.complex128), need


def read_mat_bytes(buf: bytes, complex_scalars: bool = True) -> sp.csr_matrix:
    w = _int_width(buf, MAT_CLASSID)
    hdr, off = _ints(buf, 0, 4, w)
    _, M, N, nz = (int(x) for x in hdr)
    if M < 0 or N < 0:
        raise PetscFormatError("negative matrix size")
    if nz == -1:  # MATRIX_BINARY_FORMAT_DENSE
        vals, off = _scalars(buf, off, M * N, complex_scalars)
        return sp.csr_matrix(vals.reshape(M, N))
    rl, off = _ints(buf, off, M, w)
    if rl.sum() != nz or (rl < 0).any():
        raise PetscFormatError("row lengths do not sum to nz")
    ci, off = _ints(buf, off, nz, w)
    if nz and (ci.min() < 0 or ci.max() >= N):
        raise PetscFormatError("column index out of range")
    vals, off = _scalars(buf, off, nz, complex_scalars)
    indptr = np.concatenate([[0], np.cumsum(rl)]).astype(np.int64)
    A = sp.csr_matrix((vals, ci, indptr), shape=(M, N))
    return A


def read_mat(path: str, complex_scalars: bool = True) -> sp.csr_matrix:
    with open(path, "rb") as f:
        return read_mat_bytes(f.read(), complex_scalars)


def write_mat(path: str, A, index_bytes: int = 8) -> None:
    """Writes A (scipy sparse or dense array) in PETSc AIJ binary layout. A
    dense array is written with every entry present, as MatView does."""
    it = ">i8" if index_bytes == 8 else ">i4"
    if sp.issparse(A):
        A = A.tocsr()
        A.sort_indices()
        M, N = A.shape
        rl = np.diff(A.indptr)
        ci = A.indices
        vals = A.data.astype(np.complex128)
    else:
        A = np.asarray(A, dtype=np.complex128)
        M, N = A.shape
        rl = np.full(M, N)
        ci = np.tile(np.arange(N), M)
        vals = A.reshape(-1)  # row-major
    with open(path, "wb") as f:
        f.write(np.array([MAT_CLASSID, M, N, int(rl.sum())], dtype=it).tobytes())
        f.write(np.asarray(rl, dtype=it).tobytes())
        f.write(np.asarray(ci, dtype=it).tobytes())
        f.write(np.asarray(vals, dtype=">c16").tobytes())


def read_vec(path: str, complex_scalars: bool = True) -> np.ndarray:
    with open(path, "rb") as f:
        buf = f.read()
    w = _int_width(buf, VEC_CLASSID)
    hdr, off = _ints(buf, 0, 2, w)
    n = int(hdr[1])
    vals, _ = _scalars(buf, off, n, complex_scalars)
    return vals


def write_vec(path: str, v: np.ndarray, index_bytes: int = 8) -> None:
    it = ">i8" if index_bytes == 8 else ">i4"
    v = np.asarray(v, dtype=np.complex128)
    with open(path, "wb") as f:
        f.write(np.array([VEC_CLASSID, v.size], dtype=it).tobytes())
        f.write(v.astype(">c16").tobytes())
