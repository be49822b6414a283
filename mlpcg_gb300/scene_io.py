"""The reference's on-disk scene files (flags, matrix, vectors) and its
compressed-vector helpers.

Formats (lib/read_data.py:18-26, 41-49, 110-165; lib/write_data.py:11-48):

* ``flags_<frame>.bin``      -- size_t N, then N int32 cell flags (BOUNDARY 0,
  SOLID 1, FLUID 2, AIR 3), flat in the grid's z-fastest order;
* ``div_v_star_<frame>.bin`` / ``pressure_<frame>.bin`` -- size_t N, then N
  doubles (the reference's loader reads the whole file as doubles and drops
  the first, i.e. the header's 8 bytes);
* ``A_<frame>.bin``          -- int32 rows, cols, nnz, outer size, inner size;
  nnz values (double, or float with ``dtype='f'``); the outer index array
  (outer-size int32, Eigen's compressed layout without the closing nnz, or
  rows + 1 entries as the Python writer stores it); nnz inner (column) indices.

The matrix covers every grid cell; ``compressed_mat`` keeps the rows and
columns with entries (the fluid cells), ``compressed_vec`` / ``expand_vec``
move between grid vectors and those fluid-DOF vectors.
"""
from __future__ import annotations

import os

import numpy as np
import scipy.sparse as sparse

BOUNDARY, SOLID, FLUID, AIR = 0, 1, 2, 3


def read_flags(path, dtype="int32") -> np.ndarray:
    """Cell flags of ``flags_<frame>.bin`` (lib/read_data.py:18-26)."""
    with open(path, "rb") as f:
        n = int(np.frombuffer(f.read(8), dtype="<u8")[0])
        flags = np.frombuffer(f.read(4 * n), dtype="<i4", count=n)
    return flags.astype(dtype)


def write_flags(path, flags) -> None:
    """The simulator's flags file: size_t count, then int32 flags."""
    flags = np.ascontiguousarray(np.asarray(flags).ravel(), dtype="<i4")
    with open(path, "wb") as f:
        f.write(np.array([flags.size], dtype="<u8").tobytes())
        f.write(flags.tobytes())


def load_vector(path, normalize=False, dtype="double") -> np.ndarray:
    """A serialised vector (lib/read_data.py:41-49): the file as doubles without the first."""
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    v = np.fromfile(path, dtype=dtype)[1:]
    return v / np.linalg.norm(v) if normalize else v


def write_vector(path, v) -> None:
    """size_t length, then the doubles (lib/write_data.py:11-17)."""
    v = np.ascontiguousarray(np.asarray(v, dtype="<f8").ravel())
    with open(path, "wb") as f:
        f.write(np.array([v.size], dtype="<u8").tobytes())
        f.write(v.tobytes())


def read_matrix(path, dtype="d", sparse_type="csr", shape=None):
    """The matrix of ``A_<frame>.bin`` (lib/read_data.py:110-162) as a scipy CSR / CSC / COO matrix
    (CSC reads the same arrays the reference reads, like ``readA_sparse(..., sparse_type='csc')``)."""
    size = {"d": 8, "f": 4}[dtype]
    with open(path, "rb") as f:
        rows, cols, nnz, outer, _inner = (int(v) for v in np.frombuffer(f.read(20), dtype="<i4"))
        data = np.frombuffer(f.read(size * nnz), dtype="<f8" if dtype == "d" else "<f4", count=nnz)
        outer_idx = np.frombuffer(f.read(4 * outer), dtype="<i4", count=outer)
        inner_idx = np.frombuffer(f.read(4 * nnz), dtype="<i4", count=nnz)
    indptr = np.concatenate([outer_idx[:rows].astype(np.int64), [nnz]])
    shape = (rows, cols) if shape is None else tuple(shape)
    csr = sparse.csr_matrix((data.astype(dtype), inner_idx.astype(np.int64), indptr), shape=shape)
    kind = sparse_type.lower()
    if kind == "csr":
        return csr
    if kind == "csc":
        return csr.tocsc()
    if kind == "coo":
        return csr.tocoo()
    raise ValueError("sparse_type must be csr, csc or coo")


def write_matrix(A, path, dtype="d") -> None:
    """``A_<frame>.bin`` as the reference's Python writer stores it (lib/write_data.py:19-48)."""
    A = sparse.csr_matrix(A)
    A.sort_indices()
    rows, cols = A.shape
    outer = len(A.indptr)
    with open(path, "wb") as f:
        f.write(np.array([rows, cols, A.nnz, outer, outer], dtype="<i4").tobytes())
        f.write(np.asarray(A.data, dtype="<f8" if dtype == "d" else "<f4").tobytes())
        f.write(np.asarray(A.indptr, dtype="<i4").tobytes())
        f.write(np.asarray(A.indices, dtype="<i4").tobytes())


def compressed_mat(A):
    """Rows and columns of A with entries (lib/read_data.py:164-165)."""
    A = sparse.csr_matrix(A)
    return A[A.getnnz(1) > 0][:, A.getnnz(0) > 0]


def compressed_vec(b, flags) -> np.ndarray:
    """The fluid cells' values of a grid vector (lib/read_data.py:166-168)."""
    return np.asarray(b).ravel()[np.flatnonzero(np.asarray(flags).ravel() == FLUID)]


def expand_vec(b, flags) -> np.ndarray:
    """A fluid-DOF vector on the grid, 0 elsewhere (lib/read_data.py:169-174)."""
    flags = np.asarray(flags).ravel()
    v = np.zeros(flags.shape, np.asarray(b).dtype)
    v[np.flatnonzero(flags == FLUID)] = b
    return v


def convert_to_binary_images(flags, num_imgs=3) -> np.ndarray:
    """[air, fluid, non-solid] (or fewer) 0/1 channels (lib/read_data.py:28-39)."""
    flags = np.asarray(flags)
    air = (flags == AIR).astype(np.int64)
    fluid = (flags == FLUID).astype(np.int64)
    nonsolid = (flags > SOLID).astype(np.int64)
    if num_imgs == 1:
        return fluid.reshape((1,) + flags.shape)
    if num_imgs == 2:
        return np.stack([air, nonsolid])
    if num_imgs == 3:
        return np.stack([air, fluid, nonsolid])
    raise ValueError("num_imgs must be 1, 2 or 3")


def load_frame(scene_path, frame, shape):
    """(flags (N1, N2, N3) uint8, fluid-DOF rhs, compressed FP64 CSR matrix) of one frame, as the
    reference's test.py:75-77 loads them."""
    flags = read_flags(os.path.join(scene_path, f"flags_{frame}.bin")).reshape(shape).astype(np.uint8)
    rhs = load_vector(os.path.join(scene_path, f"div_v_star_{frame}.bin"))
    A = compressed_mat(read_matrix(os.path.join(scene_path, f"A_{frame}.bin")))
    if rhs.size == flags.size:
        rhs = compressed_vec(rhs, flags)
    return flags, rhs, A.astype(np.float64)
