"""FP64 assembled Poisson matrix and FP64 CG (oracle; test infrastructure only).

``assemble`` restates lib/discrete_laplacian.py:122-160 (lap_with_bc with
bd_padding=True) followed by compressedMat (lib/read_data.py:164-165): the
7-point Laplacian on FLUID cells, whose diagonal counts the non-solid face
neighbours and whose off-diagonals are -1 between fluid face neighbours.
Rows and columns of non-fluid cells are dropped.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

BOUNDARY, SOLID, FLUID, AIR = 0, 1, 2, 3


def assemble(flags: np.ndarray) -> tuple[sp.csr_matrix, np.ndarray]:
    """(A, fluid_cells): A is FP64 CSR over the fluid cells in flat (z-fastest) order."""
    flags = np.asarray(flags)
    n1, n2, n3 = flags.shape
    f = flags.ravel()
    fluid = np.flatnonzero(f == FLUID)
    idx = -np.ones(f.size, dtype=np.int64)
    idx[fluid] = np.arange(fluid.size)
    i, j, k = np.unravel_index(fluid, flags.shape)
    diag = np.zeros(fluid.size)
    rows, cols = [], []
    for di, dj, dk in ((-1, 0, 0), (0, -1, 0), (0, 0, -1), (0, 0, 1), (0, 1, 0), (1, 0, 0)):
        ii, jj, kk = i + di, j + dj, k + dk
        inside = (ii >= 0) & (ii < n1) & (jj >= 0) & (jj < n2) & (kk >= 0) & (kk < n3)
        nb = np.where(inside, (ii * n2 + jj) * n3 + kk, 0)
        fn = np.where(inside, f[nb], SOLID)
        diag += (fn == FLUID) | (fn == AIR)
        m = fn == FLUID
        rows.append(np.flatnonzero(m))
        cols.append(idx[nb[m]])
    r = np.concatenate(rows + [np.arange(fluid.size)])
    c = np.concatenate(cols + [np.arange(fluid.size)])
    v = np.concatenate([-np.ones(sum(len(x) for x in rows)), diag])
    A = sp.csr_matrix((v, (r, c)), shape=(fluid.size, fluid.size))
    A.sort_indices()
    return A, fluid


def apply_grid(flags: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Matrix-free form on full-grid vectors (zero outside fluid cells)."""
    A, fluid = assemble(flags)
    y = np.zeros(flags.size)
    y[fluid] = A @ np.asarray(x, dtype=np.float64).ravel()[fluid]
    return y.reshape(flags.shape)


def cg_fp64(A, b, tol=1e-12, max_it=100000, x0=None):
    """Unpreconditioned FP64 CG to ||b - A x|| <= tol ||b|| (true residual checked)."""
    b = np.asarray(b, dtype=np.float64)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
    r = b - A @ x
    p = r.copy()
    rr = r @ r
    nb = np.linalg.norm(b)
    if nb == 0:
        return x, 0
    for it in range(1, max_it + 1):
        Ap = A @ p
        alpha = rr / (p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        rr_new = r @ r
        if np.sqrt(rr_new) <= tol * nb:
            r = b - A @ x
            rr_new = r @ r
            if np.sqrt(rr_new) <= tol * nb:
                return x, it
        p = r + (rr_new / rr) * p
        rr = rr_new
    return x, max_it
