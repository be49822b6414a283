"""The mixed-boundary Poisson operator of a flag grid.

``FluidLaplacian`` is matrix-free: ``A @ x`` runs the sm_103a 7-point kernel
(mlpcg_laplacian_apply) on full-grid vectors, or scatters / gathers around it
for the compressed fluid-only vectors the reference's solvers use
(test.py:320-321).  ``csr_from_flags`` assembles the same matrix as an FP64
torch CSR tensor, the form the reference builds from the simulator's A_*.bin
(lib/read_data.py:110-165, lib/discrete_laplacian.py:122-160).
"""
from __future__ import annotations

import numpy as np
import torch

from . import ops

BOUNDARY, SOLID, FLUID, AIR = 0, 1, 2, 3


class FluidLaplacian:
    """A such that (A x)(c) = d(c) x(c) - sum_{fluid face nbrs n} x(n) on FLUID cells."""

    def __init__(self, flags: torch.Tensor):
        if flags.dtype != torch.uint8 or flags.dim() != 3:
            raise ValueError("flags must be a (N1, N2, N3) uint8 tensor of flag codes")
        self.flags = flags.contiguous()
        self.shape_grid = tuple(flags.shape)
        self.fluid_cells = torch.nonzero(self.flags.reshape(-1) == FLUID).reshape(-1)
        self.n_fluid = int(self.fluid_cells.numel())
        self.shape = (self.n_fluid, self.n_fluid)
        self.layout = "matrix-free"

    def matvec_grid(self, x: torch.Tensor) -> torch.Tensor:
        """x, result: full-grid (N1, N2, N3) F32 or F64 tensors."""
        return ops.laplacian(self.flags, x.reshape(self.shape_grid).contiguous())

    def __matmul__(self, x: torch.Tensor) -> torch.Tensor:
        n = int(np.prod(self.shape_grid))
        if x.numel() == n and x.numel() != self.n_fluid:
            return self.matvec_grid(x).reshape(x.shape)
        if x.dim() != 1 or x.numel() != self.n_fluid:
            raise RuntimeError(f"vector of size {x.numel()} matches neither the grid ({n}) "
                               f"nor the fluid cells ({self.n_fluid})")
        g = torch.zeros(n, dtype=x.dtype, device=x.device)
        g[self.fluid_cells] = x
        return self.matvec_grid(g).reshape(-1)[self.fluid_cells]


def csr_from_flags(flags_np: np.ndarray, device="cuda", dtype=torch.float64):
    """(A, fluid_cells): FP64 torch sparse CSR over the fluid cells in flat order."""
    f = np.asarray(flags_np)
    n1, n2, n3 = f.shape
    flat = f.ravel()
    fluid = np.flatnonzero(flat == FLUID)
    idx = -np.ones(flat.size, dtype=np.int64)
    idx[fluid] = np.arange(fluid.size)
    i, j, k = np.unravel_index(fluid, f.shape)
    diag = np.zeros(fluid.size)
    rows, cols = [], []
    for di, dj, dk in ((-1, 0, 0), (0, -1, 0), (0, 0, -1), (0, 0, 1), (0, 1, 0), (1, 0, 0)):
        ii, jj, kk = i + di, j + dj, k + dk
        inside = (ii >= 0) & (ii < n1) & (jj >= 0) & (jj < n2) & (kk >= 0) & (kk < n3)
        nb = np.where(inside, (ii * n2 + jj) * n3 + kk, 0)
        fn = np.where(inside, flat[nb], SOLID)
        diag += (fn == FLUID) | (fn == AIR)
        m = fn == FLUID
        rows.append(np.flatnonzero(m))
        cols.append(idx[nb[m]])
    r = np.concatenate(rows + [np.arange(fluid.size)])
    c = np.concatenate(cols + [np.arange(fluid.size)])
    v = np.concatenate([-np.ones(sum(len(a) for a in rows)), diag])
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    indptr = np.zeros(fluid.size + 1, dtype=np.int64)
    np.add.at(indptr, r + 1, 1)
    indptr = np.cumsum(indptr)
    A = torch.sparse_csr_tensor(torch.from_numpy(indptr), torch.from_numpy(c), torch.from_numpy(v),
                                (fluid.size, fluid.size), dtype=dtype, device=device)
    return A, torch.from_numpy(fluid).to(device)
