"""Training right-hand sides from Lanczos Ritz vectors, on the GPU.

The reference builds them on the CPU (lib/create_dataset.py:28-70): FP64
Lanczos with full reorthogonalisation started from the scene's rhs, then
scipy's eigh_tridiagonal, Ritz vectors = V^T Q.  Here the Lanczos vectors
live on the GPU (FP64), the operator is the matrix-free kernel, and the
reorthogonalisation is two classical Gram-Schmidt passes against all
previous vectors (as robust as the reference's modified Gram-Schmidt loop,
with two matrix-vector products per step instead of j dot products).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg
import torch

from .laplacian import FluidLaplacian


def lanczos_ritz(A: FluidLaplacian, v0: torch.Tensor, steps: int, n_ritz: int, cutoff=1e-10):
    """Lowest ``n_ritz`` Ritz pairs after ``steps`` Lanczos steps: (values (k,), vectors (k, n_fluid) FP64)."""
    n = A.n_fluid
    m = min(steps, n)
    V = torch.empty((m, n), dtype=torch.float64, device=v0.device)
    alpha = np.zeros(m)
    beta = np.zeros(max(m - 1, 0))
    V[0] = v0 / v0.norm()
    w = A @ V[0]
    alpha[0] = float(w @ V[0])
    w = w - alpha[0] * V[0]
    used = m
    for j in range(1, m):
        bj = float(w.norm())
        if bj < cutoff:
            used = j
            break
        beta[j - 1] = bj
        V[j] = w / bj
        w = A @ V[j]
        alpha[j] = float(w @ V[j])
        w = w - alpha[j] * V[j] - bj * V[j - 1]
        for _ in range(2):  # full reorthogonalisation
            w = w - V[: j + 1].T @ (V[: j + 1] @ w)
    alpha, beta = alpha[:used], beta[: used - 1]
    k = min(n_ritz, used)
    vals, Q = scipy.linalg.eigh_tridiagonal(alpha, beta, select="i", select_range=(0, k - 1))
    Qt = torch.as_tensor(Q, device=v0.device)
    ritz = (V[:used].T @ Qt).T.contiguous()
    return vals, ritz


def mix_rhs(ritz: torch.Tensor, batch: int, n_focus: int = 32, focus_weight: float = 9.0, generator=None):
    """Normalised random combinations of Ritz vectors, N(0,1) weights with the
    lowest ``n_focus`` scaled by ``focus_weight`` (the reference weights its
    first 60 % by 9, preprocess.py:44-55)."""
    k = ritz.shape[0]
    w = torch.randn((batch, k), dtype=ritz.dtype, device=ritz.device, generator=generator)
    scale = torch.ones(k, dtype=ritz.dtype, device=ritz.device)
    scale[:n_focus] = focus_weight
    b = (w * scale) @ ritz
    return b / b.norm(dim=1, keepdim=True)
