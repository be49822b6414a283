"""The reference's neural CG iterations in numpy FP64 (oracle; test infrastructure only).

``predict(r) -> z`` plays the role of Tests.model_predict (test.py:42-51).
Each solver returns (x, iterations, history) where history[k] is
||b - A x_k|| / ||b|| after iteration k (history[0] is the initial residual),
the quantity the reference prints and passes to ``callback``.
"""
from __future__ import annotations

import numpy as np


def npcg(b, A, x_init, predict, max_it, tol=1e-10, atol=1e-12):
    """cg_tests.py:26-101."""
    norm_b = np.linalg.norm(b)
    r = b - A @ x_init
    hist = [np.linalg.norm(r) / norm_b]
    x = np.array(x_init, dtype=np.float64)
    z = predict(r)
    p = z
    w = A @ p
    rz = rz_old = r @ z
    alpha = rz / (p @ w)
    x = x + alpha * p
    r = b - A @ x
    norm = np.linalg.norm(r) / norm_b
    hist.append(norm)
    k = 1
    while norm > max(tol, atol / norm_b) and k < max_it:
        z = predict(r)
        rz = r @ z
        beta = rz / rz_old
        p = z + beta * p
        w = A @ p
        alpha = rz / (p @ w)
        x = x + alpha * p
        r = b - A @ x
        k += 1
        rz_old = rz
        norm = np.linalg.norm(r) / norm_b
        hist.append(norm)
    return x, k, hist


def npcg_flex(b, A, x_init, predict, max_it, tol=1e-10, atol=1e-12):
    """cg_tests.py:103-183 (Polak-Ribiere beta)."""
    norm_b = np.linalg.norm(b)
    r = b - A @ x_init
    hist = [np.linalg.norm(r) / norm_b]
    x = np.array(x_init, dtype=np.float64)
    z = predict(r)
    p = z
    w = A @ p
    rz = rz_old = r @ z
    r_old = r
    alpha = rz / (p @ w)
    x = x + alpha * p
    r = b - A @ x
    norm = np.linalg.norm(r) / norm_b
    hist.append(norm)
    k = 1
    while norm > max(tol, atol / norm_b) and k < max_it:
        z = predict(r)
        rz = r @ z
        beta = z @ (r - r_old) / rz_old
        p = z + beta * p
        w = A @ p
        alpha = rz / (p @ w)
        x = x + alpha * p
        r_old = r
        r = b - A @ x
        rz_old = rz
        k += 1
        norm = np.linalg.norm(r) / norm_b
        hist.append(norm)
    return x, k, hist


def npsd(b, A, x_init, predict, max_it, tol=1e-10, atol=1e-10, num_prev=2):
    """cg_tests.py:189-284: preconditioned descent, A-orthogonalised against the
    last ``num_prev`` directions."""
    norm_b = np.linalg.norm(b)
    r = b - A @ x_init
    hist = [np.linalg.norm(r) / norm_b]
    p, Ap, alfa = [], [], []
    x = np.array(x_init, dtype=np.float64)
    norm = hist[0]
    for i in range(1, max_it + 1):
        q = predict(r)
        if i > num_prev:
            for j in reversed(range(num_prev)):
                q = q - (q @ Ap[j]) / alfa[j] * p[j]
            for j in range(num_prev - 1):
                p[j], Ap[j], alfa[j] = p[j + 1], Ap[j + 1], alfa[j + 1]
            p[num_prev - 1] = q
            Ap[num_prev - 1] = A @ q
            alfa[num_prev - 1] = p[-1] @ Ap[-1]
        else:
            for j in reversed(range(i - 1)):
                q = q - (q @ Ap[j]) / alfa[j] * p[j]
            p.append(q)
            Ap.append(A @ q)
            alfa.append(p[-1] @ Ap[-1])
        beta = (p[-1] @ r) / alfa[-1]
        x = x + q * beta
        r = b - A @ x
        norm = np.linalg.norm(r) / norm_b
        hist.append(norm)
        if norm < max(tol, atol / norm_b):
            return x, i, hist
    return x, max_it, hist


def make_predict(model_fn, fluid_cells, shape):
    """Tests.model_predict (test.py:42-51): normalise r in FP32, scatter to the
    grid, run the network, gather the fluid cells back as FP64."""
    n = int(np.prod(shape))

    def predict(r):
        r32 = np.asarray(r, dtype=np.float32)
        r32 = r32 / max(np.linalg.norm(r32), 1e-12)
        g = np.zeros(n, dtype=np.float64)
        g[fluid_cells] = r32
        out = np.asarray(model_fn(g.reshape(shape))).ravel()
        return out[fluid_cells].astype(np.float64)

    return predict
