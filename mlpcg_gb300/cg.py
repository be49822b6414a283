"""Drop-in neural CG solvers: npcg, npcg_flex, npsd (cg_tests.py:26-284) and
model_predict (test.py:42-51).

Same signatures and return values as the reference:
``solver(b, A, x_init, model_predict, max_it, tol, atol, verbose, callback)
-> (x, iterations, timer, relative_residual)``.  ``A`` may be the reference's
torch sparse CSR tensor or a ``laplacian.FluidLaplacian`` (matrix-free
sm_103a kernel).  These keep the reference's precision split (FP64 vectors,
FP32 network) and its per-iteration host synchronisation, so they are the
plain drop-in; ``solver.FusedSolver`` is the graph-captured fast path.
"""
from __future__ import annotations

import time

import numpy as np
import torch
from torch.nn.functional import normalize

from .clock import GlobalClock


def _sync():
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def npcg(b, A, x_init, model_predict, max_it, tol=1e-10, atol=1e-12, verbose=False, callback=None):
    """Preconditioned CG with a (possibly non-symmetric) network preconditioner (cg_tests.py:26-101)."""
    timer = GlobalClock()
    timer.start("Total")
    timer.start("Init")
    norm_b = b.norm().item()
    r = b - A @ x_init
    norm = r.norm().item() / norm_b
    if callback:
        _sync()
        callback(norm, time.perf_counter() - timer.top_level_clocks["Total"].start)
    if verbose:
        print(f"Iter {0}, residual {norm}, ares {r.norm().item()}")
    x = torch.clone(x_init)
    _sync()
    timer.stop("Init")

    timer.start("NN")
    z = model_predict(r, timer)
    _sync()
    timer.stop("NN")

    timer.start("CG")
    p = z
    w = A @ p
    rz = rz_old = r.dot(z)
    alpha = rz / p.dot(w)
    x += alpha * p
    r = b - A @ x
    _sync()
    timer.stop("CG")

    timer.start("Norm")
    norm = r.norm().item() / norm_b
    if callback:
        _sync()
        callback(norm, time.perf_counter() - timer.top_level_clocks["Total"].start)
    _sync()
    timer.stop("Norm")

    k = 1
    while norm > max(tol, atol / norm_b) and k < max_it:
        timer.start("NN")
        z = model_predict(r, timer)
        _sync()
        timer.stop("NN")
        timer.start("CG")
        rz = r.dot(z)
        beta = rz / rz_old
        p = z + beta * p
        w = A @ p
        alpha = rz / p.dot(w)
        x += alpha * p
        r = b - A @ x
        k += 1
        rz_old = rz
        _sync()
        timer.stop("CG")
        timer.start("Norm")
        norm = r.norm().item() / norm_b
        _sync()
        timer.stop("Norm")
        if callback:
            _sync()
            callback(norm, time.perf_counter() - timer.top_level_clocks["Total"].start)
        if verbose:
            print(f"Iter {k}, residual {norm}, ares {r.norm().item()}")
    _sync()
    timer.stop("Total")
    return x, k, timer, norm


def npcg_flex(b, A, x_init, model_predict, max_it, tol=1e-10, atol=1e-12, verbose=False, callback=None):
    """Flexible PCG, Polak-Ribiere beta (cg_tests.py:103-183)."""
    timer = GlobalClock()
    timer.start("Total")
    timer.start("Init")
    norm_b = b.norm().item()
    r = b - A @ x_init
    norm = r.norm().item() / norm_b
    if callback:
        _sync()
        callback(norm, time.perf_counter() - timer.top_level_clocks["Total"].start)
    if verbose:
        print(f"Iter {0}, residual {norm}, ares {r.norm().item()}")
    x = torch.clone(x_init)
    _sync()
    timer.stop("Init")
    timer.start("NN")
    z = model_predict(r, timer)
    _sync()
    timer.stop("NN")
    timer.start("CG")
    p = z
    w = A @ p
    rz = rz_old = r.dot(z)
    r_old = r
    alpha = rz / p.dot(w)
    x += alpha * p
    r = b - A @ x
    _sync()
    timer.stop("CG")
    timer.start("Norm")
    norm = r.norm().item() / norm_b
    if callback:
        _sync()
        callback(norm, time.perf_counter() - timer.top_level_clocks["Total"].start)
    _sync()
    timer.stop("Norm")
    k = 1
    while norm > max(tol, atol / norm_b) and k < max_it:
        timer.start("NN")
        z = model_predict(r, timer)
        _sync()
        timer.stop("NN")
        timer.start("CG")
        rz = r.dot(z)
        beta = z.dot(r - r_old) / rz_old
        p = z + beta * p
        w = A @ p
        alpha = rz / p.dot(w)
        x += alpha * p
        r_old = r
        r = b - A @ x
        rz_old = rz
        k += 1
        _sync()
        timer.stop("CG")
        timer.start("Norm")
        norm = r.norm().item() / norm_b
        _sync()
        timer.stop("Norm")
        if callback:
            _sync()
            callback(norm, time.perf_counter() - timer.top_level_clocks["Total"].start)
        if verbose:
            print(f"Iter {k}, residual {norm}, ares {r.norm().item()}")
    _sync()
    timer.stop("Total")
    return x, k, timer, norm


def npsd(b, A, x_init, model_predict, max_it, tol=1e-10, atol=1e-10, verbose=False, callback=None):
    """Neural-preconditioned steepest descent, A-orthogonalised against the last
    two directions (cg_tests.py:189-284); the solver of test.py:327-328."""
    timer = GlobalClock()
    timer.start("Total")
    timer.start("Init")
    norm_b = b.norm().item()
    r = b - A @ x_init
    norm = r.norm().item() / norm_b
    if callback:
        _sync()
        callback(norm, time.perf_counter() - timer.top_level_clocks["Total"].start)
    if verbose:
        print(f"Iter {0}, residual {norm}, ares {r.norm().item()}")
    num_prev = 2
    p, Ap, alfa = [], [], []
    x_sol = torch.clone(x_init)
    imgs, c0, c1 = [], [], []
    _sync()
    timer.stop("Init")
    for i in range(1, max_it + 1):
        timer.start("NN")
        q = model_predict(r, timer, imgs, c0, c1)
        _sync()
        timer.stop("NN")
        timer.start("Ortho")
        if i > num_prev:
            for j in reversed(range(num_prev)):
                q = q - q.dot(Ap[j]) / alfa[j] * p[j]
            for j in range(num_prev - 1):
                p[j], Ap[j], alfa[j] = p[j + 1], Ap[j + 1], alfa[j + 1]
        else:
            for j in reversed(range(i - 1)):
                q = q - q.dot(Ap[j]) / alfa[j] * p[j]
        _sync()
        timer.stop("Ortho")
        timer.start("CG")
        if i > num_prev:
            p[num_prev - 1] = q
            Ap[num_prev - 1] = A @ q
            alfa[num_prev - 1] = p[-1].dot(Ap[-1])
        else:
            p.append(q)
            Ap.append(A @ q)
            alfa.append(p[-1].dot(Ap[-1]))
        beta = p[-1].dot(r) / alfa[-1]
        x_sol += q * beta
        r = b - A @ x_sol
        _sync()
        timer.stop("CG")
        timer.start("Norm")
        norm = r.norm().item() / norm_b
        if callback:
            _sync()
            callback(norm, time.perf_counter() - timer.top_level_clocks["Total"].start)
        if verbose:
            print(f"Iter {i}, residual {norm}, ares {r.norm().item()}")
        stop = norm < max(tol, atol / norm_b)
        _sync()
        timer.stop("Norm")
        if stop:
            _sync()
            timer.stop("Total")
            return x_sol, i, timer, norm
    _sync()
    timer.stop("Total")
    return x_sol, max_it, timer, norm


def model_predict(model, image, fluid_cells, dtype=torch.float32):
    """Tests.model_predict (test.py:42-51): normalise r in FP32, scatter onto the
    grid, run ``model.eval_forward``, gather the fluid cells back as FP64.  The
    image pyramid and c0/c1 are cached per returned closure, as in the reference."""
    shape = tuple(image.shape[1:])
    n = int(np.prod(shape))

    def predict(r, timer=None, imgs=[], c0=[], c1=[]):  # noqa: B006 -- per-closure cache, as in test.py
        with torch.no_grad():
            r = normalize(r.to(dtype), dim=0)
            b = torch.zeros(n, device=r.device, dtype=dtype)
            b[fluid_cells] = r
            x = model.eval_forward(image, b.view((1, 1) + shape), timer, imgs, c0, c1).flatten().double()
        return x[fluid_cells]

    return predict
