"""Drop-in neural CG solvers: npcg, npcg_flex, npsd (cg_tests.py:26-284) and
model_predict (test.py:42-51).

Same signatures and return values as the reference:
``solver(b, A, x_init, model_predict, max_it, tol, atol, verbose, callback)
-> (x, iterations, timer, relative_residual)``.  ``A`` may be the reference's
torch sparse CSR tensor or a ``laplacian.FluidLaplacian`` (matrix-free
sm_103a kernel).  These keep the reference's precision split (FP64 vectors,
FP32 network) and a host synchronisation per iteration, so they are the plain
drop-in; ``solver.FusedSolver`` is the graph-captured fast path.

All three solvers share one driver (``_iterate``): every iteration
preconditions the current residual, asks the method's direction rule for a
search direction d and a step s, moves x by s*d and recomputes r = b - A x
from scratch.  The rules differ only in how d and s are formed:

* ``_ConjugateDirections`` (npcg, npcg_flex): d = z + beta d_prev with the
  Fletcher-Reeves ratio r.z / r_prev.z_prev (or the Polak-Ribiere one,
  z.(r - r_prev) / r_prev.z_prev), s = r.z / d.A d;
* ``_ProjectedDescent`` (npsd): z A-orthogonalised against the last two
  directions, newest first, s = z.r / z.A z.

The floating-point operations and their order are the reference's, so
residual histories agree with it iteration by iteration; the two families
also keep the reference's stopping rules (npcg: at least one iteration, then
while ||r||/||b|| > threshold; npsd: up to max_it iterations, stopping once
||r||/||b|| < threshold).  The returned timer's top-level clock is 'Total',
as test.py:331 reads it.
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


class _ConjugateDirections:
    """Conjugate directions from the preconditioned residual (npcg / npcg_flex)."""

    fresh_cache = False      # the closure's own cache lists (cg_tests.py:54 calls model_predict(r, timer))
    at_least_one = True      # one step before the first convergence test

    def __init__(self, flexible: bool):
        self.flexible = flexible
        self.d = None        # previous direction
        self.rz = None       # previous r.z
        self.r = None        # residual the previous direction was built from

    def direction(self, r, z, A):
        rz = r.dot(z)
        if self.d is None:
            d = z
        else:
            num = z.dot(r - self.r) if self.flexible else rz
            d = z + (num / self.rz) * self.d
        s = rz / d.dot(A @ d)
        self.d, self.rz, self.r = d, rz, r
        return d, s

    @staticmethod
    def done(rel, threshold):
        return not rel > threshold


class _ProjectedDescent:
    """Steepest descent in the preconditioned residual, A-orthogonalised against
    the most recent directions (npsd, two of them)."""

    fresh_cache = True       # npsd hands model_predict per-solve caches (cg_tests.py:216)
    at_least_one = False

    def __init__(self, depth: int = 2):
        self.depth = depth
        self.kept = []       # (d, A d, d.A d), oldest first

    def direction(self, r, z, A):
        for d, Ad, dAd in reversed(self.kept):
            z = z - z.dot(Ad) / dAd * d
        Az = A @ z
        zAz = z.dot(Az)
        self.kept.append((z, Az, zAz))
        if len(self.kept) > self.depth:
            self.kept.pop(0)
        return z, z.dot(r) / zAz

    @staticmethod
    def done(rel, threshold):
        return rel < threshold


def _iterate(name, rule, b, A, x_init, model_predict, max_it, tol, atol, verbose, callback):
    clock = GlobalClock()
    clock.start("Total")

    def report(k, rel, r):
        if callback:
            _sync()
            callback(rel, time.perf_counter() - clock.top_level_clocks["Total"].start)
        if verbose:
            print(f"{name}: iteration {k}, relative residual {rel:.6e}, |r| = {r.norm().item():.6e}")

    clock.start("start")
    b_norm = b.norm().item()
    r = b - A @ x_init
    rel = r.norm().item() / b_norm
    report(0, rel, r)
    x = torch.clone(x_init)
    threshold = max(tol, atol / b_norm)
    caches = ([], [], []) if rule.fresh_cache else ()
    _sync()
    clock.stop("start")

    k = 0
    while rule.at_least_one or k < max_it:
        clock.start("precondition")
        z = model_predict(r, clock, *caches)
        _sync()
        clock.stop("precondition")

        clock.start("step")
        d, s = rule.direction(r, z, A)
        x += s * d
        r = b - A @ x
        k += 1
        _sync()
        clock.stop("step")

        clock.start("residual")
        rel = r.norm().item() / b_norm
        _sync()
        clock.stop("residual")
        report(k, rel, r)
        if rule.done(rel, threshold) or k >= max_it:
            break

    _sync()
    clock.stop("Total")
    return x, k, clock, rel


def npcg(b, A, x_init, model_predict, max_it, tol=1e-10, atol=1e-12, verbose=False, callback=None):
    """Preconditioned CG with a (possibly non-symmetric) network preconditioner (cg_tests.py:26-101)."""
    return _iterate("npcg", _ConjugateDirections(flexible=False), b, A, x_init, model_predict, max_it, tol, atol,
                    verbose, callback)


def npcg_flex(b, A, x_init, model_predict, max_it, tol=1e-10, atol=1e-12, verbose=False, callback=None):
    """Flexible PCG, Polak-Ribiere beta (cg_tests.py:103-183)."""
    return _iterate("npcg_flex", _ConjugateDirections(flexible=True), b, A, x_init, model_predict, max_it, tol,
                    atol, verbose, callback)


def npsd(b, A, x_init, model_predict, max_it, tol=1e-10, atol=1e-10, verbose=False, callback=None):
    """Neural-preconditioned steepest descent, A-orthogonalised against the last
    two directions (cg_tests.py:189-284); the solver of test.py:327-328."""
    return _iterate("npsd", _ProjectedDescent(2), b, A, x_init, model_predict, max_it, tol, atol, verbose,
                    callback)


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
