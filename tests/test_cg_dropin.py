"""The drop-in solvers' iteration driver (mlpcg_gb300/cg.py) on the CPU.

npcg, npcg_flex and npsd run on FP64 torch-CPU tensors with the reference's
torch sparse CSR matrix and a fixed non-symmetric linear preconditioner, and
are compared with the oracle's restatement of cg_tests.py:26-284 (numpy):
the same iteration counts and residual histories (each iterate's relative
residual, passed to ``callback``) to 1e-6 (numpy and torch sum the dot products
in different orders), the same solutions.  Stopping
rules: npcg always takes one step and then continues while the residual is
above the threshold; npsd stops once it is below, or after max_it steps
(max_it = 0 gives back the initial guess).
"""
import numpy as np
import pytest
import torch

from mlpcg_gb300 import cg
from mlpcg_gb300.scenes import make_scene
from oracle import cg as ocg
from oracle import laplacian as olap


@pytest.fixture(scope="module")
def system():
    scene = make_scene(12, 3)
    A, fluid = olap.assemble(scene.flags)
    b = scene.rhs.ravel()[fluid]
    rng = np.random.default_rng(4)
    # a fixed non-symmetric preconditioner: Jacobi plus a small random coupling
    m = fluid.size
    D = 1.0 / A.diagonal()
    E = 0.005 * rng.standard_normal((m, m)) / np.sqrt(m)
    M = np.diag(D) + E
    At = torch.sparse_csr_tensor(torch.from_numpy(A.indptr.astype(np.int64)),
                                 torch.from_numpy(A.indices.astype(np.int64)),
                                 torch.from_numpy(A.data), size=A.shape)
    return A, At, b, M


def _run(fn, ofn, system, max_it, tol, atol):
    A, At, b, M = system
    Mt = torch.from_numpy(M)
    hist = []
    x, k, timer, rel = fn(torch.from_numpy(b), At, torch.zeros(b.size, dtype=torch.float64),
                          lambda r, *args: Mt @ r, max_it, tol=tol, atol=atol,
                          callback=lambda nrm, t: hist.append(nrm))
    xo, ko, ho = ofn(b, A, np.zeros(b.size), lambda r: M @ r, max_it, tol=tol, atol=atol)
    assert k == ko
    assert len(hist) == len(ho)
    np.testing.assert_allclose(hist, ho, rtol=1e-6, atol=0)
    assert rel == pytest.approx(ho[-1], rel=1e-6)
    np.testing.assert_allclose(x.numpy(), xo, rtol=0, atol=1e-10 * np.abs(xo).max())
    assert timer.top_level_clocks["Total"].tot_time >= 0.0
    return k, hist


@pytest.mark.parametrize("name", ["npcg", "npcg_flex", "npsd"])
def test_dropin_solvers_follow_the_oracle(system, name):
    fn, ofn = getattr(cg, name), getattr(ocg, name)
    k, hist = _run(fn, ofn, system, 100, 1e-8, 1e-20)
    assert hist[-1] < 1e-8 and k < 100


@pytest.mark.parametrize("name", ["npcg", "npcg_flex", "npsd"])
def test_dropin_solvers_stop_at_max_it(system, name):
    fn, ofn = getattr(cg, name), getattr(ocg, name)
    k, hist = _run(fn, ofn, system, 5, 1e-14, 1e-30)
    assert k == 5 and len(hist) == 6


def test_stopping_rules_at_the_edges(system):
    A, At, b, M = system
    Mt = torch.from_numpy(M)
    bt = torch.from_numpy(b)
    x0 = torch.zeros(b.size, dtype=torch.float64)
    pred = lambda r, *args: Mt @ r  # noqa: E731
    # npsd with max_it = 0: no step, the initial guess and residual come back
    x, k, _, rel = cg.npsd(bt, At, x0, pred, 0)
    assert k == 0 and torch.equal(x, x0) and rel == pytest.approx(1.0)
    # npcg always takes its first step, even with a threshold above the initial residual
    x, k, _, rel = cg.npcg(bt, At, x0, pred, 10, tol=2.0)
    assert k == 1 and rel < 1.0
    # npsd tests before counting the step as converged: a threshold above 1 stops after one step
    x, k, _, rel = cg.npsd(bt, At, x0, pred, 10, tol=2.0)
    assert k == 1


def test_npsd_hands_model_predict_fresh_caches(system):
    """npsd passes per-solve cache lists (the same lists through one solve, new ones for the
    next solve); npcg passes none, so the closure's own defaults serve every solve."""
    A, At, b, M = system
    Mt = torch.from_numpy(M)
    seen = []

    def pred(r, timer=None, *caches):
        seen.append(tuple(id(c) for c in caches))
        return Mt @ r

    bt = torch.from_numpy(b)
    x0 = torch.zeros(b.size, dtype=torch.float64)
    cg.npsd(bt, At, x0, pred, 3, tol=1e-30, atol=0.0)
    first = list(seen)
    assert len(first) == 3 and len(first[0]) == 3 and first[0] == first[1] == first[2]
    seen.clear()
    cg.npcg(bt, At, x0, pred, 3, tol=1e-30, atol=0.0)
    assert seen == [(), (), ()]
