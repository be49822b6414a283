"""Size-independent properties at the full benchmark size: a 256^3 scene (seed 7, 6 spheres),
5 levels, the committed trained weights -- the workload bench.py times.

At this size the oracle is too slow to run a solve, so the checks are the ones that do not depend
on size: the fused npsd solve converges and its residual, recomputed in FP64 with the matrix-free
operator, meets the tolerance; its residual history follows the drop-in path's (test.py's npsd
semantics, cg_tests.py:189-284) iteration by iteration; the classed coefficient layout gives the
dense planes' output bit for bit; and the symmetric network's plan is a symmetric operator
(the reference's self-test, sm_model_3d.py:476-485).
"""
from pathlib import Path

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N, LEVELS, SEED, SPHERES = 256, 5, 7, 6
WEIGHTS = Path(__file__).resolve().parent.parent / "mlpcg_gb300" / "weights"


@pytest.fixture(scope="module")
def scene():
    from mlpcg_gb300.scenes import make_scene
    return make_scene(N, SEED, SPHERES)


def _trained(cls_name, prefix, dev):
    from mlpcg_gb300 import sm_model_3d
    cls = getattr(sm_model_3d, cls_name)
    m = cls(LEVELS, 3, "trilinear") if cls_name == "SmallSMModelDn3D" else cls(LEVELS)
    d = np.load(WEIGHTS / f"{prefix}_l{LEVELS}.npz")
    m.load_state_dict({k: torch.from_numpy(d[k]) for k in m.state_dict()})
    return m.to(dev)


def _fp64_rel_residual(flags, b, x):
    from mlpcg_gb300.laplacian import FluidLaplacian
    A = FluidLaplacian(flags)
    bf = torch.where(flags == 2, b, torch.zeros_like(b))
    r = bf - A.matvec_grid(x.to(torch.float64))
    return float(r.norm() / bf.norm())


def test_fused_npsd_meets_tolerance_in_fp64(cuda, scene):
    """The benchmarked solve (BF16 storage, graph launch): converged, and ||b - A x|| / ||b|| with
    the FP64 operator at most the tolerance, as the solver reports it."""
    from mlpcg_gb300.solver import FusedSolver
    flags = torch.as_tensor(scene.flags, device=cuda)
    b = torch.as_tensor(scene.rhs, device=cuda)
    model = _trained("SmallSMModelDn3D", "smallsm", cuda)
    solver = FusedSolver(model, flags, method="npsd", max_it=100, tol=1e-6, storage=torch.bfloat16)
    res = solver.solve(b)
    assert res.status == "converged" and res.iterations <= 30, (res.status, res.iterations)
    assert not solver.plan.copy_failed()
    true_rel = _fp64_rel_residual(flags, b, res.x)
    assert true_rel <= 1.01e-6, true_rel
    assert abs(true_rel - res.rel_res) <= 1e-2 * true_rel, (true_rel, res.rel_res)
    assert np.all(np.diff(res.history[:4]) < 0)  # the first steps reduce the residual


def test_fused_history_follows_dropin(cuda, scene):
    """FP32 plan, true residual every iteration (the reference's r = b - A x): the fused solve's
    relative residuals equal the drop-in npsd's (FP64 vectors, eval_forward) within 2e-3."""
    from mlpcg_gb300 import cg
    from mlpcg_gb300.laplacian import FluidLaplacian
    from mlpcg_gb300.solver import FusedSolver
    flags = torch.as_tensor(scene.flags, device=cuda)
    model = _trained("SmallSMModelDn3D", "smallsm", cuda)
    solver = FusedSolver(model, flags, method="npsd", max_it=100, tol=1e-6, storage=torch.float32,
                         true_every=1)
    res = solver.solve(torch.as_tensor(scene.rhs, device=cuda))
    assert res.status == "converged"
    A = FluidLaplacian(flags)
    img = torch.as_tensor(scene.image(), device=cuda)
    b = torch.as_tensor(scene.rhs.ravel(), device=cuda)[A.fluid_cells]
    hist = []
    pred = cg.model_predict(model, img, A.fluid_cells)
    cg.npsd(b, A, torch.zeros_like(b), pred, 100, tol=1e-6, atol=1e-20, callback=lambda nrm, t: hist.append(nrm))
    assert hist[-1] < 1e-6
    assert abs(res.iterations - (len(hist) - 1)) <= 1, (res.iterations, len(hist) - 1)
    k = min(len(hist), len(res.history))
    np.testing.assert_allclose(res.history[:k], np.array(hist[:k]), rtol=2e-3)


def test_classed_layout_equals_dense_planes(cuda, scene):
    """One application of the benchmarked plan (BF16 coefficients and activations): run words,
    uniform vectors and mixed-run records reproduce the dense coefficient planes exactly."""
    from mlpcg_gb300.precond import PrecondPlan
    img = torch.as_tensor(scene.image(), device=cuda)
    model = _trained("SmallSMModelDn3D", "smallsm", cuda)
    cls = PrecondPlan(model, img, storage=torch.bfloat16, layout="classed")
    r = torch.randn(N ** 3, device=cuda, generator=torch.Generator(device=cuda).manual_seed(5))
    scale = torch.tensor([0.25], device=cuda)
    zc = cls.apply(r, scale)
    g0, m0 = cls.class_counts(0)
    assert 0 < g0 < N ** 3 // 4 and m0 > 0, (g0, m0)
    del cls
    dense = PrecondPlan(model, img, storage=torch.bfloat16, layout="dense")
    zd = dense.apply(r, scale)
    assert torch.equal(zc, zd), float((zc - zd).abs().max())
    assert torch.isfinite(zc).all() and float(zc.abs().max()) > 0.0


def test_symmetric_network_plan_is_symmetric(cuda, scene):
    """SmallSPDSMModelDn3D (trained weights, FP32 plan): <x, M y> = <y, M x> on fluid-supported
    vectors, and <x, M x> > 0."""
    from mlpcg_gb300.precond import PrecondPlan
    img = torch.as_tensor(scene.image(), device=cuda)
    model = _trained("SmallSPDSMModelDn3D", "smallspd", cuda)
    plan = PrecondPlan(model, img, storage=torch.float32)
    fluid = (img[1] != 0).reshape(-1)
    g = torch.Generator(device=cuda).manual_seed(0)
    x = torch.randn(fluid.numel(), device=cuda, generator=g) * fluid
    y = torch.randn(fluid.numel(), device=cuda, generator=g) * fluid
    a = torch.dot(x.double(), plan.apply(y).double())
    b = torch.dot(y.double(), plan.apply(x).double())
    assert abs(float(a - b)) <= 1e-5 * float(torch.sqrt(a.abs() * b.abs())), (float(a), float(b))
    assert float(torch.dot(x.double(), plan.apply(x).double())) > 0.0
