"""Preconditioner plan and fused graph-captured solver vs the drop-in path and the FP64 oracle (GPU)."""
import ctypes as C

import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import laplacian as olap

pytestmark = pytest.mark.gpu


def _model(n, dev, seed=0, swap=False, mask=False):
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D
    torch.manual_seed(seed)
    return SmallSMModelDn3D(n, 3, "trilinear", mask=mask, swap_sm_order=swap).to(dev)


def _near_identity_model(n, dev, eps=0.02, seed=1):
    """M = I plus a small non-symmetric perturbation through every block and level."""
    m = _model(n, dev, seed)
    with torch.no_grad():
        for p in m.parameters():
            p.mul_(eps)
        m.pre[0].bias[13] += 1.0
        m.c0[0].bias[0] += 1.0
    return m


def _scene(shape, seed, dev):
    from mlpcg_gb300.scenes import make_scene
    s = make_scene(shape, seed)
    return s, torch.as_tensor(s.flags, device=dev), torch.as_tensor(s.image(), device=dev)


@pytest.mark.parametrize("shape,n", [((16, 16, 16), 3), ((32, 16, 24), 3), ((64, 64, 64), 4), ((24, 40, 8), 3)])
@pytest.mark.parametrize("swap,mask", [(False, False), (True, False), (False, True)])
def test_plan_fp32_matches_eval_forward(cuda, shape, n, swap, mask):
    s, flags, img = _scene(shape, 2, cuda)
    m = _model(n, cuda, swap=swap, mask=mask)
    plan = m.precond_plan(img, storage=torch.float32)
    b = torch.randn((1, 1) + shape, device=cuda)
    ref = m.eval_forward(img, b)
    ref = torch.where(img[1] == 0, 0.0, ref)          # the fluid gather of test.py:49-50
    z = plan.apply(b.reshape(-1)).reshape(ref.shape)
    assert rel_err(z.cpu().numpy(), ref.cpu().numpy()) < 1e-5
    scale = torch.tensor([0.37], device=cuda)
    z2 = plan.apply(b.reshape(-1).contiguous(), scale).reshape(ref.shape)
    assert rel_err(z2.cpu().numpy(), 0.37 * ref.cpu().numpy()) < 1e-5


@pytest.mark.parametrize("shape,n", [((128, 128, 128), 4), ((96, 64, 128), 4), ((256, 256, 256), 5)])
@pytest.mark.parametrize("storage", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("swap,mask,layout", [(False, False, "classed"), (True, True, "classed"),
                                              (False, False, "dense")])
def test_coarse_cluster_equals_per_level_kernels(cuda, shape, n, storage, swap, mask, layout):
    """With the cluster switched on, a whole application runs the coarse levels (from the first level
    with at most four tiles per CTA down to the coarsest) in one thread-block cluster launch; the
    application split into stages [0, n] and [n + 1, 2n] runs the per-level kernels instead.  Same
    bodies, same arithmetic: the outputs agree bit for bit."""
    s, flags, img = _scene(shape, 3, cuda)
    m = _model(n, cuda, seed=2, swap=swap, mask=mask)
    plan = m.precond_plan(img, storage=storage) if layout == "classed" else None
    if plan is None:
        from mlpcg_gb300.precond import PrecondPlan
        plan = PrecondPlan(m, img, storage=storage, layout="dense")
    assert plan.coarse_cluster()[0] == -1  # off by default
    plan.set_coarse_cluster(True)
    assert plan.coarse_cluster()[0] > 0
    r = torch.randn(int(np.prod(shape)), device=cuda, generator=torch.Generator(device=cuda).manual_seed(5))
    z_cluster = plan.apply(r).clone()
    z_levels = torch.empty_like(z_cluster)
    plan.apply_stages(0, n, r, None, z_levels)
    plan.apply_stages(n + 1, 2 * n, r, None, z_levels)
    assert torch.equal(z_cluster, z_levels)
    assert bool(torch.isfinite(z_cluster).all()) and float(z_cluster.abs().max()) > 0


@pytest.mark.parametrize("storage,act", [(torch.bfloat16, torch.bfloat16), (torch.bfloat16, torch.float32),
                                         (torch.float32, torch.bfloat16)])
def test_plan_bf16_storage(cuda, storage, act):
    s, flags, img = _scene((64, 64, 64), 4, cuda)
    m = _model(4, cuda)
    ref = m.precond_plan(img, storage=torch.float32).apply(torch.ones(64 ** 3, device=cuda))
    b = torch.randn(64 ** 3, device=cuda)
    ref = m.precond_plan(img, storage=torch.float32).apply(b)
    z = m.precond_plan(img, storage=storage, act_storage=act).apply(b)
    err = (z - ref).norm() / ref.norm()
    assert err < 2e-2, float(err)


@pytest.mark.parametrize("shape,n,seed", [((64, 64, 64), 4, 4), ((32, 48, 64), 3, 9), ((128, 128, 128), 5, 7)])
@pytest.mark.parametrize("storage", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("swap,mask", [(False, False), (True, True)])
def test_plan_classed_is_bit_identical_to_dense(cuda, shape, n, seed, storage, swap, mask):
    """Run words + uniform vectors + mixed-run records give exactly the dense planes' output."""
    from mlpcg_gb300.precond import PrecondPlan
    s, flags, img = _scene(shape, seed, cuda)
    m = _model(n, cuda, seed=3, swap=swap, mask=mask)
    dense = PrecondPlan(m, img, storage=storage, layout="dense")
    cls = PrecondPlan(m, img, storage=storage, layout="classed")
    g0 = cls.general_cells(0)
    n0 = int(np.prod(shape))
    assert 0 < g0 < n0 // 2, g0
    b = torch.randn(n0, device=cuda)
    scale = torch.tensor([0.5], device=cuda)
    zd = dense.apply(b, scale)
    zc = cls.apply(b, scale)
    assert torch.equal(zd, zc), float((zd - zc).abs().max())
    # every stage on its own as well
    for st in range(2 * n + 1):
        a = dense.apply_stages(st, st, b, scale)
        c = cls.apply_stages(st, st, b, scale)
    torch.cuda.synchronize()


@pytest.mark.parametrize("storage", [torch.float32, torch.bfloat16])
def test_plan_classed_equals_dense_with_non_one_hot_finest_image(cuda, storage):
    """A finest image with fractional values in places: the general cells around them are not
    one-hot patterns, so they take no pattern-table row and are evaluated one by one
    (k_kgen_list's path behind the table's failure flag) -- the output still equals the dense
    planes' bit for bit."""
    from mlpcg_gb300.precond import PrecondPlan
    s, flags, img = _scene((64, 64, 64), 4, cuda)
    img = img.clone()
    g = torch.Generator(device=cuda).manual_seed(3)
    pick = torch.rand(img.shape[1:], device=cuda, generator=g) < 0.002
    img[:, pick] = 0.5
    m = _model(4, cuda, seed=3)
    dense = PrecondPlan(m, img, storage=storage, layout="dense")
    cls = PrecondPlan(m, img, storage=storage, layout="classed")
    b = torch.randn(64 ** 3, device=cuda, generator=g)
    assert cls.general_cells(0) > 0
    assert torch.equal(dense.apply(b), cls.apply(b))


def test_plan_classed_uniform_grid(cuda):
    """An all-fluid interior (only the wall layer differs) is almost entirely uniform."""
    from mlpcg_gb300.precond import PrecondPlan
    flags = torch.full((32, 32, 32), 2, dtype=torch.uint8, device=cuda)
    flags[0], flags[-1], flags[:, 0], flags[:, -1], flags[:, :, 0], flags[:, :, -1] = 0, 0, 0, 0, 0, 0
    from mlpcg_gb300.solver import flags_to_image
    img = flags_to_image(flags)
    m = _model(3, cuda, seed=5)
    dense = PrecondPlan(m, img, storage=torch.float32, layout="dense")
    cls = PrecondPlan(m, img, storage=torch.float32, layout="classed")
    interior = 28 ** 3
    assert cls.general_cells(0) == 32 ** 3 - interior
    # runs of 8 z-cells: uniform where i, j are interior and the run avoids k < 2 and k > 29
    assert cls.mixed_runs(0) == 32 * 32 * 4 - 28 * 28 * 2
    b = torch.randn(32 ** 3, device=cuda)
    assert torch.equal(dense.apply(b), cls.apply(b))


def test_plan_coefficients_match_linear_blocks(cuda):
    s, flags, img = _scene((32, 32, 32), 5, cuda)
    m = _model(3, cuda)
    plan = m.precond_plan(img, storage=torch.float32)
    c = plan.coefficients().cpu().numpy()
    imgs = [img]
    from mlpcg_gb300 import ops
    for _ in range(2):
        imgs.append(ops.avg_pool2(imgs[-1]))
    for l in range(3):
        c0 = float(m.c0[l].eval_forward(imgs[l]))
        c1 = float(m.c1[l].eval_forward(imgs[l]))
        assert abs(c[l] - c0) <= 1e-6 * max(1, abs(c0)) and abs(c[3 + l] - c1) <= 1e-6 * max(1, abs(c1))


@pytest.mark.parametrize("method", ["npcg", "npsd"])
@pytest.mark.parametrize("use_graph", [True, False])
def test_fused_identity_preconditioner_is_cg(cuda, method, use_graph):
    """With M = I, npcg is plain CG: converge to 1e-6 and match the FP64 oracle solution."""
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene((24, 24, 24), 3, cuda)
    m = _near_identity_model(3, cuda, eps=0.0)
    solver = FusedSolver(m, flags, method=method, max_it=400, tol=1e-6, storage=torch.float32)
    res = solver.solve(torch.as_tensor(s.rhs, device=cuda), use_graph=use_graph)
    assert res.status == "converged", (res.status, res.iterations, res.rel_res)
    A, fluid = olap.assemble(s.flags)
    b = s.rhs.ravel()[fluid]
    x = res.x.cpu().numpy().ravel()[fluid]
    true_rel = np.linalg.norm(b - A @ x) / np.linalg.norm(b)
    assert true_rel < 1e-6 and abs(true_rel - res.rel_res) <= 1e-3 * true_rel
    xo, it_o = olap.cg_fp64(A, b, tol=1e-12)
    assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-4
    if method == "npcg":
        _, it_cg = olap.cg_fp64(A, b, tol=1e-6)
        assert abs(res.iterations - it_cg) <= 3
    assert np.all(solver.flags.cpu().numpy().ravel()[res.x.cpu().numpy().ravel() != 0] == 2)


@pytest.mark.parametrize("method", ["npsd", "npcg"])
def test_fused_matches_dropin_history(cuda, method):
    """Fused (FP32 vectors, FP64 reductions) vs drop-in (FP64 vectors, reference recurrences)."""
    from mlpcg_gb300 import cg
    from mlpcg_gb300.laplacian import FluidLaplacian
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene((32, 32, 32), 6, cuda)
    m = _near_identity_model(3, cuda)
    solver = FusedSolver(m, flags, method=method, max_it=400, tol=1e-6, storage=torch.float32, true_every=1)
    res = solver.solve(torch.as_tensor(s.rhs, device=cuda))
    A = FluidLaplacian(flags)
    b = torch.as_tensor(s.rhs.ravel(), device=cuda)[A.fluid_cells]
    hist = []
    pred = cg.model_predict(m, img, A.fluid_cells)
    getattr(cg, method)(b, A, torch.zeros_like(b), pred, 400, tol=1e-6, atol=1e-20,
                        callback=lambda nrm, t: hist.append(nrm))
    k = min(25, len(hist), len(res.history))
    np.testing.assert_allclose(res.history[:k], np.array(hist[:k]), rtol=2e-3)
    if method == "npsd":
        assert res.status == "converged" and hist[-1] < 1e-6
        assert abs(res.iterations - (len(hist) - 1)) <= max(3, 0.05 * res.iterations)
    else:
        # PCG with a non-symmetric, input-normalised M may stagnate (in both implementations)
        assert abs(np.log10(res.rel_res) - np.log10(hist[-1])) < 1.0


def test_fused_warm_start_and_off_fluid_values(cuda):
    """x0 enters through its double-float pair: restarting from the solution is already converged,
    a perturbed start converges to the same solution, and x0 off the fluid cells is left as given."""
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene((24, 24, 24), 3, cuda)
    m = _near_identity_model(3, cuda, eps=0.0)
    solver = FusedSolver(m, flags, method="npsd", max_it=400, tol=1e-6, storage=torch.float32)
    b = torch.as_tensor(s.rhs, device=cuda)
    fluid = flags == 2
    cold = solver.solve(b)
    assert cold.status == "converged"
    xc = cold.x.clone()
    warm = solver.solve(b, x0=xc.clone())
    assert warm.status == "converged" and warm.iterations == 0
    assert rel_err(warm.x[fluid].cpu(), xc[fluid].cpu()) < 1e-12
    g = torch.Generator(device=cuda).manual_seed(4)
    x0 = xc + 0.1 * xc.abs().max() * torch.randn(xc.shape, generator=g, device=cuda, dtype=torch.float64)
    x0[~fluid] = 7.0
    pert = solver.solve(b, x0=x0)
    assert pert.status == "converged" and pert.iterations > 0
    assert torch.all(pert.x[~fluid] == 7.0)
    assert rel_err(pert.x[fluid].cpu(), xc[fluid].cpu()) < 1e-4


def test_solve_host_matches_device_solve(cuda):
    """The host-to-host form (rhs copied on a side stream during the set-up) gives the device
    solve's result, also for a new frame whose flags differ from the solver's current ones."""
    from mlpcg_gb300.solver import FusedSolver, flags_to_image
    s, flags, img = _scene((32, 32, 32), 5, cuda)
    s2, flags2, img2 = _scene((32, 32, 32), 6, cuda)
    m = _near_identity_model(3, cuda)
    ref = FusedSolver(m, flags2.clone(), method="npsd", max_it=60, tol=1e-6)
    r_ref = ref.solve(torch.as_tensor(s2.rhs, device=cuda))
    x_ref = r_ref.x.cpu()
    solver = FusedSolver(m, flags.clone(), method="npsd", max_it=60, tol=1e-6)
    solver.solve(torch.as_tensor(s.rhs, device=cuda))
    flags_h = torch.from_numpy(s2.flags).pin_memory()
    b_h = torch.from_numpy(s2.rhs).pin_memory()
    x_h = torch.empty(s2.rhs.shape, dtype=torch.float64).pin_memory()
    solver.solve_host(flags_h, b_h, x_h)
    r = solver.result()
    torch.cuda.synchronize()
    assert r.iterations == r_ref.iterations and r.status == r_ref.status
    assert torch.equal(x_h, x_ref)


@pytest.mark.parametrize("shape", [(16, 16, 16), (7, 13, 29), (64, 64, 64)])
def test_fluid_vectors_scatter_gather(cuda, shape):
    """Fluid-DOF order, scatter and gather against torch indexing of the fluid cells (flat order),
    including a capacity shorter than the fluid count."""
    from mlpcg_gb300._lib import call, load
    from mlpcg_gb300.ops import _p, _stream
    g = torch.Generator(device=cuda).manual_seed(11)
    flags = torch.randint(0, 4, shape, generator=g, device=cuda, dtype=torch.uint8)
    n = flags.numel()
    fluid = torch.nonzero(flags.view(-1) == 2).view(-1)
    m = fluid.numel()
    order = torch.empty(int(load().mlpcg_fluid_order_entries(n)), dtype=torch.int32, device=cuda)
    st = _stream(flags.device)
    call("mlpcg_fluid_order", _p(flags), n, _p(order), st)
    vals = torch.randn(m, dtype=torch.float64, device=cuda, generator=g)
    grid = torch.full((n,), 5.0, dtype=torch.float64, device=cuda)
    call("mlpcg_scatter_fluid", _p(vals), m, _p(flags), _p(order), n, _p(grid), st)
    ref = torch.zeros(n, dtype=torch.float64, device=cuda)
    ref[fluid] = vals
    assert torch.equal(grid, ref)
    src = torch.randn(n, dtype=torch.float64, device=cuda, generator=g)
    out = torch.full((m + 3,), 9.0, dtype=torch.float64, device=cuda)
    call("mlpcg_gather_fluid", _p(src), _p(flags), _p(order), n, _p(out), m, st)
    assert torch.equal(out[:m], src[fluid]) and torch.all(out[m:] == 9.0)
    k = m // 2  # a short vector: the cells beyond it read as 0 / are not written
    call("mlpcg_scatter_fluid", _p(vals), k, _p(flags), _p(order), n, _p(grid), st)
    ref2 = torch.zeros(n, dtype=torch.float64, device=cuda)
    ref2[fluid[:k]] = vals[:k]
    assert torch.equal(grid, ref2)
    out.fill_(9.0)
    call("mlpcg_gather_fluid", _p(src), _p(flags), _p(order), n, _p(out), k, st)
    assert torch.equal(out[:k], src[fluid[:k]]) and torch.all(out[k:] == 9.0)


@pytest.mark.parametrize("shape", [(7, 13, 29), (128, 128, 96)])
def test_fluid_scatter_gather_with_pinned_host_memory(cuda, shape):
    """The scatter reading pinned host memory runs on a capped grid whose CTAs step through the
    cell blocks (1,536 blocks at 128 x 128 x 96, several per CTA): the same grid as torch indexing,
    for the full and for a short vector; the gather writes pinned host memory directly."""
    from mlpcg_gb300._lib import call, load
    from mlpcg_gb300.ops import _p, _stream
    g = torch.Generator(device=cuda).manual_seed(12)
    flags = torch.randint(0, 4, shape, generator=g, device=cuda, dtype=torch.uint8)
    n = flags.numel()
    fluid = torch.nonzero(flags.view(-1) == 2).view(-1)
    m = fluid.numel()
    order = torch.empty(int(load().mlpcg_fluid_order_entries(n)), dtype=torch.int32, device=cuda)
    st = _stream(flags.device)
    call("mlpcg_fluid_order", _p(flags), n, _p(order), st)
    vals = torch.randn(m, dtype=torch.float64, device=cuda, generator=g)
    vals_h = vals.cpu().pin_memory()
    for k in (m, m // 3):
        grid = torch.full((n,), 5.0, dtype=torch.float64, device=cuda)
        call("mlpcg_scatter_fluid", C.c_void_p(vals_h.data_ptr()), k, _p(flags), _p(order), n, _p(grid), st)
        torch.cuda.synchronize()
        ref = torch.zeros(n, dtype=torch.float64, device=cuda)
        ref[fluid[:k]] = vals[:k]
        assert torch.equal(grid, ref)
    src = torch.randn(n, dtype=torch.float64, device=cuda, generator=g)
    for k in (m, m // 3):  # the gather into pinned host memory
        out_h = torch.full((m + 3,), 9.0, dtype=torch.float64).pin_memory()
        call("mlpcg_gather_fluid", _p(src), _p(flags), _p(order), n, C.c_void_p(out_h.data_ptr()), k, st)
        torch.cuda.synchronize()
        assert torch.equal(out_h[:k], src[fluid[:k]].cpu()) and torch.all(out_h[k:] == 9.0)


def test_solve_host_fluid_vectors(cuda):
    """solve_host with fluid-DOF vectors (the reference's compressed rhs / solution) equals the
    grid solve on the fluid cells, whether the kernels read and write the pinned host vectors
    themselves or pageable vectors go through device copies."""
    from mlpcg_gb300.solver import FusedSolver, _host_mapped
    s, flags, img = _scene((32, 32, 32), 6, cuda)
    m = _near_identity_model(3, cuda)
    solver = FusedSolver(m, flags.clone(), method="npsd", max_it=60, tol=1e-6)
    ref = solver.solve(torch.as_tensor(s.rhs, device=cuda))
    fl = s.flags.reshape(-1) == 2
    x_ref = ref.x.cpu().reshape(-1)[torch.from_numpy(fl)]
    b_h = torch.from_numpy(np.ascontiguousarray(s.rhs.reshape(-1)[fl])).pin_memory()
    x_h = torch.empty(b_h.numel(), dtype=torch.float64).pin_memory()
    assert _host_mapped(b_h) and _host_mapped(x_h) and not _host_mapped(b_h.clone())
    solver.solve_host(torch.from_numpy(s.flags).pin_memory(), b_h, x_h)
    r = solver.result()
    torch.cuda.synchronize()
    assert r.iterations == ref.iterations and torch.equal(x_h, x_ref)
    b_p, x_p = b_h.clone(), torch.zeros_like(x_ref)       # pageable: staged copies
    solver.solve_host(torch.from_numpy(s.flags), b_p, x_p)
    r = solver.result()
    torch.cuda.synchronize()
    assert r.iterations == ref.iterations and torch.equal(x_p, x_ref)


def test_batch_of_uneven_systems_matches_single_solves(cuda):
    """Systems of different sizes (16^3 to 96^3), methods and limits in one batched launch: every
    system's iterations, status and solution equal its own solve; a system that starts converged
    stays at zero iterations while the others run; the batch graph is reusable."""
    from mlpcg_gb300.solver import BatchSolver, FusedSolver
    # the 96^3 system's levels 3 (12^3) and its coarsest run the general (untiled) kernels
    specs = [((16, 16, 16), 3, "npsd", 60, 1e-6, 1), ((24, 16, 32), 3, "npcg", 80, 1e-5, 2),
             ((32, 32, 32), 3, "npsd", 100, 1e-6, 3), ((16, 24, 16), 2, "npsd", 50, 1e-6, 4),
             ((96, 96, 96), 4, "npsd", 30, 1e-6, 5)]
    solvers, rhs, singles = [], [], []
    for shape, n, method, max_it, tol, seed in specs:
        s, flags, img = _scene(shape, seed, cuda)
        m = _near_identity_model(n, cuda, seed=seed)
        solver = FusedSolver(m, flags, method=method, max_it=max_it, tol=tol)
        b = torch.as_tensor(s.rhs, device=cuda)
        if seed == 4:
            b = torch.zeros_like(b)  # converged from the start
        r = solver.solve(b)
        singles.append((r.iterations, r.status, r.x.clone()))
        solvers.append(solver)
        rhs.append(b)
    batch = BatchSolver(solvers)
    for _ in range(2):
        res = batch.solve(rhs)
        for (it, st, x), r in zip(singles, res):
            assert r.iterations == it and r.status == st
            assert torch.equal(r.x, x)
    assert res[3].iterations == 0 and res[3].status == "converged"
    assert max(r.iterations for r in res) > 0


def test_fused_graph_reuse_is_deterministic(cuda):
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene((32, 32, 32), 7, cuda)
    m = _near_identity_model(3, cuda)
    solver = FusedSolver(m, flags, method="npsd", max_it=40, tol=1e-6)
    r1 = solver.solve(torch.as_tensor(s.rhs, device=cuda))
    x1 = r1.x.clone()
    assert r1.status == "max_it" and r1.iterations == 40 and r1.history[-1] < r1.history[0]
    r2 = solver.solve(torch.as_tensor(s.rhs, device=cuda))
    assert r2.iterations == r1.iterations and torch.equal(x1, r2.x)  # deterministic reductions
    r3 = solver.solve(torch.as_tensor(s.rhs, device=cuda), use_graph=False)
    assert torch.equal(x1, r3.x) and r3.iterations == r1.iterations


@pytest.mark.parametrize("method", ["npsd", "npcg"])
def test_dependent_launch_gives_identical_solves(cuda, method):
    """Programmatic edges in the captured iteration (the default): the graph has them, and x, the
    iteration count and the residual history equal those of the graph with ordinary edges and of
    the uncaptured loop, bit for bit (64^3, BF16 plan with TMA level-0 tiles and small levels)."""
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene((64, 64, 64), 7, cuda)
    m = _near_identity_model(4, cuda)
    solver = FusedSolver(m, flags, method=method, max_it=30, tol=1e-9, storage=torch.bfloat16)
    b = torch.as_tensor(s.rhs, device=cuda)
    runs = {}
    for key, dep, graph in (("dependent", True, True), ("ordinary", False, True), ("loop", True, False)):
        solver.set_dependent_launch(dep)
        r = solver.solve(b, use_graph=graph)
        runs[key] = (r.iterations, r.status, r.x.clone(), np.array(r.history))
        if key == "dependent":
            assert solver.dependent_edges() > 10
        if key == "ordinary":
            assert solver.dependent_edges() == 0
    it0, st0, x0, h0 = runs["dependent"]
    assert it0 > 5
    for key in ("ordinary", "loop"):
        it, st, x, h = runs[key]
        assert it == it0 and st == st0 and torch.equal(x, x0) and np.array_equal(h, h0), key


@pytest.mark.parametrize("method", ["npsd", "npcg"])
def test_solver_products_in_the_preconditioner_epilogue(cuda, method):
    """The solver's products summed by the level-0 post-block (npsd z . Ap, npcg r . z; the
    default for this plan) against the separate pass: the same products added in another order.
    The rounding differences grow slowly over 40 iterations of this slowly converging system
    (measured 4.4e-5 relative at most), so the histories agree to 2e-4 and the solutions to 1e-3,
    with the same iteration count and status; the epilogue is off when switched off, and graph
    and loop solves with it agree bit for bit."""
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene((64, 64, 64), 7, cuda)
    m = _near_identity_model(4, cuda)
    b = torch.as_tensor(s.rhs, device=cuda)
    solver = FusedSolver(m, flags, method=method, max_it=40, tol=1e-7, storage=torch.bfloat16)
    assert solver.fused_dots()
    r_fused = solver.solve(b)
    x_fused, h_fused = r_fused.x.clone(), np.array(r_fused.history)
    r_loop = solver.solve(b, use_graph=False)
    assert torch.equal(r_loop.x, x_fused) and np.array_equal(np.array(r_loop.history), h_fused)
    solver.set_fused_dots(False)
    assert not solver.fused_dots()
    r_sep = solver.solve(b)
    assert r_sep.iterations == r_fused.iterations and r_sep.status == r_fused.status
    h_sep = np.array(r_sep.history)[: r_sep.iterations + 1]
    np.testing.assert_allclose(h_fused[: r_fused.iterations + 1], h_sep, rtol=2e-4)
    assert float((r_sep.x - x_fused).norm() / r_sep.x.norm()) < 1e-3


def test_fused_status_words(cuda):
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene((16, 16, 16), 8, cuda)
    m = _near_identity_model(2, cuda)
    solver = FusedSolver(m, flags, method="npsd", max_it=2, tol=1e-6)
    r = solver.solve(torch.zeros(s.shape, dtype=torch.float64, device=cuda))
    assert r.status == "converged" and r.iterations == 0
    r = solver.solve(torch.as_tensor(s.rhs, device=cuda))
    assert r.status == "max_it" and r.iterations == 2
    bad = torch.as_tensor(s.rhs, device=cuda).clone()
    bad.view(-1)[torch.nonzero(flags.view(-1) == 2)[0]] = float("nan")
    r = solver.solve(bad)
    assert r.status == "nonfinite"
    # the solver still works after a non-finite solve
    r = solver.solve(torch.as_tensor(s.rhs, device=cuda))
    assert r.status == "max_it" and np.isfinite(r.rel_res)


def test_all_solid_grid(cuda):
    from mlpcg_gb300.solver import FusedSolver
    flags = torch.full((16, 16, 16), 1, dtype=torch.uint8, device=cuda)
    m = _near_identity_model(2, cuda)
    solver = FusedSolver(m, flags, method="npcg", max_it=5, tol=1e-6)
    r = solver.solve(torch.ones((16, 16, 16), dtype=torch.float64, device=cuda))
    assert r.status == "converged" and r.iterations == 0


def test_tile_copies_complete(cuda):
    """The level-0 pre-block's input tiles (loaded by the tensor-memory accelerator) all land: the
    plan's copy-failure flag stays clear over applications and a graph-captured solve."""
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene((64, 64, 64), 3, cuda)
    m = _near_identity_model(4, cuda)
    solver = FusedSolver(m, flags, method="npsd", max_it=60, tol=1e-6, storage=torch.bfloat16)
    for _ in range(3):
        solver.plan.apply(torch.randn(64 ** 3, device=cuda))
    res = solver.solve(torch.as_tensor(s.rhs, device=cuda))
    assert res.status in ("converged", "max_it") and np.isfinite(res.rel_res)
    assert res.history[-1] < 0.1 * res.history[0]
    assert not solver.plan.copy_failed()


def test_tma_wait_timeout_reports_copy_failed(cuda):
    """The bounded waits on the tensor-memory accelerator's tile copies, made to run out on ordinary
    copies by the copy-stall knob (the first wait polls a barrier that nothing arrives on; the real
    copy still completes and is waited for before the CTA leaves): the plan reports copy_failed, a
    solve using it ends with status 'copy_failed', and so does a solve whose SpMV waits run out.
    With the knobs off, the same plan and solver give the same results as before, bit for bit."""
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene((64, 64, 64), 3, cuda)
    m = _near_identity_model(4, cuda)
    solver = FusedSolver(m, flags, method="npsd", max_it=60, tol=1e-6, storage=torch.bfloat16)
    plan = solver.plan
    b = torch.as_tensor(s.rhs, device=cuda)
    r = torch.randn(64 ** 3, device=cuda, generator=torch.Generator(device=cuda).manual_seed(3))
    z_ok = plan.apply(r).clone()
    ok = solver.solve(b)
    x_ok = ok.x.clone()
    assert ok.status in ("converged", "max_it") and not plan.copy_failed()
    # the plan's level-0 tile waits run out
    plan.set_copy_stall(True)
    plan.apply(r)
    assert plan.copy_failed()
    res = solver.solve(b)
    assert res.status == "copy_failed"
    plan.set_copy_stall(False)
    assert not plan.copy_failed()
    z = plan.apply(r)
    assert not plan.copy_failed() and torch.equal(z, z_ok)
    # the SpMV's tile waits run out
    solver.set_copy_stall(True)
    res = solver.solve(b)
    assert res.status == "copy_failed" and res.iterations <= 1
    solver.set_copy_stall(False)
    res = solver.solve(b)
    assert res.status == ok.status and res.iterations == ok.iterations and torch.equal(res.x, x_ok)
    assert not plan.copy_failed()


def test_zero_guess_solve_writes_every_cell(cuda):
    """solve(b) without x0 starts from x0 = 0 without reading or clearing x: the result equals the
    solve from an explicit zero guess, and the cells off the fluid hold 0 even if x held other
    values before."""
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene((32, 32, 32), 5, cuda)
    m = _near_identity_model(3, cuda)
    solver = FusedSolver(m, flags, method="npsd", max_it=100, tol=1e-6, storage=torch.bfloat16)
    b = torch.as_tensor(s.rhs, device=cuda)
    ref = solver.solve(b, x0=torch.zeros_like(b))
    xr = ref.x.clone()
    solver.x.fill_(3.0)
    out = solver.solve(b)
    assert out.status == ref.status and out.iterations == ref.iterations
    assert torch.equal(out.x, xr)
    assert torch.all(out.x[flags != 2] == 0)


@pytest.mark.parametrize("n", [16, 24, 48])
def test_copy_flag_clear_with_general_path_levels(cuda, n):
    """Plans whose coarse levels run the general (untiled) kernels keep the tile-copy flag clear
    (their temporaries must not overlap it) and still match eval_forward."""
    s, flags, img = _scene((n, n, n), 3, cuda)
    m = _model(3, cuda)
    plan = m.precond_plan(img, storage=torch.float32)
    b = torch.randn((1, 1, n, n, n), device=cuda)
    z = plan.apply(b.reshape(-1)).reshape(b.shape)
    ref = torch.where(img[1] == 0, 0.0, m.eval_forward(img, b))
    assert rel_err(z.cpu().numpy(), ref.cpu().numpy()) < 1e-5
    assert not plan.copy_failed()


@pytest.mark.parametrize("shape", [(20, 36, 40), (12, 8, 16)])
def test_fused_solve_on_uneven_grids(cuda, shape):
    """Partial tiles in x and y (TMA-tiled SpMV, TMA level-0 blocks) and untiled coarse levels: the
    fused npsd solve converges and meets the tolerance against the oracle's FP64 matrix."""
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene(shape, 4, cuda)
    m = _near_identity_model(2, cuda)
    solver = FusedSolver(m, flags, method="npsd", max_it=3000, tol=1e-6, storage=torch.float32)
    res = solver.solve(torch.as_tensor(s.rhs, device=cuda))
    assert res.status == "converged", res.status
    A, fluid = olap.assemble(s.flags)
    x = res.x.reshape(-1).cpu().numpy()[fluid]
    b = s.rhs.reshape(-1)[fluid]
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 2e-6
    assert not solver.plan.copy_failed()


def test_plan_and_solver_refuse_mis_sized_tensors(cuda):
    """Wrong sizes, dtypes or empty scales are refused in Python before any kernel sees them
    (the kernels index by the plan's grid alone); a valid call still works afterwards."""
    from mlpcg_gb300.precond import PrecondPlan
    from mlpcg_gb300.solver import FusedSolver
    s, flags, img = _scene((16, 16, 16), 2, cuda)
    m = _model(2, cuda)
    plan = PrecondPlan(m, img, storage=torch.float32)
    n = 16 ** 3
    good = torch.ones(n, device=cuda)
    with pytest.raises(RuntimeError):
        plan.apply(torch.zeros(n - 8, device=cuda))
    with pytest.raises(RuntimeError):
        plan.apply(good, out=torch.empty(n // 2, device=cuda))
    with pytest.raises(RuntimeError):
        plan.apply(good.double())
    with pytest.raises(RuntimeError):
        plan.apply_stages(0, 0, torch.zeros(2 * n, device=cuda))
    with pytest.raises(RuntimeError):
        plan.apply(good, scale=torch.zeros(0, device=cuda))
    solver = FusedSolver(m, flags, plan=plan)
    with pytest.raises(RuntimeError):
        solver.set_image(None, torch.zeros((3, 8, 16, 16), device=cuda))
    z = plan.apply(good)
    assert z.shape == good.shape and bool(torch.isfinite(z).all())
