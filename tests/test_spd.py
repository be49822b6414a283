"""SPD preconditioners SPDSMModelDn3D / SmallSPDSMModelDn3D (sm_model_3d.py:290-444).

CPU: the oracle compositions against the reference's own outputs, the module
tree against its state dict and initial weights.  GPU: the drop-in classes
(library kernels) against the oracle and the reference, their gradients against
FP64 central differences, the operator's symmetry (the reference's self-test,
sm_model_3d.py:476-485), and the drop-in CG solvers' residual histories against
the reference's cg_tests.py run with the same network.
"""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import cg as ocg
from oracle import laplacian as olap
from oracle import model as omodel

MODELS = [("spd_16_l2.npz", "SPDSMModelDn3D", omodel.spd_forward),
          ("small_spd_16_l3.npz", "SmallSPDSMModelDn3D", omodel.small_spd_forward)]
IDS = ["SPDSMModelDn3D", "SmallSPDSMModelDn3D"]


def _params(d, dt=None):
    return {k[len("param:"):]: (v if dt is None else v.astype(dt)) for k, v in d.items() if k.startswith("param:")}


@pytest.mark.parametrize("fname,cls,fwd", MODELS, ids=IDS)
def test_oracle_vs_reference(golden, fname, cls, fwd):
    d = golden(fname)
    p, n = _params(d), int(d["n"])
    assert rel_err(fwd(p, d["image"], d["b"][:, 0], n), d["y"][:, 0]) < 1e-5  # reference ran in fp32
    assert rel_err(fwd(p, d["image"], d["b"][:1, 0], n), d["y_eval"][:, 0]) < 1e-5


@pytest.mark.parametrize("fname,cls,fwd", MODELS, ids=IDS)
def test_init_order_and_keys(golden, fname, cls, fwd):
    """The module tree draws the reference's initial weights under torch.manual_seed(0) and has its
    state-dict keys (the transposed blocks list the shared parameters again)."""
    from mlpcg_gb300 import sm_model_3d
    d = golden(fname)
    ref = _params(d)
    torch.manual_seed(0)
    m = getattr(sm_model_3d, cls)(int(d["n"]))
    sd = m.state_dict()
    assert sorted(sd) == sorted(ref)
    for k, v in sd.items():
        np.testing.assert_array_equal(v.numpy(), ref[k])
    assert m.l0_t[0].weight is m.l0[0].weight and m.l_t.bias is m.l.bias
    small = cls.startswith("Small")
    names = omodel.spd_param_names(int(d["n"]), small=small)
    # drawing in that order reproduces every initial weight
    torch.manual_seed(0)
    for name in names:
        w, bias = torch.ones(27, 3, 3, 3, 3), torch.ones(27)
        m.reset_parameters(w, bias)
        if name[0] == "c":  # SmallLinearBlock3DNew keeps the means
            w, bias = w.mean(0, keepdim=True), bias.mean(0, keepdim=True)
        np.testing.assert_array_equal(w.numpy(), ref[name + ".weight"])
        np.testing.assert_array_equal(bias.numpy(), ref[name + ".bias"])


@pytest.mark.parametrize("fname,cls,fwd", MODELS, ids=IDS)
def test_oracle_symmetry(golden, fname, cls, fwd):
    """<x, M y> = <y, M x> in FP64 for both SPD compositions (M = V^T V, M = S^T S)."""
    d = golden(fname)
    p, n = _params(d, np.float64), int(d["n"])
    rng = np.random.default_rng(3)
    x, y = rng.standard_normal((2,) + d["image"].shape[1:])
    a = float((x * fwd(p, d["image"], y, n)).sum())
    b = float((y * fwd(p, d["image"], x, n)).sum())
    assert abs(a - b) <= 1e-12 * max(abs(a), 1.0)
    assert float((x * fwd(p, d["image"], x, n)).sum()) >= 0.0


@pytest.mark.parametrize("fname,cpu_cls", [("small_spd_16_l3.npz", "CPUSPDModel"), ("spd_16_l2.npz", "CPUSPDFullModel")])
def test_cpu_path_spd(golden, fname, cpu_cls):
    """The timed CPU baseline's symmetric networks (torch-CPU blocks, scatter transpose) against
    the reference's output."""
    from oracle import cpu_path
    d = golden(fname)
    m = getattr(cpu_path, cpu_cls)({k: torch.from_numpy(v) for k, v in _params(d).items()}, int(d["n"]))
    y = m(torch.from_numpy(d["image"]), torch.from_numpy(d["b"][:1])).numpy()
    assert rel_err(y, d["y_eval"]) < 1e-5


# ---------------------------------------------------------------------------- GPU
def _t(a, dev, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


def _model(d, cls, cuda):
    from mlpcg_gb300 import sm_model_3d
    m = getattr(sm_model_3d, cls)(int(d["n"])).to(cuda)
    m.load_state_dict({k: torch.as_tensor(v) for k, v in _params(d).items()})
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("fname,cls,fwd", MODELS, ids=IDS)
def test_forward_and_eval_forward(golden, cuda, fname, cls, fwd):
    d = golden(fname)
    m = _model(d, cls, cuda)
    img = _t(d["image"], cuda)
    ref = fwd(_params(d), d["image"], d["b"][:, 0], int(d["n"]))
    with torch.no_grad():
        y = m(img, _t(d["b"], cuda))
    assert rel_err(y.cpu().numpy()[:, 0], ref) < 1e-5
    assert rel_err(y.cpu().numpy(), d["y"]) < 1e-5
    imgs, c0, c1 = [], [], []
    ye = m.eval_forward(img, _t(d["b"][:1], cuda), None, imgs, c0, c1)
    assert rel_err(ye.cpu().numpy(), d["y_eval"]) < 1e-5
    # a second call reuses the cached pyramid and level coefficients
    assert len(imgs) == int(d["n"]) + 1 and len(c0) == len(c1) == int(d["n"])
    ye2 = m.eval_forward(img, _t(d["b"][1:], cuda), None, imgs, c0, c1)
    assert rel_err(ye2.cpu().numpy()[:, 0], ref[1:]) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("fname,cls,fwd", MODELS, ids=IDS)
def test_gradients_vs_fp64_finite_differences(golden, cuda, fname, cls, fwd):
    """d<g, M b> / d(theta, b) from the adjoint kernels vs FP64 central differences of the oracle;
    a shared parameter collects the gradients of the block and of its transpose."""
    d = golden(fname)
    m = _model(d, cls, cuda)
    n = int(d["n"])
    p = _params(d, np.float64)
    img_np = d["image"].astype(np.float64)
    b_np = d["b"][:1, 0].astype(np.float64)
    g_np = np.random.default_rng(5).standard_normal(b_np.shape)
    b = _t(b_np[:, None], cuda).requires_grad_(True)
    out = m(_t(img_np, cuda), b)
    (out * _t(g_np[:, None], cuda)).sum().backward()
    grads = {k: v.grad.detach().cpu().numpy() for k, v in m.named_parameters()}

    def loss(pp=p, bb=b_np):
        return float((fwd(pp, img_np, bb, n) * g_np).sum())

    rng = np.random.default_rng(13)
    h = 1e-4
    names = ["l0.0.weight", "l0.1.bias", "l.weight", "c0.0.weight", "c1.1.bias"]
    if not cls.startswith("Small"):
        names += ["l1.0.weight", "l1.1.bias"]
    for name in names:
        for _ in range(2):
            idx = tuple(rng.integers(0, s) for s in p[name].shape)
            pp, pm = dict(p), dict(p)
            pp[name] = p[name].copy(); pp[name][idx] += h
            pm[name] = p[name].copy(); pm[name][idx] -= h
            fd = (loss(pp) - loss(pm)) / (2 * h)
            assert abs(grads[name][idx] - fd) <= 2e-3 * max(1.0, abs(fd)) + 1e-5, (name, idx, grads[name][idx], fd)
    v = rng.standard_normal(b_np.shape)
    fd = (loss(bb=b_np + h * v) - loss(bb=b_np - h * v)) / (2 * h)
    assert abs(float((b.grad.cpu().numpy()[:, 0] * v).sum()) - fd) <= 1e-4 * max(1.0, abs(fd))


@pytest.mark.gpu
@pytest.mark.parametrize("cls,n,shape,batch", [("SmallSPDSMModelDn3D", 4, (64, 64, 64), 8),
                                               ("SPDSMModelDn3D", 3, (32, 48, 64), 4)])
def test_symmetry_self_test(cuda, cls, n, shape, batch):
    """The reference's self-test (sm_model_3d.py:476-485): |x^T M y - y^T M x| over a batch of
    random vectors on a random image, absolute and relative to sqrt(|a| |b|)."""
    from mlpcg_gb300 import sm_model_3d
    torch.manual_seed(0)
    model = getattr(sm_model_3d, cls)(n).to(cuda)
    x = torch.rand(batch, 1, *shape, device=cuda)
    y = torch.rand(batch, 1, *shape, device=cuda)
    img = torch.rand(3, *shape, device=cuda)
    with torch.no_grad():
        z = model(img, x)
        z1 = model(img, y)
    a = torch.bmm(x.flatten(2).double(), z1.flatten(1).unsqueeze(-1).double())
    b = torch.bmm(y.flatten(2).double(), z.flatten(1).unsqueeze(-1).double())
    rel = ((a - b).norm() / torch.sqrt(a.abs() * b.abs()).norm()).item()
    assert rel < 1e-5, rel


@pytest.mark.gpu
@pytest.mark.parametrize("fname,cls,fwd", MODELS, ids=IDS)
def test_solver_histories_vs_reference(golden, cuda, fname, cls, fwd):
    """npsd / npcg / npcg_flex with the SPD network through the drop-in solvers vs the
    reference's cg_tests.py run and the oracle's (first 30 iterations)."""
    from mlpcg_gb300 import cg
    from mlpcg_gb300.laplacian import FluidLaplacian
    d = golden("cg_" + fname)
    md = golden(fname)
    m = _model(md, cls, cuda)
    flags = torch.as_tensor(d["flags"], device=cuda)
    A = FluidLaplacian(flags)
    img = _t(md["image"], cuda)
    b = _t(d["rhs"].ravel()[A.fluid_cells.cpu().numpy()], cuda, torch.float64)
    Ao, fluid = olap.assemble(d["flags"])
    p, n = _params(md, np.float64), int(md["n"])
    pred_o = ocg.make_predict(lambda g: fwd(p, md["image"], g, n), fluid, d["flags"].shape)
    for name in ("npsd", "npcg", "npcg_flex"):
        hist = []
        pred = cg.model_predict(m, img, A.fluid_cells)
        getattr(cg, name)(b, A, torch.zeros_like(b), pred, 50, tol=1e-6, atol=1e-20,
                          callback=lambda nrm, t: hist.append(nrm))
        ref = d[f"{name}_hist"]
        k = min(len(hist), len(ref))
        # random-init networks: the residual stagnates and FP32 rounding builds up; first 30 pinned
        np.testing.assert_allclose(np.array(hist[:k])[:31], ref[:k][:31], rtol=1e-4)
        _, _, hist_o = getattr(ocg, name)(d["rhs"].ravel()[fluid], Ao, np.zeros(fluid.size), pred_o, 30,
                                          tol=1e-6, atol=1e-20)
        np.testing.assert_allclose(np.array(hist[:31]), np.array(hist_o[:31]), rtol=1e-4)


# ---------------------------------------------------------------------------- fused plan (GPU)
PLAN_CLASSES = ["SmallSPDSMModelDn3D", "SPDSMModelDn3D"]


def _spd_model(n, dev, seed=0, eps=0.05, cls="SmallSPDSMModelDn3D"):
    """A symmetric network with small random weights around the identity stencil."""
    from mlpcg_gb300 import sm_model_3d
    torch.manual_seed(seed)
    m = getattr(sm_model_3d, cls)(n).to(dev)
    with torch.no_grad():
        for p in m.parameters():
            p.mul_(eps)
        for blk in list(m.l0) + list(getattr(m, "l1", [])) + [m.l]:
            blk.bias[13] += 1.0
        for c in m.c0:
            c.bias[0] += 1.0
    return m


def _scene(shape, seed, dev):
    from mlpcg_gb300.scenes import make_scene
    s = make_scene(shape, seed)
    return s, torch.as_tensor(s.flags, device=dev), torch.as_tensor(s.image(), device=dev)


@pytest.mark.gpu
@pytest.mark.parametrize("cls", PLAN_CLASSES)
@pytest.mark.parametrize("shape,n", [((16, 16, 16), 3), ((32, 16, 24), 3), ((64, 64, 64), 4), ((24, 40, 8), 3)])
def test_plan_matches_eval_forward(cuda, shape, n, cls):
    """The fused plan (transposed blocks gathered from the forward coefficients, nearest x2 / 8
    prolongation fused into the combine) against the drop-in eval_forward on the fluid cells."""
    s, flags, img = _scene(shape, 2, cuda)
    torch.manual_seed(1)
    from mlpcg_gb300 import sm_model_3d
    m = getattr(sm_model_3d, cls)(n).to(cuda)
    plan = m.precond_plan(img, storage=torch.float32)
    b = torch.randn((1, 1) + shape, device=cuda)
    ref = m.eval_forward(img, b)
    ref = torch.where(img[1] == 0, 0.0, ref)
    z = plan.apply(b.reshape(-1)).reshape(ref.shape)
    assert rel_err(z.cpu().numpy(), ref.cpu().numpy()) < 1e-5
    # the stages one at a time give the same output
    names = plan.stage_names()
    assert len(names) == (4 * n + 2 if cls == "SPDSMModelDn3D" else 2 * n + 1)
    zs = torch.empty_like(z.reshape(-1))
    for st in range(len(names)):
        plan.apply_stages(st, st, b.reshape(-1), None, zs)
    assert torch.equal(zs, z.reshape(-1))
    c = plan.coefficients()
    imgs = [img]
    from mlpcg_gb300 import ops
    for l in range(n):
        c0 = float(m.c0[l].eval_forward(imgs[l]))
        want = c0 * c0 if cls == "SmallSPDSMModelDn3D" else c0
        assert abs(float(c[l]) - want) <= 1e-6 * max(1.0, abs(want))
        imgs.append(ops.avg_pool2(imgs[-1]))


@pytest.mark.gpu
@pytest.mark.parametrize("cls", PLAN_CLASSES)
@pytest.mark.parametrize("shape,n,seed", [((64, 64, 64), 4, 4), ((32, 48, 64), 3, 9), ((128, 128, 128), 5, 7)])
@pytest.mark.parametrize("storage", [torch.float32, torch.bfloat16])
def test_plan_classed_is_bit_identical_to_dense(cuda, shape, n, seed, storage, cls):
    """The transposed blocks' classed records (radius-2 classes, gathered general cells) give
    exactly the dense transposed planes' output."""
    from mlpcg_gb300.precond import PrecondPlan
    s, flags, img = _scene(shape, seed, cuda)
    m = _spd_model(n, cuda, seed=3, cls=cls)
    dense = PrecondPlan(m, img, storage=storage, layout="dense")
    cls = PrecondPlan(m, img, storage=storage, layout="classed")
    n0 = int(np.prod(shape))
    b = torch.randn(n0, device=cuda)
    scale = torch.tensor([0.5], device=cuda)
    zd = dense.apply(b, scale)
    zc = cls.apply(b, scale)
    assert torch.equal(zd, zc), float((zd - zc).abs().max())


@pytest.mark.gpu
@pytest.mark.parametrize("cls", PLAN_CLASSES)
@pytest.mark.parametrize("layout", ["classed", "dense"])
def test_plan_operator_is_symmetric(cuda, layout, cls):
    """On fluid-supported vectors the plan's z = D M D r is symmetric positive definite."""
    from mlpcg_gb300.precond import PrecondPlan
    shape = (64, 64, 64)
    s, flags, img = _scene(shape, 5, cuda)
    m = _spd_model(4, cuda, seed=2, eps=0.2, cls=cls)
    plan = PrecondPlan(m, img, storage=torch.float32, layout=layout)
    fluid = (img[1] != 0).reshape(-1)
    g = torch.Generator(device=cuda).manual_seed(0)
    x = torch.randn(fluid.numel(), device=cuda, generator=g) * fluid
    y = torch.randn(fluid.numel(), device=cuda, generator=g) * fluid
    a = torch.dot(x.double(), plan.apply(y).double())
    b = torch.dot(y.double(), plan.apply(x).double())
    assert abs(float(a - b)) <= 1e-5 * float(torch.sqrt(a.abs() * b.abs())), (float(a), float(b))
    assert float(torch.dot(x.double(), plan.apply(x).double())) > 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("cls", PLAN_CLASSES)
@pytest.mark.parametrize("storage", [torch.float32, torch.bfloat16])
def test_fused_npcg_with_spd_network(cuda, storage, cls):
    """Textbook PCG (npcg) in the graph-captured solver with the symmetric network converges, and
    its FP64 residual against the oracle's matrix meets the tolerance."""
    from mlpcg_gb300.solver import FusedSolver
    shape = (64, 64, 64)
    s, flags, img = _scene(shape, 3, cuda)
    m = _spd_model(4, cuda, seed=4, cls=cls)
    solver = FusedSolver(m, flags, method="npcg", max_it=500, tol=1e-6, storage=storage)
    b = torch.as_tensor(s.rhs, device=cuda)
    res = solver.solve(b)
    assert res.status == "converged", res
    A, fluid = olap.assemble(s.flags)
    x = res.x.reshape(-1).cpu().numpy()[fluid]
    rhs = s.rhs.reshape(-1)[fluid]
    assert np.linalg.norm(rhs - A @ x) / np.linalg.norm(rhs) < 2e-6
