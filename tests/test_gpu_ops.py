"""sm_103a kernels through the C ABI against the oracle and the reference fixtures (GPU)."""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

from conftest import rel_err
from oracle import laplacian as olap
from oracle import model as omodel
from oracle import ops as oops

pytestmark = pytest.mark.gpu
OPS = ["ops_8x8x8.npz", "ops_6x4x10.npz", "ops_16x16x16.npz"]
TOL = 1e-5  # FP32 kernels vs FP64 reference: max |diff| / max |ref|


def _t(a, dev, dt=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)


@pytest.mark.parametrize("name", OPS)
@pytest.mark.parametrize("transpose", [False, True])
def test_block_forward(golden, cuda, name, transpose):
    from mlpcg_gb300 import ops
    d = golden(name)
    y = ops.block_forward(_t(d["image"], cuda), _t(d["x"], cuda), _t(d["W"], cuda), _t(d["b"], cuda),
                          transpose=transpose)
    assert y.shape == d["x"].shape
    assert rel_err(y.cpu().numpy(), d["yt" if transpose else "y"]) < TOL


@pytest.mark.parametrize("name", OPS[:2])
@pytest.mark.parametrize("transpose", [False, True])
def test_extension_shims_take_padded_inputs(golden, cuda, name, transpose):
    from mlpcg_gb300.sm_model_3d import smblock3d, smblocktrans3d
    d = golden(name)
    ext = smblocktrans3d if transpose else smblock3d
    img, x = _t(d["image"], cuda), _t(d["x"], cuda)
    W, b = _t(d["W"], cuda), _t(d["b"], cuda)
    (y,) = ext.inference(F.pad(img, (1,) * 6), F.pad(x, (1,) * 6), W, b)
    assert rel_err(y.cpu().numpy(), d["yt" if transpose else "y"]) < TOL
    g = _t(d["g"], cuda)
    gx, gw, gb = ext.backward(g, F.pad(img, (1,) * 6), F.pad(x, (1,) * 6), W, b)
    sfx = "t" if transpose else ""
    assert rel_err(gx.cpu().numpy(), d["dx" + sfx]) < TOL
    assert rel_err(gw.cpu().numpy(), d["dW" + sfx]) < TOL
    assert rel_err(gb.cpu().numpy(), d["db" + sfx]) < TOL


def test_extension_rejects_cpu_and_noncontiguous(golden, cuda):
    from mlpcg_gb300.sm_model_3d import smblock3d
    d = golden(OPS[0])
    img, x = _t(d["image"], cuda), _t(d["x"], cuda)
    W, b = _t(d["W"], cuda), _t(d["b"], cuda)
    with pytest.raises(RuntimeError, match="must be a CUDA tensor"):
        smblock3d.inference(F.pad(img, (1,) * 6).cpu(), F.pad(x, (1,) * 6), W, b)
    with pytest.raises(RuntimeError, match="must be contiguous"):
        smblock3d.inference(F.pad(img, (1,) * 6), F.pad(x, (1,) * 6).transpose(-1, -2), W, b)


@pytest.mark.parametrize("name", OPS)
@pytest.mark.parametrize("transpose", [False, True])
def test_block_backward(golden, cuda, name, transpose):
    from mlpcg_gb300 import ops
    d = golden(name)
    gx, gw, gb, gi = ops.block_backward(_t(d["g"], cuda), _t(d["image"], cuda), _t(d["x"], cuda),
                                        _t(d["W"], cuda), _t(d["b"], cuda), transpose=transpose,
                                        image_grad=True)
    sfx = "t" if transpose else ""
    assert rel_err(gx.cpu().numpy(), d["dx" + sfx]) < TOL
    assert rel_err(gw.cpu().numpy(), d["dW" + sfx]) < TOL
    assert rel_err(gb.cpu().numpy(), d["db" + sfx]) < TOL
    assert rel_err(gi.cpu().numpy(), d["dimg" + sfx]) < TOL


@pytest.mark.parametrize("B", [1, 3, 128])
def test_block_any_batch(cuda, B):
    """The reference's dx kernels are only correct for B = 128; these take any B."""
    from mlpcg_gb300 import ops
    rng = np.random.default_rng(B)
    shape = (8, 6, 10)
    img = rng.random((3,) + shape)
    x = rng.random((B, 1) + shape)
    g = rng.random((B, 1) + shape)
    W = rng.uniform(-1 / 9, 1 / 9, (27, 3, 3, 3, 3))
    b = rng.uniform(-1 / 9, 1 / 9, 27)
    y = ops.block_forward(_t(img, cuda), _t(x, cuda), _t(W, cuda), _t(b, cuda))
    assert rel_err(y.cpu().numpy()[:, 0], oops.sm_block(img, x[:, 0], W, b)) < TOL
    gx, gw, gb, _ = ops.block_backward(_t(g, cuda), _t(img, cuda), _t(x, cuda), _t(W, cuda), _t(b, cuda))
    rgx, rgw, rgb, _ = oops.block_backward(g[:, 0], img, x[:, 0], W, b)
    assert rel_err(gx.cpu().numpy()[:, 0], rgx) < TOL
    assert rel_err(gw.cpu().numpy(), rgw) < TOL
    assert rel_err(gb.cpu().numpy(), rgb) < TOL


@pytest.mark.parametrize("kdt", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("xdt", [torch.float32, torch.bfloat16])
def test_precomputed_coefficients(golden, cuda, kdt, xdt):
    from mlpcg_gb300 import ops
    d = golden(OPS[2])
    dims = d["image"].shape[1:]
    K = ops.stencil_gen(_t(d["image"], cuda), _t(d["W"], cuda), _t(d["b"], cuda), dtype=kdt)
    Kref = oops.stencil_coeffs(d["image"], d["W"], d["b"]).reshape(27, -1)
    n = Kref.shape[1]
    tolK = TOL if kdt == torch.float32 else 4e-3
    assert rel_err(K[:, :n].float().cpu().numpy(), Kref) < tolK
    x = _t(d["x"], cuda, xdt)
    for tr, key in ((False, "y"), (True, "yt")):
        y = ops.stencil_apply(K, x, dims, transpose=tr)
        tol = TOL if (kdt == torch.float32 and xdt == torch.float32) else 3e-2
        assert rel_err(y.cpu().numpy(), d[key]) < tol


@pytest.mark.parametrize("name", OPS)
def test_linear(golden, cuda, name):
    from mlpcg_gb300 import ops
    d = golden(name)
    z, y = ops.linear_forward(_t(d["image"], cuda), _t(d["Wl"], cuda), _t(d["bl"], cuda))
    assert rel_err(z.cpu().numpy(), d["z"]) < TOL
    assert rel_err(y.cpu().numpy(), d["ylin"]) < TOL
    gi = ops.linear_image_grad(torch.ones(1, device=cuda), _t(d["Wl"], cuda), d["image"].shape[1:])
    assert rel_err(gi.cpu().numpy(), d["dimg_lin"]) < TOL
    gw, gb = ops.linear_backward(torch.full((1,), 2.0, device=cuda), y)
    assert rel_err(gw.cpu().numpy(), 2 * d["ylin"]) < TOL and float(gb) == 2.0


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 5, 2), (2, 2, 2), (3, 7, 4), (9, 2, 13)])
def test_linear_small_and_ragged(cuda, shape):
    from mlpcg_gb300 import ops
    rng = np.random.default_rng(sum(shape))
    img = rng.random((3,) + shape)
    W = rng.uniform(-1 / 9, 1 / 9, (1, 3, 3, 3, 3))
    b = rng.uniform(-1 / 9, 1 / 9, 1)
    z, y = ops.linear_forward(_t(img, cuda), _t(W, cuda), _t(b, cuda))
    rz, ry = oops.sm_linear(img, W, b)
    assert rel_err(y.cpu().numpy(), ry) < TOL
    assert abs(float(z) - rz[0]) <= TOL * max(1.0, abs(rz[0]))


@pytest.mark.parametrize("name", OPS)
def test_transfer(golden, cuda, name):
    from mlpcg_gb300 import ops
    d = golden(name)
    x = _t(d["x"], cuda)
    if "pool" in d:
        assert rel_err(ops.avg_pool2(x).cpu().numpy(), d["pool"]) < 1e-6
    assert rel_err(ops.upsample2(x).cpu().numpy(), d["up"]) < 1e-6
    # adjoints: <P x, y> = <x, P^T y>
    rng = np.random.default_rng(0)
    up = ops.upsample2(x)
    yy = _t(rng.random(up.shape), cuda)
    lhs = float((up.double() * yy.double()).sum())
    rhs = float((x.double() * ops.upsample2_adjoint(yy).double()).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)
    if "pool" in d:
        pl = ops.avg_pool2(x)
        yy = _t(rng.random(pl.shape), cuda)
        lhs = float((pl.double() * yy.double()).sum())
        rhs = float((x.double() * ops.avg_pool2_adjoint(yy).double()).sum())
        assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_axpby_and_dot(cuda):
    from mlpcg_gb300 import ops
    rng = np.random.default_rng(1)
    x, y = rng.standard_normal(100003), rng.standard_normal(100003)
    c0, c1 = torch.tensor([0.75], device=cuda), torch.tensor([-1.5], device=cuda)
    out = ops.axpby(c0, _t(x, cuda), c1, _t(y, cuda))
    np.testing.assert_allclose(out.cpu().numpy(), 0.75 * x - 1.5 * y, rtol=1e-6, atol=1e-6)
    for dt in (torch.float32, torch.float64):
        v = float(ops.dot(_t(x, cuda, dt), _t(y, cuda, dt)))
        ref = float(np.dot(_t(x, "cpu", dt).double().numpy(), _t(y, "cpu", dt).double().numpy()))
        assert abs(v - ref) <= 1e-12 * np.abs(x * y).sum()


@pytest.mark.parametrize("seed,shape", [(5, (12, 12, 12)), (6, (16, 8, 24))])
def test_laplacian(cuda, seed, shape):
    from mlpcg_gb300.laplacian import FluidLaplacian
    from mlpcg_gb300.scenes import make_scene
    s = make_scene(shape, seed)
    A, fluid = olap.assemble(s.flags)
    op = FluidLaplacian(torch.as_tensor(s.flags, device=cuda))
    xv = np.random.default_rng(seed).standard_normal(fluid.size)
    ref = A @ xv
    got = (op @ _t(xv, cuda, torch.float64)).cpu().numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-14, atol=1e-12)
    got32 = (op @ _t(xv, cuda, torch.float32)).cpu().numpy()
    assert rel_err(got32, ref) < 1e-6


def _model_from_fixture(d, cuda):
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D
    n = int(d["n"])
    m = SmallSMModelDn3D(n, 3, "trilinear").to(cuda)
    sd = {k[len("param:"):]: torch.as_tensor(v) for k, v in d.items() if k.startswith("param:")}
    m.load_state_dict(sd)
    return m


def test_model_forward_and_eval_forward(golden, cuda):
    d = golden("model_16_l3.npz")
    m = _model_from_fixture(d, cuda)
    img = _t(d["image"], cuda)
    p = {k[len("param:"):]: v for k, v in d.items() if k.startswith("param:")}
    ref = omodel.forward(p, d["image"], d["b"][:, 0], int(d["n"]))
    with torch.no_grad():
        y = m(img, _t(d["b"], cuda))
    assert rel_err(y.cpu().numpy()[:, 0], ref) < TOL
    assert rel_err(y.cpu().numpy(), d["y"]) < TOL
    ye = m.eval_forward(img, _t(d["b"][:1], cuda))
    assert rel_err(ye.cpu().numpy(), d["y_eval"]) < TOL


def test_model_gradients_vs_fp64_finite_differences(golden, cuda):
    """d<g, f(b)> / d(theta, b, image) from the adjoint kernels vs FP64 central differences of the oracle."""
    d = golden("model_16_l3.npz")
    m = _model_from_fixture(d, cuda)
    n = int(d["n"])
    p = {k[len("param:"):]: v.astype(np.float64) for k, v in d.items() if k.startswith("param:")}
    img_np = d["image"].astype(np.float64)
    b_np = d["b"][:1, 0].astype(np.float64)
    g_np = np.random.default_rng(7).standard_normal(b_np.shape)

    img = _t(img_np, cuda).requires_grad_(True)
    b = _t(b_np[:, None], cuda).requires_grad_(True)
    out = m(img, b)
    (out * _t(g_np[:, None], cuda)).sum().backward()
    grads = {k: v.grad.detach().cpu().numpy() for k, v in m.named_parameters()}

    def loss(pp=p, im=img_np, bb=b_np):
        return float((omodel.forward(pp, im, bb, n) * g_np).sum())

    rng = np.random.default_rng(11)
    h = 1e-4
    for name in ("pre.0.weight", "pre.1.bias", "post.0.weight", "l.weight", "c0.0.weight", "c1.1.bias"):
        for _ in range(3):
            idx = tuple(rng.integers(0, s) for s in p[name].shape)
            pp, pm = dict(p), dict(p)
            pp[name] = p[name].copy(); pp[name][idx] += h
            pm[name] = p[name].copy(); pm[name][idx] -= h
            fd = (loss(pp) - loss(pm)) / (2 * h)
            assert abs(grads[name][idx] - fd) <= 2e-3 * max(1.0, abs(fd)) + 1e-5, (name, idx, grads[name][idx], fd)
    # input vector: f is linear in b, so the directional derivative is exact
    v = rng.standard_normal(b_np.shape)
    fd = (loss(bb=b_np + h * v) - loss(bb=b_np - h * v)) / (2 * h)
    assert abs(float((b.grad.cpu().numpy()[:, 0] * v).sum()) - fd) <= 1e-4 * max(1.0, abs(fd))
    # image channels
    for _ in range(4):
        idx = (int(rng.integers(0, 3)),) + tuple(int(rng.integers(1, 15)) for _ in range(3))
        ip, im_ = img_np.copy(), img_np.copy()
        ip[idx] += h
        im_[idx] -= h
        fd = (loss(im=ip) - loss(im=im_)) / (2 * h)
        assert abs(img.grad.cpu().numpy()[idx] - fd) <= 2e-3 * max(1.0, abs(fd)) + 1e-5


def test_residual_histories_50_iterations(golden, cuda):
    """The plain FP32 path (drop-in solvers, FP64 vectors, FP32 network through the library
    kernels) reproduces the reference's residual histories within 1e-4 relative over the first
    50 iterations, on the reference's SmallSMModelDn3D moved near the identity (steadily falling
    residuals)."""
    from mlpcg_gb300 import cg
    from mlpcg_gb300.laplacian import FluidLaplacian
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D
    d = golden("cg_16_l3_near_identity.npz")
    m = SmallSMModelDn3D(int(d["n"]), 3, "trilinear").to(cuda)
    m.load_state_dict({k[len("param:"):]: torch.as_tensor(v) for k, v in d.items() if k.startswith("param:")})
    flags = torch.as_tensor(d["flags"], device=cuda)
    A = FluidLaplacian(flags)
    img = _t(d["image"], cuda)
    b = _t(d["rhs"].ravel()[A.fluid_cells.cpu().numpy()], cuda, torch.float64)
    for name in ("npsd", "npcg", "npcg_flex"):
        hist = []
        pred = cg.model_predict(m, img, A.fluid_cells)
        getattr(cg, name)(b, A, torch.zeros_like(b), pred, 50, tol=1e-6, atol=1e-20,
                          callback=lambda nrm, t: hist.append(nrm))
        ref = d[f"{name}_hist"]
        assert len(hist) == len(ref) == 51
        np.testing.assert_allclose(np.array(hist), ref, rtol=1e-4, err_msg=name)


def test_npsd_npcg_residual_histories(golden, cuda):
    """Drop-in solvers (FP64 vectors, FP32 network) vs the reference's cg_tests.py histories."""
    from mlpcg_gb300 import cg
    from mlpcg_gb300.laplacian import FluidLaplacian
    d = golden("cg_16_l3.npz")
    md = golden("model_16_l3.npz")
    m = _model_from_fixture(md, cuda)
    flags = torch.as_tensor(d["flags"], device=cuda)
    A = FluidLaplacian(flags)
    img = _t(md["image"], cuda)
    b = _t(d["rhs"].ravel()[A.fluid_cells.cpu().numpy()], cuda, torch.float64)
    for name in ("npsd", "npcg", "npcg_flex"):
        hist = []
        pred = cg.model_predict(m, img, A.fluid_cells)
        x, it, timer, res = getattr(cg, name)(b, A, torch.zeros_like(b), pred, 50, tol=1e-6, atol=1e-20,
                                              callback=lambda nrm, t: hist.append(nrm))
        ref = d[f"{name}_hist"]
        k = min(len(hist), len(ref))
        h, r = np.array(hist[:k]), ref[:k]
        ok = np.isfinite(r) & (r < 1e3)
        # this random-init network makes the residual stagnate near 1, where FP32 rounding of the
        # network builds up over the iterations: the first 30 are pinned here, 50 on the
        # near-identity network below
        np.testing.assert_allclose(h[ok][:31], r[ok][:31], rtol=1e-4)
        if name != "npcg_flex":
            assert it == int(d[f"{name}_iters"])


def test_ops_refuse_mismatched_sizes(cuda):
    """The size relations the kernels rely on (weights, gradients, plane strides, operand lengths)
    are checked before any launch; a valid call still runs afterwards."""
    from mlpcg_gb300 import ops
    img = torch.zeros((3, 8, 8, 8), device=cuda)
    x = torch.zeros((1, 1, 8, 8, 8), device=cuda)
    W, b = torch.zeros((27, 3, 3, 3, 3), device=cuda), torch.zeros(27, device=cuda)
    one = torch.ones(1, device=cuda)
    with pytest.raises(RuntimeError):
        ops.block_forward(img, x, W[:20], b)
    with pytest.raises(RuntimeError):
        ops.block_backward(torch.zeros((1, 1, 8, 8, 4), device=cuda), img, x, W, b)
    with pytest.raises(RuntimeError):
        ops.axpby(one, torch.zeros(10, device=cuda), one, torch.zeros(9, device=cuda))
    with pytest.raises(RuntimeError):
        ops.laplacian(torch.zeros((8, 8, 8), dtype=torch.uint8, device=cuda), torch.zeros(100, device=cuda))
    K = ops.stencil_gen(img, W, b)
    with pytest.raises(RuntimeError):
        ops.stencil_apply(K, torch.zeros(100, device=cuda), (8, 8, 8))
    with pytest.raises(RuntimeError):
        ops.stencil_apply(K[:20].contiguous(), x, (8, 8, 8))
    y = ops.block_forward(img, x, W, b)
    assert y.shape == x.shape
