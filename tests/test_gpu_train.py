"""Training pieces: Lanczos Ritz pairs vs the FP64 oracle matrix, loss adjoint, a few Adam steps (GPU)."""
import numpy as np
import pytest
import torch

from oracle import laplacian as olap

pytestmark = pytest.mark.gpu


def test_lanczos_ritz_pairs_match_dense_eigenpairs(cuda):
    """The six lowest Ritz values equal the FP64 oracle matrix's eigenvalues (dense eigvalsh), the
    Ritz vectors are eigenvectors to 1e-6, and the mixed right-hand sides have unit norm."""
    from mlpcg_gb300.lanczos import lanczos_ritz, mix_rhs
    from mlpcg_gb300.laplacian import FluidLaplacian
    from mlpcg_gb300.scenes import make_scene
    s = make_scene(12, 9)
    A = FluidLaplacian(torch.as_tensor(s.flags, device=cuda))
    Ac, fluid = olap.assemble(s.flags)
    v0 = torch.as_tensor(s.rhs.ravel()[fluid], device=cuda)
    vals, vecs = lanczos_ritz(A, v0, steps=Ac.shape[0], n_ritz=6)
    ref = np.sort(np.linalg.eigvalsh(Ac.toarray()))[:6]
    np.testing.assert_allclose(vals, ref, rtol=1e-8, atol=1e-10)
    V = vecs.cpu().numpy()
    for k in range(6):
        res = Ac @ V[k] - vals[k] * V[k]
        assert np.linalg.norm(res) < 1e-6
    b = mix_rhs(vecs, 4)
    assert torch.allclose(b.norm(dim=1), torch.ones(4, dtype=b.dtype, device=cuda))


def test_laplacian_function_adjoint(cuda):
    from mlpcg_gb300.train import LaplacianFunction
    from mlpcg_gb300.scenes import make_scene
    s = make_scene(16, 2)
    flags = torch.as_tensor(s.flags, device=cuda)
    x = torch.randn((3,) + s.shape, device=cuda, requires_grad=True)
    g = torch.randn((3,) + s.shape, device=cuda)
    y = LaplacianFunction.apply(flags, x)
    (y * g).sum().backward()
    lhs = float((y.detach().double() * g.double()).sum())
    rhs = float((x.double() * x.grad.double()).sum())
    # <A x, g> = <x, A g>
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_training_steps_reduce_loss(cuda):
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D
    from mlpcg_gb300.train import TrainScene, residual_loss
    torch.manual_seed(0)
    model = SmallSMModelDn3D(3, 3, "trilinear").to(cuda)
    sc = TrainScene((32, 32, 32), 10, cuda, n_ritz=16, lanczos_steps=80)
    opt = torch.optim.Adam(model.parameters(), lr=3e-3)
    gen = torch.Generator(device=cuda)
    gen.manual_seed(0)
    b = sc.batch(8, 0.25, gen)
    first = None
    for _ in range(30):
        loss = residual_loss(model, sc.image, sc.flags, sc.fluid, b)
        first = float(loss) if first is None else first
        opt.zero_grad()
        loss.backward()
        opt.step()
    assert float(loss) < 0.8 * first


def test_training_symmetric_network(cuda, tmp_path):
    """A few steps of the training loop on SmallSPDSMModelDn3D (near-identity start, npcg
    validation and harvesting through the fused SPD plan) reduce the loss and save smallspd_l3."""
    from mlpcg_gb300 import train
    train.main(["--out", str(tmp_path), "--model", "small_spd", "--size", "32", "--levels", "3", "--seeds", "10",
                "--steps", "100", "--batch", "4", "--lanczos-steps", "80", "--n-ritz", "16", "--eval-every", "100",
                "--val-size", "32", "--val-seed", "11", "--harvest-every", "50"])
    log = __import__("json").loads((tmp_path / "smallspd_l3.train.json").read_text())
    assert (tmp_path / "smallspd_l3.npz").exists()
    assert all(0.0 <= e["loss"] <= 1.0 for e in log["loss"]) and len(log["loss"]) == 2
    first, last = log["eval"][0], log["eval"][-1]
    assert last["status"] == "converged" and last["iterations"] <= first["iterations"], log["eval"]


def test_recompute_gives_the_same_gradients_with_less_memory(cuda):
    """SmallSMModelDn3D.recompute: per-level activations recomputed in the backward pass -- the
    same loss and gradients (input, image, every parameter), a lower peak of stored activations."""
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D
    torch.manual_seed(0)
    model = SmallSMModelDn3D(3, 3, "trilinear").to(cuda)
    shape = (64, 64, 64)
    torch.manual_seed(1)
    img = (torch.rand((3,) + shape, device=cuda) > 0.5).float()
    b0 = torch.randn((4, 1) + shape, device=cuda)
    g = torch.randn_like(b0)
    out = {}
    for rec in (False, True):
        model.recompute = rec
        model.zero_grad(set_to_none=True)
        b = b0.clone().requires_grad_(True)
        im = img.clone().requires_grad_(True)
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats(cuda)
        base = torch.cuda.memory_allocated(cuda)
        y = model(im, b)
        kept = torch.cuda.memory_allocated(cuda) - base   # what the forward keeps for the backward
        (y * g).sum().backward()
        torch.cuda.synchronize()
        out[rec] = (y.detach(), b.grad, im.grad, {k: p.grad.clone() for k, p in model.named_parameters()}, kept)
    model.recompute = False
    y0, gb0, gi0, gp0, kept0 = out[False]
    y1, gb1, gi1, gp1, kept1 = out[True]
    assert torch.equal(y0, y1) and torch.equal(gb0, gb1)
    # the image gradient sums contributions of several paths, possibly in another order
    torch.testing.assert_close(gi1, gi0, rtol=1e-5, atol=1e-7)
    for k in gp0:
        assert torch.equal(gp0[k], gp1[k]), k
    assert kept1 < 0.75 * kept0, (kept0, kept1)


def test_residual_loss_reference_kind_matches_the_reference(golden, cuda):
    """train.loss_of_outputs(kind="reference") -- the loss of residual_loss(kind="reference") -- against
    the reference's loss_functions.residual_loss (loss_functions.py:18-23, mean over the batch of
    ||y - x A||, CSC matrix) on the same FP64 batch of a 16^3 scene (fixture from the reference)."""
    from mlpcg_gb300.train import loss_of_outputs
    d = golden("residual_loss_16.npz")
    flags = torch.as_tensor(d["flags"], device=cuda)
    fluid = torch.nonzero(flags.reshape(-1) == 2).reshape(-1)
    B = d["x"].shape[0]
    n = flags.numel()
    xg = torch.zeros((B, n), dtype=torch.float64, device=cuda)
    yg = torch.zeros((B, n), dtype=torch.float64, device=cuda)
    xg[:, fluid] = torch.as_tensor(d["x"], device=cuda)
    yg[:, fluid] = torch.as_tensor(d["y"], device=cuda)
    shp = (B,) + tuple(flags.shape)
    loss = float(loss_of_outputs(xg.reshape(shp), yg.reshape(shp), flags, kind="reference"))
    assert loss == pytest.approx(float(d["loss_mean"]), rel=1e-12)
    assert loss * B == pytest.approx(float(d["loss_sum"]), rel=1e-12)


def test_bf16_training_storage(cuda):
    """Training with BF16 block storage (coefficient planes and saved inputs in BF16, FP32 sums):
    the forward output and every gradient (input, image, parameters) agree with the FP32 training
    path within BF16 rounding, the saved activations shrink, and a few optimiser steps reduce the
    loss as in FP32."""
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D, set_training_storage
    from mlpcg_gb300.train import TrainScene, residual_loss
    torch.manual_seed(0)
    model = SmallSMModelDn3D(3, 3, "trilinear").to(cuda)
    shape = (32, 32, 32)
    torch.manual_seed(1)
    img = (torch.rand((3,) + shape, device=cuda) > 0.5).float()
    b0 = torch.randn((4, 1) + shape, device=cuda)
    g = torch.randn_like(b0)
    out = {}
    for dt in (torch.float32, torch.bfloat16):
        set_training_storage(model, dt)
        model.zero_grad(set_to_none=True)
        b = b0.clone().requires_grad_(True)
        im = img.clone().requires_grad_(True)
        y = model(im, b)
        (y * g).sum().backward()
        out[dt] = (y.detach(), b.grad, im.grad, {k: p.grad.clone() for k, p in model.named_parameters()})
    set_training_storage(model, torch.float32)
    (y0, gb0, gi0, gp0), (y1, gb1, gi1, gp1) = out[torch.float32], out[torch.bfloat16]

    def rel(a, b):
        return float((a - b).norm() / b.norm())
    assert rel(y1, y0) < 2e-2 and rel(gb1, gb0) < 2e-2 and rel(gi1, gi0) < 3e-2
    for k in gp0:
        assert rel(gp1[k], gp0[k]) < 3e-2, (k, rel(gp1[k], gp0[k]))
    with pytest.raises(ValueError):
        set_training_storage(model, torch.float16)
    # a few steps reduce the loss
    set_training_storage(model, torch.bfloat16)
    sc = TrainScene(shape, 10, cuda, n_ritz=16, lanczos_steps=80)
    opt = torch.optim.Adam(model.parameters(), lr=3e-3)
    gen = torch.Generator(device=cuda)
    gen.manual_seed(0)
    b = sc.batch(8, 0.25, gen)
    first = None
    for _ in range(30):
        loss = residual_loss(model, sc.image, sc.flags, sc.fluid, b)
        first = float(loss) if first is None else first
        opt.zero_grad()
        loss.backward()
        opt.step()
    set_training_storage(model, torch.float32)
    assert float(loss) < 0.8 * first
