"""Parity at the benchmark configurations, against fixtures recorded from the reference itself.

64^3 (seed 0, 3 spheres), 4 levels, the reference's SmallSMModelDn3D drawn under
torch.manual_seed(0) (random init), FP32, max 100 iterations, tol 1e-6, atol 1e-20 --
the configuration of the plain method (cg_64_l4_seed0.npz, made by
tests/golden/make_golden.py --only=config0 from the reference's sm_model_3d.py with
its blocks evaluated by sm_model_3d_py.py, its cg_tests.py solvers and test.py's
model_predict; the matrix is the oracle's assembly, pinned to the reference's
lap_with_bc at 12^3, whose LIL assembly cannot run at 64^3).

Checked on the GPU:
* the initial weights: this package's SmallSMModelDn3D(4) under torch.manual_seed(0)
  draws the reference's (bit for bit; the linear blocks' means to 1e-6, since torch's
  CPU mean may round differently on another architecture);
* the preconditioner output on the first normalised right-hand side: the drop-in
  eval_forward and the fused FP32 plan (directly, not through the drop-in) within 1e-5
  of the reference's, the BF16 plan within the stated 2e-2;
* the residual histories of npsd, npcg and npcg_flex over the first 50 iterations
  within 1e-4 relative: the drop-in solvers (FP64 vectors) and the fused FP32 solver
  (FP32 CG vectors, double-float iterate).  With this random-init network the residual
  stagnates near 0.97 of ||b||, far above 1e-3, so the whole 50-iteration prefix is
  compared.
"""
import numpy as np
import pytest
import torch

from conftest import rel_err

pytestmark = pytest.mark.gpu

FIX = "cg_64_l4_seed0.npz"


def _setup(golden, cuda):
    from mlpcg_gb300.laplacian import FluidLaplacian
    from mlpcg_gb300.scenes import make_scene
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D
    d = golden(FIX)
    size, seed, n = int(d["size"]), int(d["seed"]), int(d["n"])
    scene = make_scene(size, seed, int(d["spheres"]))
    assert int(scene.flags.astype(np.int64).sum()) == int(d["flags_sum"])
    m = SmallSMModelDn3D(n, 3, "trilinear").to(cuda)
    m.load_state_dict({k[len("param:"):]: torch.as_tensor(v) for k, v in d.items() if k.startswith("param:")})
    flags = torch.as_tensor(scene.flags, device=cuda)
    A = FluidLaplacian(flags)
    img = torch.as_tensor(scene.image(), device=cuda)
    b = torch.as_tensor(scene.rhs.ravel()[A.fluid_cells.cpu().numpy()], device=cuda, dtype=torch.float64)
    assert abs(float(b.norm()) - float(d["rhs_norm"])) <= 1e-12 * float(d["rhs_norm"])
    return d, scene, m, flags, A, img, b


def test_config0_initial_weights_are_the_references(golden, cuda):
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D
    d = golden(FIX)
    torch.manual_seed(0)
    m = SmallSMModelDn3D(int(d["n"]), 3, "trilinear")
    sd = m.state_dict()
    keys = [k[len("param:"):] for k in d if k.startswith("param:")]
    assert sorted(keys) == sorted(sd.keys())
    for k in keys:
        ref = torch.as_tensor(d["param:" + k])
        if k.startswith(("c0.", "c1.")):
            # the linear blocks' weights are the mean of a (27, 3, 3, 3, 3) draw (sm_model_3d.py:149-153):
            # torch's CPU mean may round its sum differently on another CPU architecture or torch version
            torch.testing.assert_close(sd[k], ref, rtol=1e-6, atol=1e-9, msg=k)
        else:
            assert torch.equal(sd[k], ref), k


def test_config0_preconditioner_output(golden, cuda):
    d, scene, m, flags, A, img, b = _setup(golden, cuda)
    b0 = torch.as_tensor(d["b0"], device=cuda).reshape((1, 1) + scene.shape)
    y0 = d["y0"]
    # the drop-in path (library kernels, coefficients evaluated per block call)
    ye = m.eval_forward(img, b0).cpu().numpy().reshape(scene.shape)
    assert rel_err(ye, y0) < 1e-5
    # the fused FP32 plan: precomputed coefficients, fused restriction / prolongation / combine;
    # its output is zero off the fluid cells (the solver reads z there as zero)
    fluid = scene.flags == 2
    yref = np.where(scene.image()[1] == 0, 0.0, y0)
    z = m.precond_plan(img, storage=torch.float32).apply(b0.reshape(-1)).cpu().numpy().reshape(scene.shape)
    assert rel_err(z, yref) < 1e-5
    # BF16 coefficients and activations (FP32 accumulation): the stated bound of the fast form
    zb = m.precond_plan(img, storage=torch.bfloat16).apply(b0.reshape(-1)).cpu().numpy().reshape(scene.shape)
    err = rel_err(zb[fluid], y0[fluid])
    assert err < 2e-2, err


@pytest.mark.parametrize("name", ["npsd", "npcg", "npcg_flex"])
def test_config0_dropin_histories_50_iterations(golden, cuda, name):
    from mlpcg_gb300 import cg
    d, scene, m, flags, A, img, b = _setup(golden, cuda)
    hist = []
    pred = cg.model_predict(m, img, A.fluid_cells)
    x, it, _, res = getattr(cg, name)(b, A, torch.zeros_like(b), pred, 50, tol=1e-6, atol=1e-20,
                                      callback=lambda nrm, t: hist.append(nrm))
    ref = d[f"{name}_hist"][:51]
    assert len(hist) == 51
    assert np.all(ref > 1e-3)  # the prefix rule: the whole compared prefix is above 1e-3
    np.testing.assert_allclose(np.array(hist), ref, rtol=1e-4, err_msg=name)


@pytest.mark.parametrize("method", ["npsd", "npcg"])
def test_config0_fused_fp32_histories_50_iterations(golden, cuda, method):
    """The graph-captured solver with the FP32 plan against the reference's own history (not the
    drop-in's): FP32 CG vectors, FP64 reductions and a double-float iterate."""
    from mlpcg_gb300.solver import FusedSolver
    d, scene, m, flags, A, img, b = _setup(golden, cuda)
    solver = FusedSolver(m, flags, method=method, max_it=50, tol=1e-6, storage=torch.float32, image=img)
    out = solver.solve(torch.as_tensor(scene.rhs, device=cuda))
    assert out.status == "max_it" and out.iterations == 50
    np.testing.assert_allclose(out.history, d[f"{method}_hist"][:51], rtol=1e-4, err_msg=method)
