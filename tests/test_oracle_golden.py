"""The CPU oracle against fixtures recorded from the reference's own code (CPU only)."""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import cg as ocg
from oracle import laplacian as olap
from oracle import model as omodel
from oracle import ops

OPS = ["ops_8x8x8.npz", "ops_6x4x10.npz", "ops_16x16x16.npz"]
TOL = 1e-12  # FP64 vs FP64


@pytest.mark.parametrize("name", OPS)
def test_block_forward_and_transpose(golden, name):
    d = golden(name)
    x = d["x"][:, 0]
    assert rel_err(ops.sm_block(d["image"], x, d["W"], d["b"]), d["y"][:, 0]) < TOL
    assert rel_err(ops.sm_block(d["image"], x, d["W"], d["b"], transpose=True), d["yt"][:, 0]) < TOL


@pytest.mark.parametrize("name", OPS)
def test_block_gradients(golden, name):
    d = golden(name)
    x, g = d["x"][:, 0], d["g"][:, 0]
    gx, gw, gb, gi = ops.block_backward(g, d["image"], x, d["W"], d["b"])
    assert rel_err(gx, d["dx"][:, 0]) < TOL
    assert rel_err(gw, d["dW"]) < TOL
    assert rel_err(gb, d["db"]) < TOL
    assert rel_err(gi, d["dimg"]) < TOL
    gx, gw, gb, gi = ops.block_backward(g, d["image"], x, d["W"], d["b"], transpose=True)
    assert rel_err(gx, d["dxt"][:, 0]) < TOL
    assert rel_err(gw, d["dWt"]) < TOL
    assert rel_err(gb, d["dbt"]) < TOL
    assert rel_err(gi, d["dimgt"]) < TOL


@pytest.mark.parametrize("name", OPS)
def test_linear_and_transfer(golden, name):
    d = golden(name)
    z, y = ops.sm_linear(d["image"], d["Wl"], d["bl"])
    assert rel_err(z, d["z"]) < TOL
    assert rel_err(y, d["ylin"]) < TOL
    shape = d["image"].shape[1:]
    assert rel_err(ops.linear_image_grad([1.0], d["Wl"], shape), d["dimg_lin"]) < TOL
    if "pool" in d:
        assert rel_err(ops.avg_pool2(d["x"]), d["pool"]) < TOL
    assert rel_err(ops.upsample2(d["x"]), d["up"]) < 1e-7  # torch CPU computes the weights in fp32


def _params(d):
    return {k[len("param:"):]: v for k, v in d.items() if k.startswith("param:")}


def test_model_forward(golden):
    d = golden("model_16_l3.npz")
    p = _params(d)
    n = int(d["n"])
    y = omodel.forward(p, d["image"], d["b"][:, 0], n)
    assert rel_err(y, d["y"][:, 0]) < 1e-5  # reference ran in fp32
    ye = omodel.forward(p, d["image"], d["b"][:1, 0], n)
    assert rel_err(ye, d["y_eval"][:, 0]) < 1e-5


def test_init_order_and_keys(golden):
    """Our module tree draws the reference's initial weights under the same seed."""
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D
    for n in (4, 5):
        ref = golden(f"init_l{n}_seed0.npz")
        torch.manual_seed(0)
        m = SmallSMModelDn3D(n, 3, "trilinear")
        sd = m.state_dict()
        assert sorted(sd) == sorted(ref)
        for k, v in sd.items():
            assert tuple(v.shape) == ref[k].shape, k
            np.testing.assert_array_equal(v.numpy(), ref[k])
    assert omodel.param_names(2)[:3] == ["pre.1", "pre.0", "post.1"]


def _reference_fluid_block(d):
    """The reference's compressed matrix restricted to its FLUID rows / columns.

    lap_with_bc (lib/discrete_laplacian.py:148-155) lowers the diagonal of every
    neighbour of a solid cell after zeroing the boundary rows, so boundary cells
    next to a sphere keep a lone negative diagonal and survive compressedMat as
    extra rows.  They are decoupled from the fluid system (checked here) and
    have no right-hand side entry (compressedVec keeps fluid cells only).
    """
    import scipy.sparse as sp
    n = len(d["indptr"]) - 1
    A = sp.csr_matrix((d["data"], d["indices"], d["indptr"]), shape=(n, n))
    kept = d["kept_cells"]
    is_fluid = d["flags"].ravel()[kept] == olap.FLUID
    extra = np.flatnonzero(~is_fluid)
    if extra.size:
        E = A[extra]
        assert np.all(E.indices == extra[np.repeat(np.arange(extra.size), np.diff(E.indptr))])
    sel = np.flatnonzero(is_fluid)
    Af = A[sel][:, sel].tocsr()
    Af.sort_indices()
    return Af


def test_laplacian_assembly(golden):
    d = golden("laplacian_12.npz")
    A, fluid = olap.assemble(d["flags"])
    R = _reference_fluid_block(d)
    assert A.shape == R.shape
    np.testing.assert_array_equal(A.indptr, R.indptr)
    np.testing.assert_array_equal(A.indices, R.indices)
    np.testing.assert_array_equal(A.data, R.data)
    from mlpcg_gb300.scenes import flags_to_image
    np.testing.assert_array_equal(flags_to_image(d["flags"]), d["image"])


def test_product_csr_builder_matches_reference(golden):
    from mlpcg_gb300.laplacian import csr_from_flags
    d = golden("laplacian_12.npz")
    A, fluid = csr_from_flags(d["flags"], device="cpu")
    R = _reference_fluid_block(d)
    np.testing.assert_array_equal(A.crow_indices().numpy(), R.indptr)
    np.testing.assert_array_equal(A.col_indices().numpy(), R.indices)
    np.testing.assert_array_equal(A.values().numpy(), R.data)


def test_cg_histories(golden):
    """npsd / npcg / npcg_flex restated vs the reference's cg_tests.py run (50 its)."""
    d = golden("cg_16_l3.npz")
    m = golden("model_16_l3.npz")
    p = _params(m)
    n = int(m["n"])
    flags = d["flags"]
    A, fluid = olap.assemble(flags)
    img = m["image"]
    pred = ocg.make_predict(lambda g: omodel.forward(p, img, g, n), fluid, flags.shape)
    b = d["rhs"].ravel()[fluid]
    for name, fn in (("npsd", ocg.npsd), ("npcg", ocg.npcg), ("npcg_flex", ocg.npcg_flex)):
        x, it, hist = fn(b, A, np.zeros_like(b), pred, 50, tol=1e-6, atol=1e-20)
        ref = d[f"{name}_hist"]
        k = min(len(hist), len(ref))
        h, r = np.array(hist[:k]), ref[:k]
        ok = np.isfinite(r) & (r < 1e3)
        np.testing.assert_allclose(h[ok], r[ok], rtol=1e-4)   # every iteration, up to 50
        assert it == int(d[f"{name}_iters"]) or name == "npcg_flex"


def test_cg_histories_near_identity_50(golden):
    """The oracle's solvers against the reference's over 50 iterations with the near-identity
    network (the fixture also pins the plain GPU path)."""
    d = golden("cg_16_l3_near_identity.npz")
    p = _params(d)
    n = int(d["n"])
    flags = d["flags"]
    A, fluid = olap.assemble(flags)
    pred = ocg.make_predict(lambda g: omodel.forward(p, d["image"], g, n), fluid, flags.shape)
    b = d["rhs"].ravel()[fluid]
    for name, fn in (("npsd", ocg.npsd), ("npcg", ocg.npcg), ("npcg_flex", ocg.npcg_flex)):
        x, it, hist = fn(b, A, np.zeros_like(b), pred, 50, tol=1e-6, atol=1e-20)
        np.testing.assert_allclose(np.array(hist), d[f"{name}_hist"], rtol=1e-4, err_msg=name)


def test_fp64_cg_oracle_converges():
    from mlpcg_gb300.scenes import make_scene
    s = make_scene(12, 4)
    A, fluid = olap.assemble(s.flags)
    b = s.rhs.ravel()[fluid]
    x, it = olap.cg_fp64(A, b, tol=1e-12)
    assert np.linalg.norm(b - A @ x) <= 1e-12 * np.linalg.norm(b) * 1.0001


def test_residual_loss_restated(golden):
    """The reference's residual_loss (loss_functions.py:18-23) with the oracle's matrix: the mean and
    the sum over the batch of ||y - A x|| equal the reference's on its fixture."""
    d = golden("residual_loss_16.npz")
    A, fluid = olap.assemble(d["flags"])
    r = d["y"] - (A @ d["x"].T).T
    norms = np.linalg.norm(r, axis=1)
    assert norms.mean() == pytest.approx(float(d["loss_mean"]), rel=1e-12)
    assert norms.sum() == pytest.approx(float(d["loss_sum"]), rel=1e-12)
