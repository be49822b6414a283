"""Generates the golden fixtures of tests/golden/ from the reference itself.

Run in a container that has the reference checkout (its Python CPU path needs
only torch, numpy and scipy):

    python tests/golden/make_golden.py /path/to/MLPCG

What it imports from the reference, unmodified:

* sm_model_3d_py.py -- SmallSMBlock3DPY (Conv3d + unfold) and SmallLinearBlock3DPY,
  the reference's own CPU statement of the block and linear ops;
* sm_model_3d.py    -- SmallSMModelDn3D, SPDSMModelDn3D, SmallSPDSMModelDn3D and
  their autograd Functions; its JIT
  extension modules (CUDA, cannot run here) are replaced by thin adapters that
  evaluate the ops with the SmallSMBlock3DPY / SmallLinearBlock3DPY math, so
  the reference's own module tree, initialisation order and orchestration
  (forward / eval_forward) run on the CPU;
* model.py          -- BaseModel.reset_parameters;
* lib/discrete_laplacian.py, lib/read_data.py, lib/write_data.py -- lap_with_bc,
  compressedMat, convert_to_binary_images, the file readers and writers;
* cg_tests.py       -- npcg, npcg_flex, npsd (cupy / AMGCL imports stubbed,
  torch.cuda.synchronize made a no-op).

Outputs (FP64 unless noted): ops_*.npz, model_*.npz, spd_*.npz / small_spd_*.npz (fp32) with\ntheir cg_spd_* / cg_small_spd_* solver histories,
laplacian_*.npz, cg_*.npz, and
scene_8/ (simulator-format files) with scene_files_8.npz (what the reference reads from them).
The scenes come from mlpcg_gb300.scenes (seeded), stored in the fixtures.
"""
from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np
import torch
import torch.nn.functional as F

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

from mlpcg_gb300.scenes import make_scene  # noqa: E402


def _import_reference(ref: Path):
    sys.path.insert(0, str(ref))
    sys.path.insert(0, str(ref / "lib"))
    # sm_model_3d.py JIT-builds CUDA extensions at import; the adapters below replace them.
    import torch.utils.cpp_extension as ce
    real_load = ce.load
    ce.load = lambda *a, **k: types.SimpleNamespace()
    try:
        import sm_model_3d as ref_model
    finally:
        ce.load = real_load
    import sm_model_3d_py as ref_py
    import discrete_laplacian as ref_lap
    import read_data as ref_read
    # cg_tests.py imports cupy and the AMGCL/IC builds at module level
    for name in ("cupy", "cupyx", "cupyx.scipy", "cupyx.scipy.sparse", "cupyx.scipy.sparse.linalg",
                 "cxx_src", "cxx_src.build"):
        sys.modules.setdefault(name, types.ModuleType(name))
    b = sys.modules["cxx_src.build"]
    for n in ("pyamgcl", "pyamgcl_cuda", "pyamgcl_vexcl", "pyic", "pyic_cuda", "pyic_vexcl"):
        setattr(b, n, None)
    torch.cuda.synchronize = lambda *a, **k: None
    import cg_tests as ref_cg
    return ref_model, ref_py, ref_lap, ref_read, ref_cg


class _BlockAdapter:
    """smblock3d / smblocktrans3d interface evaluated with SmallSMBlock3DPY."""

    def __init__(self, ref_py, transpose):
        self.ref_py = ref_py
        self.t = transpose

    def _blk(self, W, b):
        blk = self.ref_py.SmallSMBlock3DPY(3).to(W.dtype)
        with torch.no_grad():
            blk.KL.weight.copy_(W)
            blk.KL.bias.copy_(b)
        return blk

    def _fwd(self, image_p, x_p, W, b):
        image = image_p[:, 1:-1, 1:-1, 1:-1]
        x = x_p[..., 1:-1, 1:-1, 1:-1]
        blk = self._blk(W, b)
        if not self.t:
            with torch.no_grad():
                return blk(image, x)
        xx = torch.zeros_like(x, requires_grad=True)
        with torch.enable_grad():
            out = blk(image, xx)
            (gx,) = torch.autograd.grad(out, xx, grad_outputs=x)
        return gx.detach()

    def inference(self, image_p, x_p, W, b):
        return [self._fwd(image_p, x_p, W, b)]

    forward = inference


class _LinearAdapter:
    """smlinear3d interface evaluated with SmallLinearBlock3DPY."""

    def __init__(self, ref_py):
        self.ref_py = ref_py

    def inference(self, image, W, b):
        blk = self.ref_py.SmallLinearBlock3DPY(3).to(W.dtype)
        with torch.no_grad():
            blk.KL.weight.copy_(W.reshape(1, 3, 3, 3, 3).expand(27, 3, 3, 3, 3))
            blk.KL.bias.copy_(b.reshape(1).expand(27))
            z = blk(image).reshape(1)
            eye = torch.eye(81, dtype=image.dtype).reshape(81, 3, 3, 3, 3)
            y = F.conv3d(image[None], eye, padding=1).mean(dim=(2, 3, 4)).reshape(1, 3, 3, 3, 3)
        return [z, y]

    forward = inference


def _py_block(ref_py, W, b, dtype):
    blk = ref_py.SmallSMBlock3DPY(3).to(dtype)
    with torch.no_grad():
        blk.KL.weight.copy_(W)
        blk.KL.bias.copy_(b)
    return blk


def make_ops(ref_py, shape, seed, B=2):
    torch.manual_seed(seed)
    dt = torch.float64
    image = torch.rand(3, *shape, dtype=dt)
    x = torch.rand(B, 1, *shape, dtype=dt)
    g = torch.rand(B, 1, *shape, dtype=dt)
    blk0 = ref_py.SmallSMBlock3DPY(3)
    W = blk0.KL.weight.detach().to(dt).clone()
    b = blk0.KL.bias.detach().to(dt).clone()
    out = dict(image=image.numpy(), x=x.numpy(), g=g.numpy(), W=W.numpy(), b=b.numpy())
    # forward block, its gradients (autograd through the reference's Conv3d + unfold)
    blk = _py_block(ref_py, W, b, dt)
    xx = x.clone().requires_grad_(True)
    img = image.clone().requires_grad_(True)
    y = blk(img, xx)
    y.backward(g)
    out.update(y=y.detach().numpy(), dx=xx.grad.numpy(), dW=blk.KL.weight.grad.numpy(),
               db=blk.KL.bias.grad.numpy(), dimg=img.grad.numpy())
    # transposed block: y_t = B^T x as a vector-Jacobian product of the forward block
    blk = _py_block(ref_py, W, b, dt)
    img = image.clone().requires_grad_(True)
    v = torch.zeros_like(x, requires_grad=True)
    with torch.enable_grad():
        yv = blk(img, v)
        (yt,) = torch.autograd.grad(yv, v, grad_outputs=x, create_graph=True)
    out["yt"] = yt.detach().numpy()
    blk.zero_grad()
    yt.backward(g)
    out.update(dxt=None if v.grad is None else v.grad.numpy())
    out["dWt"] = blk.KL.weight.grad.numpy()
    out["dbt"] = blk.KL.bias.grad.numpy()
    out["dimgt"] = img.grad.numpy()
    # B applied to g equals the gradient of <g, B^T x> w.r.t. x
    with torch.no_grad():
        out["dxt"] = blk(image, g).numpy()
    # linear block (mean-weight form of SmallLinearBlock3DNew)
    lin = ref_py.SmallLinearBlock3DPY(3).to(dt)
    Wl = lin.KL.weight.detach().mean(0, keepdim=True)
    bl = lin.KL.bias.detach().mean(0, keepdim=True)
    img = image.clone().requires_grad_(True)
    z = lin(img)
    z.backward()
    eye = torch.eye(81, dtype=dt).reshape(81, 3, 3, 3, 3)
    ymean = F.conv3d(image[None], eye, padding=1).mean(dim=(2, 3, 4)).reshape(1, 3, 3, 3, 3)
    out.update(Wl=Wl.numpy(), bl=bl.numpy(), z=np.array([z.item()]), ylin=ymean.numpy(),
               dimg_lin=img.grad.numpy())
    # pooling / interpolation (torch CPU = ATen reference semantics)
    if all(s % 2 == 0 for s in shape):
        out["pool"] = F.avg_pool3d(x, (2, 2, 2)).numpy()
    out["up"] = F.interpolate(x, scale_factor=2, mode="trilinear").numpy()
    return out


def make_model(ref_model, ref_py, shape, n, seed_scene, seed_init=0):
    ref_model.smblock3d = _BlockAdapter(ref_py, False)
    ref_model.smblocktrans3d = _BlockAdapter(ref_py, True)
    ref_model.smlinear3d = _LinearAdapter(ref_py)
    torch.manual_seed(seed_init)
    model = ref_model.SmallSMModelDn3D(n, 3, "trilinear")
    sd = {k: v.detach().numpy().copy() for k, v in model.state_dict().items()}
    scene = make_scene(shape, seed_scene)
    image = torch.from_numpy(scene.image())
    torch.manual_seed(1234)
    b = torch.rand(2, 1, *shape)
    with torch.no_grad():
        y = model(image, b)
        from global_clock import GlobalClock
        ye = model.eval_forward(image, b[:1], GlobalClock(), [], [], [])
    out = {"flags": scene.flags, "image": scene.image(), "b": b.numpy(), "y": y.numpy(), "y_eval": ye.numpy(),
           "n": np.array(n)}
    out.update({"param:" + k: v for k, v in sd.items()})
    return out, model, scene


def make_spd(ref_model, ref_py, cls_name, shape, n, seed_scene, seed_init=0):
    """The reference's SPD preconditioners (SPDSMModelDn3D / SmallSPDSMModelDn3D) under the
    adapters: state dict under ``torch.manual_seed(seed_init)``, forward on a batch of two and
    eval_forward on one right-hand side."""
    ref_model.smblock3d = _BlockAdapter(ref_py, False)
    ref_model.smblocktrans3d = _BlockAdapter(ref_py, True)
    ref_model.smlinear3d = _LinearAdapter(ref_py)
    torch.manual_seed(seed_init)
    model = getattr(ref_model, cls_name)(n)
    sd = {k: v.detach().numpy().copy() for k, v in model.state_dict().items()}
    scene = make_scene(shape, seed_scene)
    image = torch.from_numpy(scene.image())
    torch.manual_seed(4321)
    b = torch.rand(2, 1, *shape)
    with torch.no_grad():
        y = model(image, b)
        ye = model.eval_forward(image, b[:1])
    out = {"flags": scene.flags, "image": scene.image(), "b": b.numpy(), "y": y.numpy(), "y_eval": ye.numpy(),
           "n": np.array(n)}
    out.update({"param:" + k: v for k, v in sd.items()})
    return out, model, scene


def make_laplacian(ref_lap, ref_read, shape, seed):
    scene = make_scene(shape, seed)
    f = scene.flags
    n = f.shape[0]
    idx = lambda code: [tuple(int(c) for c in t) for t in np.argwhere(f == code)]
    A_full = ref_lap.lap_with_bc(n, 3, solid=idx(1), air=idx(3), bd=idx(0), bd_padding=True, dtype=np.float64)
    # the flat cell index of every row compressedMat keeps (rows with stored entries)
    kept = np.flatnonzero(A_full.tocsr().getnnz(1) > 0)
    A = ref_read.compressedMat(A_full, f)
    A = A.tocsr()
    A.sort_indices()
    img = ref_read.convert_to_binary_images(f, 3)
    return {"flags": f, "indptr": A.indptr, "indices": A.indices, "data": A.data, "kept_cells": kept,
            "image": img.astype(np.float32), "rhs": scene.rhs}


def make_cg(ref_cg, model, scene, max_it=50):
    import scipy.sparse as sp
    lap = sys.modules["discrete_laplacian"]
    rd = sys.modules["read_data"]
    f = scene.flags
    n = f.shape[0]
    idx = lambda code: [tuple(int(c) for c in t) for t in np.argwhere(f == code)]
    A = lap.lap_with_bc(n, 3, solid=idx(1), air=idx(3), bd=idx(0), bd_padding=True, dtype=np.float64)
    A = rd.compressedMat(A, f).tocsr()
    A.sort_indices()
    assert A.shape[0] == int((f == 2).sum()), "scene must have no sphere touching the wall layer"
    At = torch.sparse_csr_tensor(A.indptr, A.indices, A.data, A.shape, dtype=torch.float64)
    fluid = torch.from_numpy(np.flatnonzero(f.ravel() == 2))
    rhs = torch.from_numpy(scene.rhs.ravel()[fluid.numpy()]).double()
    image = torch.from_numpy(scene.image())
    shape = tuple(f.shape)

    def predict(r, timer, imgs=[], c0=[], c1=[]):  # test.py:42-51 restated (test.py cannot be imported)
        with torch.no_grad():
            r = F.normalize(r.to(torch.float32), dim=0)
            bb = torch.zeros(int(np.prod(shape)), dtype=torch.float32)
            bb[fluid] = r
            x = model.eval_forward(image, bb.view((1, 1) + shape), timer, imgs, c0, c1).flatten().double()
        return x[fluid]

    out = {"flags": f, "rhs": scene.rhs}
    for name in ("npsd", "npcg", "npcg_flex"):
        hist = []
        solver = getattr(ref_cg, name)
        pred = predict if name == "npsd" else (lambda r, timer, _p=predict, _c=([], [], []): _p(r, timer, *_c))
        x, iters, _, res = solver(rhs, At, torch.zeros_like(rhs), pred, max_it, tol=1e-6, atol=1e-20,
                                  callback=lambda nrm, t: hist.append(nrm))
        out[f"{name}_hist"] = np.array(hist)
        out[f"{name}_iters"] = np.array(iters)
        out[f"{name}_x"] = x.numpy()
    return out


def _fluid_matrix(f, use_reference_assembly):
    """The compressed FP64 matrix of flags f: the reference's lap_with_bc + compressedMat, or, where
    their LIL assembly cannot run (at 64^3 it grew past 48 GB of host memory before it was stopped),
    the oracle's assembly, which is pinned entry for entry to the reference's at 12^3
    (laplacian_12.npz) and evaluates the same formula."""
    if use_reference_assembly:
        lap = sys.modules["discrete_laplacian"]
        rd = sys.modules["read_data"]
        n = f.shape[0]
        idx = lambda code: [tuple(int(c) for c in t) for t in np.argwhere(f == code)]
        A = lap.lap_with_bc(n, 3, solid=idx(1), air=idx(3), bd=idx(0), bd_padding=True, dtype=np.float64)
        A = rd.compressedMat(A, f).tocsr()
    else:
        from oracle.laplacian import assemble
        A, _ = assemble(f)
    A.sort_indices()
    assert A.shape[0] == int((f == 2).sum()), "scene must have no sphere touching the wall layer"
    return A


def make_config_scene(ref_cg, ref_model, ref_py, size, seed, n, max_it=100, state=None, n_spheres=3,
                      use_reference_assembly=False):
    """A BASELINE-style scene solved by the reference: make_scene(size, seed) (one wall layer, a
    height-field fluid, n_spheres spheres), the reference's SmallSMModelDn3D(n, 3, 'trilinear') in
    FP32 -- drawn under torch.manual_seed(0) (random init), or given weights ``state`` -- and the
    reference's npsd / npcg / npcg_flex (cg_tests.py) with test.py's model_predict and its call
    (max_it 100, tol 1e-6, atol 1e-20).  Records the weights, the preconditioner output on the
    normalised right-hand side (what model_predict feeds the network first), each solver's residual
    history, iteration count and a few moments of its solution."""
    ref_model.smblock3d = _BlockAdapter(ref_py, False)
    ref_model.smblocktrans3d = _BlockAdapter(ref_py, True)
    ref_model.smlinear3d = _LinearAdapter(ref_py)
    torch.manual_seed(0)
    model = ref_model.SmallSMModelDn3D(n, 3, "trilinear")
    if state is not None:
        model.load_state_dict({k: torch.as_tensor(v, dtype=torch.float32) for k, v in state.items()})
    scene = make_scene(size, seed, n_spheres)
    f = scene.flags
    A = _fluid_matrix(f, use_reference_assembly)
    At = torch.sparse_csr_tensor(A.indptr, A.indices, A.data, A.shape, dtype=torch.float64)
    fluid = torch.from_numpy(np.flatnonzero(f.ravel() == 2))
    rhs = torch.from_numpy(scene.rhs.ravel()[fluid.numpy()]).double()
    image = torch.from_numpy(scene.image())
    shape = tuple(f.shape)
    from global_clock import GlobalClock

    def predict(r, timer, imgs=[], c0=[], c1=[]):  # test.py:42-51 restated (test.py cannot be imported)
        with torch.no_grad():
            r = F.normalize(r.to(torch.float32), dim=0)
            bb = torch.zeros(int(np.prod(shape)), dtype=torch.float32)
            bb[fluid] = r
            x = model.eval_forward(image, bb.view((1, 1) + shape), timer, imgs, c0, c1).flatten().double()
        return x[fluid]

    with torch.no_grad():
        r0 = F.normalize(rhs.to(torch.float32), dim=0)
        b0 = torch.zeros(int(np.prod(shape)), dtype=torch.float32)
        b0[fluid] = r0
        y0 = model.eval_forward(image, b0.view((1, 1) + shape), GlobalClock(), [], [], [])
    out = {"size": np.array(size), "seed": np.array(seed), "n": np.array(n), "spheres": np.array(n_spheres),
           "flags_sum": np.array(int(f.astype(np.int64).sum())), "rhs_norm": np.array(float(rhs.norm())),
           "max_it": np.array(max_it), "assembly": np.array("reference" if use_reference_assembly else "oracle")}
    if size <= 64:
        out.update(b0=b0.numpy().reshape(shape), y0=y0.numpy().reshape(shape))
    else:
        # larger grids: the output at 65,536 cells drawn without replacement (the input b0 is the
        # normalised rhs, rebuilt from the scene), to keep the fixture small
        idx = np.sort(np.random.default_rng(7).choice(int(np.prod(shape)), 65536, replace=False))
        out.update(y0_index=idx.astype(np.int64), y0_sample=y0.numpy().reshape(-1)[idx],
                   y0_norm=np.array(float(y0.double().norm())))
    out.update({"param:" + k: v.detach().numpy().copy() for k, v in model.state_dict().items()})
    w = np.random.default_rng(99).standard_normal(fluid.numel())
    for name in ("npsd", "npcg", "npcg_flex"):
        hist = []
        solver = getattr(ref_cg, name)
        pred = predict if name == "npsd" else (lambda r, timer, _p=predict, _c=([], [], []): _p(r, timer, *_c))
        x, iters, _, res = solver(rhs, At, torch.zeros_like(rhs), pred, max_it, tol=1e-6, atol=1e-20,
                                  callback=lambda nrm, t: hist.append(nrm))
        xn = x.numpy()
        out[f"{name}_hist"] = np.array(hist)
        out[f"{name}_iters"] = np.array(iters)
        out[f"{name}_x_moments"] = np.array([np.linalg.norm(xn), float(xn @ w), float(xn.sum())])
        print(f"{size}^3 seed {seed}: {name} {iters} iterations, rel res {res:.3e}", flush=True)
    return out


def make_cg_near_identity(ref_cg, ref_model, ref_py, shape, n, seed_scene, max_it=50):
    """Solver histories over max_it iterations with the reference's SmallSMModelDn3D(n) drawn under
    torch.manual_seed(0) and moved near the identity (weights x 0.1, centre tap of pre[0] and the
    bias of c0[0] + 1), so that the residual falls steadily instead of stagnating."""
    ref_model.smblock3d = _BlockAdapter(ref_py, False)
    ref_model.smblocktrans3d = _BlockAdapter(ref_py, True)
    ref_model.smlinear3d = _LinearAdapter(ref_py)
    torch.manual_seed(0)
    model = ref_model.SmallSMModelDn3D(n, 3, "trilinear")
    with torch.no_grad():
        for p in model.parameters():
            p.mul_(0.1)
        model.pre[0].bias[13] += 1.0
        model.c0[0].bias[0] += 1.0
    scene = make_scene(shape, seed_scene)
    out = make_cg(ref_cg, model, scene, max_it=max_it)
    out.update({"param:" + k: v.detach().numpy().copy() for k, v in model.state_dict().items()})
    out.update(image=scene.image(), n=np.array(n))
    return out


def make_scene_files(ref_lap, ref_read, shape, seed, frame=1):
    """A small scene as the reference's simulator files: the matrix and the rhs written by the
    reference's own writers (lib/write_data.py), the flags in the C++ Serialize layout that
    lib/read_data.py documents (size_t count + int32); the expected arrays are what the
    reference's readers return for them."""
    import struct
    import write_data as ref_write
    scene = make_scene(shape, seed)
    f = scene.flags
    n = f.shape[0]
    idx = lambda code: [tuple(int(c) for c in t) for t in np.argwhere(f == code)]
    A_full = ref_lap.lap_with_bc(n, 3, solid=idx(1), air=idx(3), bd=idx(0), bd_padding=True, dtype=np.float64)
    d = HERE / f"scene_{n}"
    d.mkdir(exist_ok=True)
    with open(d / f"flags_{frame}.bin", "wb") as out:
        out.write(struct.pack("N", f.size))
        out.write(struct.pack(f"{f.size}i", *[int(v) for v in f.ravel()]))
    ref_write.writeA_sparse(A_full.tocsr(), str(d / f"A_{frame}.bin"))
    ref_write.write_bin_file_from_nparray(str(d / f"div_v_star_{frame}.bin"), scene.rhs.ravel().astype(np.float64))
    flags = ref_read.read_flags(str(d / f"flags_{frame}.bin"))
    A = ref_read.readA_sparse(str(d / f"A_{frame}.bin"))
    Ac = ref_read.compressedMat(A, flags).tocsr()
    Ac.sort_indices()
    rhs = ref_read.load_vector(str(d / f"div_v_star_{frame}.bin"))
    return {"flags": flags, "A_indptr": A.indptr, "A_indices": A.indices, "A_data": A.data,
            "Ac_indptr": Ac.indptr, "Ac_indices": Ac.indices, "Ac_data": Ac.data, "rhs": rhs,
            "rhs_fluid": ref_read.compressedVec(rhs, flags)}


def make_residual_loss(ref: Path, shape=(16, 16, 16), seed=3, B=4):
    """The reference's residual_loss (loss_functions.py:18-23: y - x A row by row, the mean and the
    sum of the norms) on FP64 batches over the fluid cells of a scene, with the reference's own
    matrix (lap_with_bc + compressedMat, as CSC)."""
    sys.path.insert(0, str(ref))
    import loss_functions as ref_loss
    scene = make_scene(shape, seed)
    f = scene.flags
    A = _fluid_matrix(f, True).tocsc()
    At = torch.sparse_csc_tensor(A.indptr, A.indices, A.data, A.shape, dtype=torch.float64)
    rng = np.random.default_rng(seed)
    x = torch.from_numpy(rng.standard_normal((B, A.shape[0])))
    y = torch.from_numpy(rng.standard_normal((B, A.shape[0])))
    return {"flags": f, "x": x.numpy(), "y": y.numpy(),
            "loss_mean": np.array(float(ref_loss.residual_loss(x, y, At))),
            "loss_sum": np.array(float(ref_loss.residual_loss(x, y, At, mean=False)))}


def main(ref_root: str, only: str | None = None):
    ref = Path(ref_root)
    ref_model, ref_py, ref_lap, ref_read, ref_cg = _import_reference(ref)
    if only == "scene_files":
        np.savez_compressed(HERE / "scene_files_8.npz", **make_scene_files(ref_lap, ref_read, (8, 8, 8), 4))
        print("scene files written to", HERE)
        return
    torch.set_default_dtype(torch.float32)
    if only == "residual_loss":
        np.savez_compressed(HERE / "residual_loss_16.npz", **make_residual_loss(ref))
        print("residual_loss fixture written to", HERE)
        return
    if only == "config0":
        # 64^3, seed 0, 3 spheres, 4 levels, random init from torch seed 0, FP32, max 100 iterations
        np.savez_compressed(HERE / "cg_64_l4_seed0.npz",
                            **make_config_scene(ref_cg, ref_model, ref_py, 64, 0, 4))
        print("64^3 scene fixture written to", HERE)
        return
    if only == "config1":
        # 128^3, seed 1, 3 spheres, 4 levels, the committed trained weights smallsm_l4.npz
        w = np.load(REPO / "mlpcg_gb300" / "weights" / "smallsm_l4.npz")
        np.savez_compressed(HERE / "cg_128_l4_seed1.npz",
                            **make_config_scene(ref_cg, ref_model, ref_py, 128, 1, 4, state=dict(w)))
        print("128^3 scene fixture written to", HERE)
        return
    spd = {"spd_16_l2.npz": ("SPDSMModelDn3D", 2), "small_spd_16_l3.npz": ("SmallSPDSMModelDn3D", 3)}
    for fname, (cls_name, n) in spd.items():
        out, model, scene = make_spd(ref_model, ref_py, cls_name, (16, 16, 16), n, seed_scene=6)
        np.savez_compressed(HERE / fname, **out)
        np.savez_compressed(HERE / ("cg_" + fname), **make_cg(ref_cg, model, scene))
    if only == "spd":
        print("SPD fixtures written to", HERE)
        return
    if only == "near_identity":
        np.savez_compressed(HERE / "cg_16_l3_near_identity.npz",
                            **make_cg_near_identity(ref_cg, ref_model, ref_py, (16, 16, 16), 3, seed_scene=3))
        print("near-identity solver fixture written to", HERE)
        return
    for shape, seed in (((8, 8, 8), 0), ((6, 4, 10), 1), ((16, 16, 16), 2)):
        out = make_ops(ref_py, shape, seed)
        out = {k: v for k, v in out.items() if v is not None}
        np.savez_compressed(HERE / f"ops_{'x'.join(map(str, shape))}.npz", **out)
    out, model, scene = make_model(ref_model, ref_py, (16, 16, 16), 3, seed_scene=3)
    np.savez_compressed(HERE / "model_16_l3.npz", **out)
    # initial weights of the 4-level and 5-level networks under torch.manual_seed(0)
    for n in (4, 5):
        torch.manual_seed(0)
        m = ref_model.SmallSMModelDn3D(n, 3, "trilinear")
        np.savez_compressed(HERE / f"init_l{n}_seed0.npz",
                            **{k: v.detach().numpy() for k, v in m.state_dict().items()})
    np.savez_compressed(HERE / "laplacian_12.npz", **make_laplacian(ref_lap, ref_read, (12, 12, 12), 5))
    np.savez_compressed(HERE / "cg_16_l3.npz", **make_cg(ref_cg, model, scene))
    np.savez_compressed(HERE / "cg_16_l3_near_identity.npz",
                        **make_cg_near_identity(ref_cg, ref_model, ref_py, (16, 16, 16), 3, seed_scene=3))
    np.savez_compressed(HERE / "scene_files_8.npz", **make_scene_files(ref_lap, ref_read, (8, 8, 8), 4))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    # python make_golden.py [reference root] [--only=scene_files | --only=spd | --only=near_identity |
    #                                          --only=config0 | --only=config1 | --only=residual_loss]
    args = [a for a in sys.argv[1:] if not a.startswith("--only")]
    only = next((a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--only=")), None)
    main(args[0] if args else "/root/reference", only)
