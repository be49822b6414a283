"""The reference's CPU path in torch-CPU (oracle; test infrastructure and the timed CPU baseline only).

Blocks follow SmallSMBlock3DPY (sm_model_3d_py.py:10-22): the 27
coefficients are a Conv3d(3 -> 27, k=3, padding 1) of the image, applied to
the 27 shifted copies of x (unfold).  They are composed in the order of
SmallSMModelDn3D.forward (sm_model_3d.py:264-287) with trilinear upsampling
and the linear blocks of SmallLinearBlock3DPY (sm_model_3d_py.py:24-31) in
their mean-weight form (CPUSPDModel / CPUSPDFullModel: SmallSPDSMModelDn3D / SPDSMModelDn3D on the
same blocks).  The solver is npsd (cg_tests.py:189-284) with an FP64
torch CSR matrix and model_predict (test.py:42-51), all on the CPU.
"""
from __future__ import annotations

import time

import numpy as np
import torch
import torch.nn.functional as F


class CPUModel:
    def __init__(self, state_dict, n):
        self.n = n
        self.p = {k: v.detach().cpu().float() for k, v in state_dict.items()}
        self.cache = None

    def _block(self, name, img, x):
        W, b = self.p[f"{name}.weight"], self.p[f"{name}.bias"]
        K = F.conv3d(img[None], W, b, padding=1)[0]          # (27, N1, N2, N3)
        K = K.permute(1, 2, 3, 0).unflatten(3, (3, 3, 3))
        xp = F.pad(x, (1, 1, 1, 1, 1, 1))
        xu = xp.unfold(2, 3, 1).unfold(3, 3, 1).unfold(4, 3, 1)
        return (xu * K).sum(dim=(-3, -2, -1))

    def _linear(self, name, img):
        W, b = self.p[f"{name}.weight"], self.p[f"{name}.bias"]
        return F.conv3d(img[None], W, b, padding=1).mean()

    def __call__(self, img, b):
        n = self.n
        if self.cache is None:
            imgs = [img]
            for _ in range(n):
                imgs.append(F.avg_pool3d(imgs[-1][None], 2)[0])
            c0 = [self._linear(f"c0.{i}", imgs[i]) for i in range(n)]
            c1 = [self._linear(f"c1.{i}", imgs[i]) for i in range(n)]
            self.cache = (imgs, c0, c1)
        imgs, c0, c1 = self.cache
        x = [self._block("pre.0", imgs[0], b)]
        for i in range(1, n):
            x.append(F.avg_pool3d(x[-1], 2))
            x[-1] = self._block(f"pre.{i}", imgs[i], x[-1])
        x.append(F.avg_pool3d(x[-1], 2))
        x[-1] = self._block("l", imgs[n], x[-1])
        for i in range(n, 0, -1):
            x[i] = F.interpolate(x[i], scale_factor=2, mode="trilinear")
            x[i] = self._block(f"post.{i-1}", imgs[i - 1], x[i])
            x[i - 1] = c0[i - 1] * x[i - 1] + c1[i - 1] * x[i]
        return x[0]


class CPUSPDModel(CPUModel):
    """SmallSPDSMModelDn3D (sm_model_3d.py:425-444) on the same torch-CPU blocks: the transposed
    block l_t / l0_t scatters K_p(q) x(q) to q + offset(p) (the adjoint of the unfold), the
    prolongation is nearest x2 / 8, the combine uses c0^2, c1^2."""

    def _block_t(self, name, img, x):
        W, b = self.p[f"{name}.weight"], self.p[f"{name}.bias"]
        K = F.conv3d(img[None], W, b, padding=1)[0]          # (27, N1, N2, N3)
        n1, n2, n3 = x.shape[-3:]
        y = torch.zeros(x.shape[:-3] + (n1 + 2, n2 + 2, n3 + 2), dtype=x.dtype)
        for p in range(27):
            dx, dy, dz = p // 9, (p // 3) % 3, p % 3
            y[..., dx:dx + n1, dy:dy + n2, dz:dz + n3] += K[p] * x
        return y[..., 1:-1, 1:-1, 1:-1]

    def __call__(self, img, b):
        n = self.n
        if self.cache is None:
            imgs = [img]
            for _ in range(n):
                imgs.append(F.avg_pool3d(imgs[-1][None], 2)[0])
            c0 = [self._linear(f"c0.{i}", imgs[i]) for i in range(n)]
            c1 = [self._linear(f"c1.{i}", imgs[i]) for i in range(n)]
            self.cache = (imgs, c0, c1)
        imgs, c0, c1 = self.cache
        x = [self._block("l0.0", imgs[0], b)]
        for i in range(1, n):
            x.append(self._block(f"l0.{i}", imgs[i], F.avg_pool3d(x[-1], 2)))
        x.append(self._block("l", imgs[n], F.avg_pool3d(x[-1], 2)))
        x[-1] = self._block_t("l", imgs[n], x[-1])
        for i in range(n, 0, -1):
            x[i] = F.interpolate(x[i], scale_factor=2) / 8
            x[i - 1] = c0[i - 1] ** 2 * x[i - 1] + c1[i - 1] ** 2 * x[i]
            x[i - 1] = self._block_t(f"l0.{i-1}", imgs[i - 1], x[i - 1])
        return x[0]


class CPUSPDFullModel(CPUSPDModel):
    """SPDSMModelDn3D (sm_model_3d.py:313-347) on the same torch-CPU blocks: the V-cycle with l0,
    l, l1 and then its transpose with l1_t, l_t, l0_t."""

    def __call__(self, img, b):
        n = self.n
        if self.cache is None:
            imgs = [img]
            for _ in range(n):
                imgs.append(F.avg_pool3d(imgs[-1][None], 2)[0])
            c0 = [self._linear(f"c0.{i}", imgs[i]) for i in range(n)]
            c1 = [self._linear(f"c1.{i}", imgs[i]) for i in range(n)]
            self.cache = (imgs, c0, c1)
        imgs, c0, c1 = self.cache
        x = [self._block("l0.0", imgs[0], b)]
        for i in range(1, n):
            x.append(self._block(f"l0.{i}", imgs[i], F.avg_pool3d(x[-1], 2)))
        x.append(self._block("l", imgs[n], F.avg_pool3d(x[-1], 2)))
        for i in range(n, 0, -1):
            x[i] = self._block(f"l1.{i-1}", imgs[i - 1], F.interpolate(x[i], scale_factor=2) / 8)
            x[i - 1] = c0[i - 1] * x[i - 1] + c1[i - 1] * x[i]
        x = [x[0]]
        for i in range(n):
            x.append(F.avg_pool3d(self._block_t(f"l1.{i}", imgs[i], x[i]), 2))
        x[-1] = self._block_t("l", imgs[n], x[-1])
        for i in range(n - 1, -1, -1):
            x[i] = c0[i] * x[i] + c1[i] * (F.interpolate(x[i + 1], scale_factor=2) / 8)
            x[i] = self._block_t(f"l0.{i}", imgs[i], x[i])
        return x[0]


def csr_cpu(flags):
    from .laplacian import assemble
    A, fluid = assemble(flags)
    At = torch.sparse_csr_tensor(torch.from_numpy(A.indptr.astype(np.int64)),
                                 torch.from_numpy(A.indices.astype(np.int64)),
                                 torch.from_numpy(A.data), A.shape, dtype=torch.float64)
    return At, torch.from_numpy(fluid)


def npcg_iterations(model: CPUModel, img, flags, rhs, iters, tol=None):
    """Up to ``iters`` iterations of npcg (cg_tests.py:26-101: textbook PCG, the solver of a
    symmetric network) on the CPU, stopping once the relative residual is at most ``tol`` (the
    reference's rule with atol = 1e-20; None: run all ``iters``); returns (seconds per iteration
    list, rel residuals)."""
    A, fluid = csr_cpu(flags)
    shape = tuple(flags.shape)
    n = int(np.prod(shape))
    b = torch.from_numpy(rhs.ravel()[fluid.numpy()]).double()
    img_t = torch.as_tensor(img)

    def predict(r):
        r32 = F.normalize(r.float(), dim=0)
        g = torch.zeros(n, dtype=torch.float32)
        g[fluid] = r32
        return model(img_t, g.view((1, 1) + shape)).flatten().double()[fluid]

    norm_b = b.norm().item()
    x = torch.zeros_like(b)
    r = b - A @ x
    times, hist = [], []
    p = rz = None
    for _ in range(iters):
        t0 = time.perf_counter()
        z = predict(r)
        rz_new = r.dot(z)
        p = z if p is None else z + (rz_new / rz) * p
        rz = rz_new
        Ap = A @ p
        alpha = rz / p.dot(Ap)
        x = x + alpha * p
        r = b - A @ x
        hist.append(r.norm().item() / norm_b)
        times.append(time.perf_counter() - t0)
        if tol is not None and not hist[-1] > max(tol, 1e-20 / norm_b):
            break
    return times, hist


def npsd_iterations(model: CPUModel, img, flags, rhs, iters, tol=None):
    """Up to ``iters`` iterations of npsd (cg_tests.py:189-284) on the CPU, stopping once the
    relative residual is below ``tol`` (the reference's rule with atol = 1e-20, test.py:328; None:
    run all ``iters``); returns (seconds per iteration list, rel residuals)."""
    A, fluid = csr_cpu(flags)
    shape = tuple(flags.shape)
    n = int(np.prod(shape))
    b = torch.from_numpy(rhs.ravel()[fluid.numpy()]).double()
    img_t = torch.as_tensor(img)

    def predict(r):
        r32 = F.normalize(r.float(), dim=0)
        g = torch.zeros(n, dtype=torch.float32)
        g[fluid] = r32
        return model(img_t, g.view((1, 1) + shape)).flatten().double()[fluid]

    norm_b = b.norm().item()
    x = torch.zeros_like(b)
    r = b - A @ x
    p, Ap, alfa = [], [], []
    times, hist = [], []
    for i in range(1, iters + 1):
        t0 = time.perf_counter()
        q = predict(r)
        if i > 2:
            for j in (1, 0):
                q = q - q.dot(Ap[j]) / alfa[j] * p[j]
            p[0], Ap[0], alfa[0] = p[1], Ap[1], alfa[1]
            p[1] = q
            Ap[1] = A @ q
            alfa[1] = p[1].dot(Ap[1])
        else:
            for j in reversed(range(i - 1)):
                q = q - q.dot(Ap[j]) / alfa[j] * p[j]
            p.append(q)
            Ap.append(A @ q)
            alfa.append(p[-1].dot(Ap[-1]))
        beta = p[-1].dot(r) / alfa[-1]
        x = x + q * beta
        r = b - A @ x
        hist.append(r.norm().item() / norm_b)
        times.append(time.perf_counter() - t0)
        if tol is not None and hist[-1] < max(tol, 1e-20 / norm_b):
            break
    return times, hist
