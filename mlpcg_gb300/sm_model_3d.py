"""Drop-in for the reference's sm_model_3d.py: autograd Functions, blocks,
SmallSMModelDn3D and the symmetric networks SPDSMModelDn3D / SmallSPDSMModelDn3D.

Class names, constructor signatures, forward / eval_forward signatures and
parameter names (state-dict keys) are those of the reference
(sm_model_3d.py:21-444), so reference checkpoints load unchanged
(``model.load_state_dict(torch.load(f)['model_state_dict'])``).  Every
numerical step runs in the sm_103a kernels of ``libmlpcg_gb300.so``:

* blocks evaluate their coefficients from the image and apply them
  (reference semantics: recomputed per call, FP32);
* avg-pool restriction, trilinear prolongation and the c0/c1 combine are
  library kernels, each with a hand-written adjoint for training;
* the image needs no F.pad copy: out-of-grid neighbours read as zero.

For the fast solve path (coefficients precomputed once per image, BF16
storage, fused level transfers) see ``precond.PrecondPlan``.
"""
from __future__ import annotations

import torch
import torch.nn as nn

from . import ops
from .model import BaseModel

# The reference's JIT extension modules (sm_model_3d.py:11-16).
smblock3d = ops.smblock3d
smblocktrans3d = ops.smblocktrans3d
smlinear3d = ops.smlinear3d


def _tstart(timer, name):
    if timer:
        timer.start(name)


def _tstop(timer, name):
    if timer:
        torch.cuda.synchronize()
        timer.stop(name)


######################
# SM block
######################
class SMBlockFunction3D(torch.autograd.Function):
    """y(q) = sum_p K_p(q) x(q + off_p), K = bias + Conv3d(3->27)(image) (sm_model_3d.py:21-48)."""

    @staticmethod
    def inference(image, x, weights, bias, timer=None):
        _tstart(timer, "Forward")
        y = ops.block_forward(image, x, weights, bias, transpose=False)
        _tstop(timer, "Forward")
        return y

    @staticmethod
    def forward(ctx, image, x, weights, bias):
        y = ops.block_forward(image, x, weights, bias, transpose=False)
        ctx.save_for_backward(image, x, weights, bias)
        return y

    @staticmethod
    def backward(ctx, grad_output):
        image, x, weights, bias = ctx.saved_tensors
        gx, gw, gb, gi = ops.block_backward(grad_output, image, x, weights, bias, transpose=False,
                                            image_grad=ctx.needs_input_grad[0])
        return gi, gx, gw, gb


class SMBlockBF16Function3D(torch.autograd.Function):
    """The block (or its transpose) for training with BF16 storage: the coefficient planes and the
    input saved for the backward pass in BF16, every sum accumulated in FP32, outputs and gradients
    in FP32.  Backward through the same adjoint kernels as SMBlockFunction3D: dx by the transposed
    application of the BF16 planes, dK from the FP32 output gradient and the saved input, dW / db
    and the image gradient from dK (sm_block_3d_kernel.cu:122-326)."""

    @staticmethod
    def forward(ctx, image, x, weights, bias, transpose):
        dims = tuple(image.shape[1:])
        K = ops.stencil_gen(image, weights, bias, dtype=torch.bfloat16)
        xb = x.contiguous().to(torch.bfloat16)
        y = ops.stencil_apply(K, xb, dims, transpose=transpose)
        ctx.save_for_backward(image, xb, weights, bias)
        ctx.transpose = transpose
        return y.reshape(x.shape)

    @staticmethod
    def backward(ctx, grad_output):
        image, xb, weights, bias = ctx.saved_tensors
        dims = tuple(image.shape[1:])
        g = grad_output.contiguous()
        K = ops.stencil_gen(image, weights, bias, dtype=torch.bfloat16)
        gx = ops.stencil_apply(K, g, dims, transpose=not ctx.transpose)
        dK = ops.coeff_grad(g, xb.float(), dims, transpose=ctx.transpose)
        gw, gb = ops.weight_grad(dK, image)
        gi = ops.image_grad(dK, weights, dims) if ctx.needs_input_grad[0] else None
        return gi, gx.reshape(g.shape), gw, gb, None


def set_training_storage(model, dtype=torch.bfloat16):
    """Every block of ``model`` trains with BF16 coefficient planes and BF16 saved inputs
    (torch.bfloat16; FP32 accumulation) or in FP32 (torch.float32, the default).  Inference
    (eval_forward, the fused plans) is unaffected."""
    if dtype not in (torch.float32, torch.bfloat16):
        raise ValueError(f"training storage must be torch.float32 or torch.bfloat16 (got {dtype})")
    for m in model.modules():
        if isinstance(m, (SmallSMBlock3D, SmallSMBlockTrans3D)):
            m.storage = dtype
    return model


def _block_apply(module, image, x, transpose):
    if getattr(module, "storage", torch.float32) == torch.bfloat16 and torch.is_grad_enabled():
        return SMBlockBF16Function3D.apply(image, x, module.weight, module.bias, transpose)
    fn = SMBlockTransFunction3D if transpose else SMBlockFunction3D
    return fn.apply(image, x, module.weight, module.bias)


class SMBlockTransFunction3D(torch.autograd.Function):
    """Transpose of SMBlockFunction3D (sm_model_3d.py:50-76)."""

    @staticmethod
    def inference(image, x, weights, bias, timer=None):
        _tstart(timer, "Forward")
        y = ops.block_forward(image, x, weights, bias, transpose=True)
        _tstop(timer, "Forward")
        return y

    @staticmethod
    def forward(ctx, image, x, weights, bias):
        y = ops.block_forward(image, x, weights, bias, transpose=True)
        ctx.save_for_backward(image, x, weights, bias)
        return y

    @staticmethod
    def backward(ctx, grad_output):
        image, x, weights, bias = ctx.saved_tensors
        gx, gw, gb, gi = ops.block_backward(grad_output, image, x, weights, bias, transpose=True,
                                            image_grad=ctx.needs_input_grad[0])
        return gi, gx, gw, gb


class SmallSMBlock3D(BaseModel):
    def __init__(self, num_imgs=3, mask=False):
        super().__init__()
        if num_imgs != 3:
            raise ValueError("the sm_103a kernels take 3 image channels (air, fluid, non-solid)")
        self.mask = mask
        self.weight = nn.Parameter(torch.ones(27, num_imgs, 3, 3, 3))
        self.bias = nn.Parameter(torch.ones(27))
        self.reset_parameters(self.weight, self.bias)

    def forward(self, image, x):
        y = _block_apply(self, image, x, False)
        if self.mask:
            y = torch.where(image[1] == 0, 0.0, y)
        return y

    def eval_forward(self, image, x, timer=None):
        y = SMBlockFunction3D.inference(image, x, self.weight, self.bias, timer)
        if self.mask:
            y = torch.where(image[1] == 0, 0.0, y)
        return y


class SmallSMBlockTrans3D(BaseModel):
    def __init__(self, num_imgs=3, weight=None, bias=None):
        super().__init__()
        if num_imgs != 3:
            raise ValueError("the sm_103a kernels take 3 image channels (air, fluid, non-solid)")
        self.weight = nn.Parameter(torch.ones(27, num_imgs, 3, 3, 3)) if weight is None else weight
        self.bias = nn.Parameter(torch.ones(27)) if bias is None else bias
        if weight is None and bias is None:
            self.reset_parameters(self.weight, self.bias)

    def forward(self, image, x):
        return _block_apply(self, image, x, True)

    def eval_forward(self, image, x, timer=None):
        return SMBlockTransFunction3D.inference(image, x, self.weight, self.bias, timer)


######################
# SM linear
######################
class SMLinearFunction3D(torch.autograd.Function):
    """z = w . mean_q(shifted image patches) + b (sm_model_3d.py:118-144)."""

    @staticmethod
    def inference(image, weights, bias, timer=None):
        _tstart(timer, "Forward")
        z, _ = ops.linear_forward(image, weights, bias)
        _tstop(timer, "Forward")
        return z

    @staticmethod
    def forward(ctx, image, weights, bias, timer=None):
        z, y = ops.linear_forward(image, weights, bias)
        ctx.save_for_backward(y, weights)
        ctx.dims = tuple(image.shape[1:])
        return z

    @staticmethod
    def backward(ctx, grad_output):
        y, weights = ctx.saved_tensors
        gw, gb = ops.linear_backward(grad_output, y)
        gi = ops.linear_image_grad(grad_output, weights, ctx.dims) if ctx.needs_input_grad[0] else None
        return gi, gw, gb, None


class SmallLinearBlock3DNew(BaseModel):
    def __init__(self, num_imgs=3):
        super().__init__()
        if num_imgs != 3:
            raise ValueError("the sm_103a kernels take 3 image channels (air, fluid, non-solid)")
        self.weight = torch.ones(27, num_imgs, 3, 3, 3)
        self.bias = torch.ones(27)
        self.reset_parameters(self.weight, self.bias)
        self.weight = nn.Parameter(self.weight.mean(dim=0, keepdim=True))
        self.bias = nn.Parameter(self.bias.mean(dim=0, keepdim=True))

    def forward(self, image):
        return SMLinearFunction3D.apply(image, self.weight, self.bias)

    def eval_forward(self, image, timer=None):
        return SMLinearFunction3D.inference(image, self.weight, self.bias, timer)


######################
# level transfer with hand-written adjoints
######################
class AvgPool2Function(torch.autograd.Function):
    """F.avg_pool3d(x, (2, 2, 2))."""

    @staticmethod
    def forward(ctx, x):
        return ops.avg_pool2(x.contiguous())

    @staticmethod
    def backward(ctx, g):
        return ops.avg_pool2_adjoint(g.contiguous())


class Upsample2Function(torch.autograd.Function):
    """F.interpolate(x, scale_factor=2, mode='trilinear')."""

    @staticmethod
    def forward(ctx, x):
        return ops.upsample2(x.contiguous())

    @staticmethod
    def backward(ctx, g):
        return ops.upsample2_adjoint(g.contiguous())


class Prolong8Function(torch.autograd.Function):
    """F.interpolate(x, scale_factor=2) / 8 (nearest): the adjoint of the 2x2x2 average pool,
    the prolongation of the SPD models (sm_model_3d.py:332,378,415)."""

    @staticmethod
    def forward(ctx, x):
        return ops.avg_pool2_adjoint(x.contiguous())

    @staticmethod
    def backward(ctx, g):
        return ops.avg_pool2(g.contiguous())


class CombineFunction(torch.autograd.Function):
    """c0 * x + c1 * y with scalar (1,) tensors c0, c1 (sm_model_3d.py:258,286)."""

    @staticmethod
    def forward(ctx, c0, x, c1, y):
        x, y = x.contiguous(), y.contiguous()
        ctx.save_for_backward(c0, x, c1, y)
        return ops.axpby(c0, x, c1, y)

    @staticmethod
    def backward(ctx, g):
        c0, x, c1, y = ctx.saved_tensors
        g = g.contiguous()
        zero = torch.zeros(1, dtype=torch.float32, device=g.device)
        gx = ops.axpby(c0, g, zero, g) if ctx.needs_input_grad[1] else None
        gy = ops.axpby(c1, g, zero, g) if ctx.needs_input_grad[3] else None
        gc0 = ops.dot(g, x).to(c0.dtype).reshape(c0.shape) if ctx.needs_input_grad[0] else None
        gc1 = ops.dot(g, y).to(c1.dtype).reshape(c1.shape) if ctx.needs_input_grad[2] else None
        return gc0, gx, gc1, gy


def _direct(fn, *args):
    return fn(*args)


def _checkpointed(fn, *args):
    from torch.utils.checkpoint import checkpoint
    return checkpoint(fn, *args, use_reentrant=False)


def _check_mode(mode):
    if mode != "trilinear":
        raise ValueError(f"interpolation_mode {mode!r}: only 'trilinear' is provided by the sm_103a kernels")


######################
# Full SM Model
######################
class SmallSMModelDn3D(BaseModel):
    """Multilevel preconditioner network (sm_model_3d.py:164-287).

    Parameters are created in the reference's order (pre[1..n-1], pre[0],
    post[1..n-1], post[0], l, c0[*], c1[*]) so that a given torch seed gives
    the reference's initial weights.
    """

    def __init__(self, n, num_imgs=3, interpolation_mode="trilinear", mask=False, swap_sm_order=False):
        super().__init__()
        _check_mode(interpolation_mode)
        self.n = n
        self.mode = interpolation_mode
        self.swap_ord = swap_sm_order
        self.pre = nn.ModuleList([SmallSMBlock3D(num_imgs) for _ in range(n - 1)])
        self.pre.insert(0, SmallSMBlock3D(num_imgs, mask))
        self.post = nn.ModuleList([SmallSMBlock3D(num_imgs) for _ in range(n - 1)])
        self.post.insert(0, SmallSMBlock3D(num_imgs, mask))
        self.l = SmallSMBlock3D(num_imgs)
        self.c0 = nn.ModuleList([SmallLinearBlock3DNew(num_imgs) for _ in range(n)])
        self.c1 = nn.ModuleList([SmallLinearBlock3DNew(num_imgs) for _ in range(n)])

    def check_grid(self, shape):
        n1, n2, n3 = shape[-3:]
        f = 2 ** self.n
        if n1 % f or n2 % f or n3 % f:
            raise ValueError(f"grid {tuple(shape[-3:])} must be divisible by 2**n = {f} "
                             "(each level halves it and the upsampled level must match)")

    def eval_forward(self, image, b, timer=None, imgs=None, c0=None, c1=None):
        """Inference pass (sm_model_3d.py:180-262).  ``imgs``, ``c0``, ``c1`` are
        caller-owned cache lists, filled on the first call and reused after; when
        omitted a fresh cache is used (the reference shares mutable default
        lists across calls, which reuses a stale pyramid if the image changes)."""
        self.check_grid(image.shape)
        imgs = [] if imgs is None else imgs
        c0 = [] if c0 is None else c0
        c1 = [] if c1 is None else c1
        imgs_cached, c0_cached, c1_cached = bool(imgs), bool(c0), bool(c1)
        if not imgs_cached:
            imgs.extend([None] * self.n)
        if not c0_cached:
            c0.extend([None] * self.n)
        if not c1_cached:
            c1.extend([None] * self.n)

        _tstart(timer, "SM block")
        x = [self.pre[0].eval_forward(image, b, timer)]
        if not imgs_cached:
            imgs[0] = image
        _tstop(timer, "SM block")

        for i in range(1, self.n):
            _tstart(timer, "Downsampling")
            x.append(ops.avg_pool2(x[-1]))
            if not imgs_cached:
                imgs[i] = ops.avg_pool2(imgs[i - 1])
            _tstop(timer, "Downsampling")
            _tstart(timer, "SM block")
            x[-1] = self.pre[i].eval_forward(imgs[i], x[-1], timer)
            _tstop(timer, "SM block")

        _tstart(timer, "Downsampling")
        x.append(ops.avg_pool2(x[-1]))
        fine_img = ops.avg_pool2(imgs[-1])
        _tstop(timer, "Downsampling")
        _tstart(timer, "SM block")
        x[-1] = self.l.eval_forward(fine_img, x[-1], timer)
        _tstop(timer, "SM block")

        for i in range(self.n, 0, -1):
            _tstart(timer, "Upsamping")
            x[i] = ops.upsample2(x[i])
            _tstop(timer, "Upsamping")
            _tstart(timer, "SM linear")
            if not c0_cached:
                c0[i - 1] = self.c0[i - 1].eval_forward(imgs[i - 1], timer)
            if not c1_cached:
                c1[i - 1] = self.c1[i - 1].eval_forward(imgs[i - 1], timer)
            _tstop(timer, "SM linear")
            if self.swap_ord:
                x[i - 1] = ops.axpby(c0[i - 1], x[i - 1], c1[i - 1], x[i])
                x[i - 1] = self.post[i - 1].eval_forward(imgs[i - 1], x[i - 1], timer)
            else:
                x[i] = self.post[i - 1].eval_forward(imgs[i - 1], x[i], timer)
                x[i - 1] = ops.axpby(c0[i - 1], x[i - 1], c1[i - 1], x[i])
        return x[0]

    #: Training memory: when True, forward keeps only each level's input and output (the down
    #: sweep's outputs are the up sweep's skip vectors); the pooled block inputs, the prolongated
    #: vectors and the post-block outputs are recomputed level by level in the backward pass
    #: (torch.utils.checkpoint, non-reentrant).  Same gradients, one more forward's work.
    recompute = False

    def forward(self, image, b):
        """Training pass with autograd (sm_model_3d.py:264-287)."""
        self.check_grid(image.shape)
        n = self.n
        ck = _checkpointed if (self.recompute and torch.is_grad_enabled()) else _direct
        imgs = [image]
        for _ in range(n):
            imgs.append(AvgPool2Function.apply(imgs[-1]))
        x = [ck(lambda bb: self.pre[0](image, bb), b)]
        for i in range(1, n):
            x.append(ck(lambda xp, i=i: self.pre[i](imgs[i], AvgPool2Function.apply(xp)), x[-1]))
        x.append(ck(lambda xp: self.l(imgs[n], AvgPool2Function.apply(xp)), x[-1]))
        for i in range(n, 0, -1):
            c0 = self.c0[i - 1](imgs[i - 1])
            c1 = self.c1[i - 1](imgs[i - 1])

            def up(xc, yl, c0, c1, i=i):
                u = Upsample2Function.apply(xc)
                if self.swap_ord:
                    return self.post[i - 1](imgs[i - 1], CombineFunction.apply(c0, yl, c1, u))
                return CombineFunction.apply(c0, yl, c1, self.post[i - 1](imgs[i - 1], u))

            x[i - 1] = ck(up, x[i], x[i - 1], c0, c1)
        return x[0]

    def precond_plan(self, image, storage=torch.bfloat16, act_storage=None):
        """Coefficients of every block precomputed on ``image``: see precond.PrecondPlan."""
        from .precond import PrecondPlan
        return PrecondPlan(self, image, storage=storage, act_storage=act_storage)


######################
# SPD models
######################
class _Steps:
    """The primitive steps of a preconditioner pass: autograd Functions for training, the
    library calls directly for inference."""

    def __init__(self, train):
        self.train = train
        self.pool = AvgPool2Function.apply if train else ops.avg_pool2
        self.prolong = Prolong8Function.apply if train else ops.avg_pool2_adjoint
        self.combine = CombineFunction.apply if train else ops.axpby

    def block(self, module, image, x):
        return module(image, x) if self.train else module.eval_forward(image, x)

    def linear(self, module, image):
        return module(image) if self.train else module.eval_forward(image)


def _spd_pyramid(model, image, steps, imgs, c0, c1):
    """Image pyramid imgs[0..n] and the per-level c0 / c1; the caller's lists are filled when
    empty and reused when filled."""
    if not imgs:
        imgs.append(image)
        for _ in range(model.n):
            imgs.append(steps.pool(imgs[-1]))
    if not c0:
        c0.extend(steps.linear(model.c0[i], imgs[i]) for i in range(model.n))
    if not c1:
        c1.extend(steps.linear(model.c1[i], imgs[i]) for i in range(model.n))
    return imgs, c0, c1


class SPDSMModelDn3D(BaseModel):
    """Symmetric multilevel preconditioner (sm_model_3d.py:293-385): a V-cycle with blocks l0
    (down), l (coarsest) and l1 (up), followed by its mirror image with the transposed blocks
    l1_t, l_t, l0_t, which share the parameters of l1, l, l0.  Prolongation is nearest x2 / 8,
    the adjoint of the 2x2x2 average pool.  Module names and creation order are the
    reference's, so its checkpoints load and a given seed draws its initial weights."""

    def __init__(self, n):
        super().__init__()
        self.n = n
        self.l0 = nn.ModuleList()
        self.l1 = nn.ModuleList()
        self.l0_t = nn.ModuleList()
        self.l1_t = nn.ModuleList()
        for _ in range(n):
            self.l0.append(SmallSMBlock3D())
            self.l1.append(SmallSMBlock3D())
            self.l0_t.append(SmallSMBlockTrans3D(weight=self.l0[-1].weight, bias=self.l0[-1].bias))
            self.l1_t.append(SmallSMBlockTrans3D(weight=self.l1[-1].weight, bias=self.l1[-1].bias))
        self.l = SmallSMBlock3D()
        self.l_t = SmallSMBlockTrans3D(weight=self.l.weight, bias=self.l.bias)
        self.c0 = nn.ModuleList([SmallLinearBlock3DNew() for _ in range(n)])
        self.c1 = nn.ModuleList([SmallLinearBlock3DNew() for _ in range(n)])

    check_grid = SmallSMModelDn3D.check_grid

    def _run(self, image, b, steps, imgs, c0, c1):
        self.check_grid(image.shape)
        imgs, c0, c1 = _spd_pyramid(self, image, steps, imgs, c0, c1)
        n = self.n
        x = [steps.block(self.l0[0], imgs[0], b)]
        for i in range(1, n):
            x.append(steps.block(self.l0[i], imgs[i], steps.pool(x[-1])))
        x.append(steps.block(self.l, imgs[n], steps.pool(x[-1])))
        for i in range(n, 0, -1):
            x[i] = steps.block(self.l1[i - 1], imgs[i - 1], steps.prolong(x[i]))
            x[i - 1] = steps.combine(c0[i - 1], x[i - 1], c1[i - 1], x[i])
        x = [x[0]]
        for i in range(n):
            x.append(steps.pool(steps.block(self.l1_t[i], imgs[i], x[i])))
        x[-1] = steps.block(self.l_t, imgs[n], x[-1])
        for i in range(n - 1, -1, -1):
            x[i] = steps.combine(c0[i], x[i], c1[i], steps.prolong(x[i + 1]))
            x[i] = steps.block(self.l0_t[i], imgs[i], x[i])
        return x[0]

    def forward(self, image, b):
        """Training pass with autograd (sm_model_3d.py:349-385)."""
        return self._run(image, b, _Steps(True), [], [], [])

    def eval_forward(self, image, b, timer=None, imgs=None, c0=None, c1=None):
        """Inference pass (sm_model_3d.py:313-347).  ``imgs``, ``c0``, ``c1`` are optional
        caller-owned caches of the image pyramid and the level coefficients."""
        return self._run(image, b, _Steps(False), [] if imgs is None else imgs,
                         [] if c0 is None else c0, [] if c1 is None else c1)

    def precond_plan(self, image, storage=torch.bfloat16, act_storage=None):
        """Coefficients of every block (and of its transpose) precomputed on ``image``:
        see precond.PrecondPlan."""
        from .precond import PrecondPlan
        return PrecondPlan(self, image, storage=storage, act_storage=act_storage)


class SmallSPDSMModelDn3D(BaseModel):
    """Reduced symmetric preconditioner (sm_model_3d.py:388-444): M = S^T S, S the down sweep
    (blocks l0, pooling, coarsest block l); the up sweep applies l_t, the nearest x2 / 8
    prolongation, c0^2 x + c1^2 y and the transposed blocks l0_t.  Module names and creation
    order are the reference's."""

    def __init__(self, n):
        super().__init__()
        self.n = n
        self.l0 = nn.ModuleList()
        self.l0_t = nn.ModuleList()
        for _ in range(n):
            self.l0.append(SmallSMBlock3D())
            self.l0_t.append(SmallSMBlockTrans3D(weight=self.l0[-1].weight, bias=self.l0[-1].bias))
        self.l = SmallSMBlock3D()
        self.l_t = SmallSMBlockTrans3D(weight=self.l.weight, bias=self.l.bias)
        self.c0 = nn.ModuleList([SmallLinearBlock3DNew() for _ in range(n)])
        self.c1 = nn.ModuleList([SmallLinearBlock3DNew() for _ in range(n)])

    check_grid = SmallSMModelDn3D.check_grid

    def _run(self, image, b, steps, imgs, c0, c1):
        self.check_grid(image.shape)
        imgs, c0, c1 = _spd_pyramid(self, image, steps, imgs, c0, c1)
        n = self.n
        x = [steps.block(self.l0[0], imgs[0], b)]
        for i in range(1, n):
            x.append(steps.block(self.l0[i], imgs[i], steps.pool(x[-1])))
        x.append(steps.block(self.l, imgs[n], steps.pool(x[-1])))
        x[-1] = steps.block(self.l_t, imgs[n], x[-1])
        for i in range(n, 0, -1):
            x[i] = steps.prolong(x[i])
            x[i - 1] = steps.combine(c0[i - 1] * c0[i - 1], x[i - 1], c1[i - 1] * c1[i - 1], x[i])
            x[i - 1] = steps.block(self.l0_t[i - 1], imgs[i - 1], x[i - 1])
        return x[0]

    def forward(self, image, b):
        """Training pass with autograd (sm_model_3d.py:404-423)."""
        return self._run(image, b, _Steps(True), [], [], [])

    def eval_forward(self, image, b, timer=None, imgs=None, c0=None, c1=None):
        """Inference pass (sm_model_3d.py:425-444); ``imgs``, ``c0``, ``c1`` as in
        SPDSMModelDn3D.eval_forward."""
        return self._run(image, b, _Steps(False), [] if imgs is None else imgs,
                         [] if c0 is None else c0, [] if c1 is None else c1)

    def precond_plan(self, image, storage=torch.bfloat16, act_storage=None):
        """Coefficients of every block (and of its transpose) precomputed on ``image``:
        see precond.PrecondPlan."""
        from .precond import PrecondPlan
        return PrecondPlan(self, image, storage=storage, act_storage=act_storage)
