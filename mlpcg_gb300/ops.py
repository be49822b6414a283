"""torch-level wrappers of the C ABI, and drop-in stand-ins for the reference's
JIT extension modules ``smblock3d``, ``smblocktrans3d`` and ``smlinear3d``
(sm_model_3d.py:11-16).

Every function launches on the current torch CUDA stream and allocates its
outputs and workspace through torch's caching allocator.  Input checks raise
RuntimeError with the reference's messages ("x must be a CUDA tensor",
"x must be contiguous", sm_block_3d.cpp:26-28).
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import _lib
from ._lib import BF16, F32, F64, call, query

_DT = {torch.float32: F32, torch.bfloat16: BF16, torch.float64: F64}


def _stream(device=None) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _check(t: torch.Tensor, name: str, dtypes=(torch.float32,)):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a tensor")
    if not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise RuntimeError(f"{name} must be contiguous")
    if dtypes is not None and t.dtype not in dtypes:
        raise RuntimeError(f"{name} has dtype {t.dtype}; expected one of {list(dtypes)}")


def _workspace(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


def plane_stride(n: int) -> int:
    """Elements between the 27 coefficient planes: n rounded up to 64."""
    return (n + 63) // 64 * 64


def _spatial(image: torch.Tensor, padded: bool):
    if image.dim() != 4 or image.shape[0] != 3:
        raise RuntimeError(f"image must have shape (3, N1, N2, N3), got {tuple(image.shape)}")
    n1, n2, n3 = image.shape[1:]
    if padded:
        n1, n2, n3 = n1 - 2, n2 - 2, n3 - 2
    return int(n1), int(n2), int(n3)


def _batch(x: torch.Tensor, dims, padded: bool) -> int:
    n1, n2, n3 = dims
    sp = (n1 + 2, n2 + 2, n3 + 2) if padded else (n1, n2, n3)
    if tuple(x.shape[-3:]) != sp:
        raise RuntimeError(f"x spatial shape {tuple(x.shape[-3:])} does not match the image {sp}")
    return x.numel() // math.prod(sp)


def _out_shape(x: torch.Tensor, dims, padded: bool):
    return tuple(x.shape[:-3]) + tuple(dims)


def _block_params(weight: torch.Tensor, bias: torch.Tensor):
    """A block's W (27, 3, 3, 3, 3) and b (27,), by element count (the kernels read exactly these)."""
    if weight.numel() != 27 * 81 or bias.numel() != 27:
        raise RuntimeError(f"weight must hold 27 x 3 x 3 x 3 x 3 values and bias 27 "
                           f"(got {weight.numel()} and {bias.numel()})")


# ----------------------------------------------------------------------------
# stencil blocks (reference semantics: coefficients evaluated per call)
# ----------------------------------------------------------------------------
def block_forward(image, x, weight, bias, transpose=False, padded=False):
    """y = smblock3d(image, x) (transpose=False) or smblocktrans3d(image, x)."""
    for t, n in ((image, "image"), (x, "x"), (weight, "weight"), (bias, "bias")):
        _check(t, n)
    _block_params(weight, bias)
    dims = _spatial(image, padded)
    B = _batch(x, dims, padded)
    y = torch.empty(_out_shape(x, dims, padded), dtype=torch.float32, device=x.device)
    ws = _workspace(query("mlpcg_sm_block_3d_workspace", *dims), x.device)
    call("mlpcg_sm_block_3d_forward", _p(image), int(padded), _p(x), int(padded), _p(weight), _p(bias),
         _p(y), B, *dims, int(transpose), _p(ws), ws.numel(), _stream(x.device))
    return y


def block_backward(grad_out, image, x, weight, bias, transpose=False, padded=False, image_grad=False):
    """(grad_x, grad_w, grad_b, grad_image or None) of block_forward."""
    grad_out = grad_out.contiguous()
    for t, n in ((grad_out, "grad_output"), (image, "image"), (x, "x"), (weight, "weight"), (bias, "bias")):
        _check(t, n)
    _block_params(weight, bias)
    dims = _spatial(image, padded)
    B = _batch(x, dims, padded)
    if grad_out.numel() != B * math.prod(dims):
        raise RuntimeError(f"grad_output must hold {B} x {tuple(dims)} values (got {tuple(grad_out.shape)})")
    gx = torch.empty(_out_shape(x, dims, padded), dtype=torch.float32, device=x.device)
    gw = torch.empty((27, 3, 3, 3, 3), dtype=torch.float32, device=x.device)
    gb = torch.empty((27,), dtype=torch.float32, device=x.device)
    gi = torch.empty((3,) + dims, dtype=torch.float32, device=x.device) if image_grad else None
    ws = _workspace(query("mlpcg_sm_block_3d_workspace", *dims), x.device)
    call("mlpcg_sm_block_3d_backward", _p(grad_out), _p(image), int(padded), _p(x), int(padded),
         _p(weight), _p(bias), _p(gx), _p(gw), _p(gb), _p(gi), B, *dims, int(transpose),
         _p(ws), ws.numel(), _stream(x.device))
    return gx, gw, gb, gi


def linear_forward(image, weight, bias):
    """(z, y) of smlinear3d: y = the 81 shifted means of the image, z = w . y + b.

    ``weight`` may stack several linear blocks: (nlin, 81) or (nlin, 3, 3, 3, 3),
    with ``bias`` (nlin,); then z has nlin entries.
    """
    for t, n in ((image, "image"), (weight, "weights"), (bias, "bias")):
        _check(t, n)
    dims = _spatial(image, False)
    nlin = bias.numel()
    if weight.numel() != 81 * nlin:
        raise RuntimeError(f"weights must hold 81 values per output (got {weight.numel()} for {nlin})")
    z = torch.empty((nlin,), dtype=torch.float32, device=image.device)
    y = torch.empty((1, 3, 3, 3, 3), dtype=torch.float32, device=image.device)
    ws = _workspace(query("mlpcg_sm_linear_3d_workspace", *dims), image.device)
    call("mlpcg_sm_linear_3d_forward", _p(image), *dims, _p(weight), _p(bias), nlin, _p(z), _p(y),
         _p(ws), ws.numel(), _stream(image.device))
    return z, y


def linear_backward(grad_out, y):
    _check(grad_out.contiguous(), "grad_output")
    _check(y, "y")
    grad_out = grad_out.contiguous()
    gw = torch.empty_like(y)
    gb = torch.empty((1,), dtype=torch.float32, device=y.device)
    call("mlpcg_sm_linear_3d_backward", _p(grad_out), _p(y), _p(gw), _p(gb), _stream(y.device))
    return gw, gb


def linear_image_grad(grad_out, weight, dims):
    gi = torch.empty((3,) + tuple(dims), dtype=torch.float32, device=weight.device)
    call("mlpcg_sm_linear_3d_image_grad", _p(grad_out.contiguous()), _p(weight), _p(gi), *dims,
         _stream(weight.device))
    return gi


# ----------------------------------------------------------------------------
# precomputed coefficients
# ----------------------------------------------------------------------------
def stencil_gen(image, weight, bias, dtype=torch.float32, out=None):
    """K planes (27, plane_stride(n)) of one block on ``image`` (3, N1, N2, N3)."""
    for t, n in ((image, "image"), (weight, "weight"), (bias, "bias")):
        _check(t, n)
    _block_params(weight, bias)
    dims = _spatial(image, False)
    ps = plane_stride(math.prod(dims))
    if out is not None:
        _check(out, "out", (torch.float32, torch.bfloat16))
        if out.numel() < 27 * ps:
            raise RuntimeError(f"out must hold 27 planes of {ps} values (got {out.numel()} values)")
    K = out if out is not None else torch.empty((27, ps), dtype=dtype, device=image.device)
    call("mlpcg_stencil_gen", _p(image), 0, *dims, _p(weight), _p(bias), _p(K), _DT[K.dtype], ps,
         _stream(image.device))
    return K


def stencil_apply(K, x, dims, transpose=False, out_dtype=torch.float32):
    _check(K, "K", (torch.float32, torch.bfloat16))
    _check(x, "x", (torch.float32, torch.bfloat16))
    n = math.prod(dims)
    if K.dim() != 2 or K.shape[0] != 27 or K.shape[1] < n:
        raise RuntimeError(f"K must be 27 planes of at least {n} values (got {tuple(K.shape)})")
    if x.numel() == 0 or x.numel() % n:
        raise RuntimeError(f"x must hold a whole number of {tuple(dims)} grids (got {x.numel()} values)")
    B = x.numel() // n
    y = torch.empty(x.shape, dtype=out_dtype, device=x.device)
    call("mlpcg_stencil_apply", _p(K), _DT[K.dtype], K.shape[-1], _p(x), _DT[x.dtype], 0, _p(y),
         _DT[out_dtype], B, *dims, int(transpose), _stream(x.device))
    return y


def coeff_grad(grad_out, x, dims, transpose=False):
    """dK (27 planes, FP32): the gradient of the block output with respect to its coefficients,
    dK_p(q) = sum_b g_b(q) x_b(q + off_p) (transposed: the adjoint relation)."""
    _check(grad_out, "grad_output")
    _check(x, "x")
    n = math.prod(dims)
    if grad_out.numel() != x.numel() or x.numel() % n:
        raise RuntimeError(f"grad_output and x must hold the same whole number of {tuple(dims)} grids")
    ps = plane_stride(n)
    dK = torch.empty((27, ps), dtype=torch.float32, device=x.device)
    call("mlpcg_stencil_coeff_grad", _p(grad_out), _p(x), 0, _p(dK), ps, x.numel() // n, *dims, int(transpose),
         _stream(x.device))
    return dK


def weight_grad(dK, image):
    """(grad_weight (27, 3, 3, 3, 3), grad_bias (27)) from the coefficient gradient dK."""
    _check(dK, "dK")
    _check(image, "image")
    dims = _spatial(image, False)
    gw = torch.empty((27, 3, 3, 3, 3), dtype=torch.float32, device=image.device)
    gb = torch.empty((27,), dtype=torch.float32, device=image.device)
    ws = _workspace(query("mlpcg_stencil_wgrad_workspace", *dims), image.device)
    call("mlpcg_stencil_wgrad", _p(dK), dK.shape[-1], _p(image), 0, *dims, _p(gw), _p(gb), _p(ws), ws.numel(),
         _stream(image.device))
    return gw, gb


def image_grad(dK, weight, dims):
    """grad_image (3, N1, N2, N3) from the coefficient gradient dK."""
    _check(dK, "dK")
    _check(weight, "weight")
    gi = torch.empty((3,) + tuple(dims), dtype=torch.float32, device=dK.device)
    call("mlpcg_stencil_image_grad", _p(dK), dK.shape[-1], _p(weight), _p(gi), *dims, _stream(dK.device))
    return gi


# ----------------------------------------------------------------------------
# level transfer
# ----------------------------------------------------------------------------
def avg_pool2(x):
    _check(x, "x", (torch.float32, torch.bfloat16))
    n1, n2, n3 = x.shape[-3:]
    B = x.numel() // (n1 * n2 * n3)
    y = torch.empty(tuple(x.shape[:-3]) + (n1 // 2, n2 // 2, n3 // 2), dtype=x.dtype, device=x.device)
    call("mlpcg_avg_pool2", _p(x), _p(y), _DT[x.dtype], B, n1, n2, n3, _stream(x.device))
    return y


def avg_pool2_adjoint(y):
    _check(y, "y", (torch.float32, torch.bfloat16))
    c1, c2, c3 = y.shape[-3:]
    B = y.numel() // (c1 * c2 * c3)
    x = torch.empty(tuple(y.shape[:-3]) + (2 * c1, 2 * c2, 2 * c3), dtype=y.dtype, device=y.device)
    call("mlpcg_avg_pool2_adjoint", _p(y), _p(x), _DT[y.dtype], B, 2 * c1, 2 * c2, 2 * c3, _stream(y.device))
    return x


def upsample2(x):
    _check(x, "x", (torch.float32, torch.bfloat16))
    n1, n2, n3 = x.shape[-3:]
    B = x.numel() // (n1 * n2 * n3)
    y = torch.empty(tuple(x.shape[:-3]) + (2 * n1, 2 * n2, 2 * n3), dtype=x.dtype, device=x.device)
    call("mlpcg_upsample2", _p(x), _p(y), _DT[x.dtype], B, n1, n2, n3, _stream(x.device))
    return y


def upsample2_adjoint(y):
    _check(y, "y", (torch.float32, torch.bfloat16))
    f1, f2, f3 = y.shape[-3:]
    B = y.numel() // (f1 * f2 * f3)
    x = torch.empty(tuple(y.shape[:-3]) + (f1 // 2, f2 // 2, f3 // 2), dtype=y.dtype, device=y.device)
    call("mlpcg_upsample2_adjoint", _p(y), _p(x), _DT[y.dtype], B, f1 // 2, f2 // 2, f3 // 2, _stream(y.device))
    return x


def axpby(c0, x, c1, y):
    """c0 * x + c1 * y with c0, c1 one-element device tensors."""
    _check(x, "x", (torch.float32, torch.bfloat16))
    _check(y, "y", (x.dtype,))
    if x.numel() != y.numel():
        raise RuntimeError(f"axpby: x and y sizes differ ({x.numel()} vs {y.numel()})")
    c0 = c0.reshape(1).to(torch.float32).contiguous()
    c1 = c1.reshape(1).to(torch.float32).contiguous()
    out = torch.empty_like(x)
    call("mlpcg_axpby", _p(c0), _p(x), _p(c1), _p(y), _p(out), _DT[x.dtype], x.numel(), _stream(x.device))
    return out


def laplacian(flags, x):
    """Matrix-free mixed-boundary Poisson operator on full-grid vectors (F32 or F64)."""
    _check(flags, "flags", (torch.uint8,))
    _check(x, "x", (torch.float32, torch.float64))
    if flags.dim() < 3 or x.numel() != flags.numel():
        raise RuntimeError(f"laplacian: x must hold one value per cell of flags (got {x.numel()} for "
                           f"{tuple(flags.shape)})")
    dims = tuple(flags.shape[-3:])
    y = torch.empty_like(x)
    call("mlpcg_laplacian_apply", _p(flags), _p(x), _p(y), _DT[x.dtype], *dims, _stream(x.device))
    return y


def dot(x, y):
    """FP64 (1,) device tensor holding sum(x * y), deterministic."""
    _check(x, "x", (torch.float32, torch.bfloat16, torch.float64))
    _check(y, "y", (x.dtype,))
    if x.numel() != y.numel():
        raise RuntimeError("dot: size mismatch")
    out = torch.empty((1,), dtype=torch.float64, device=x.device)
    ws = _workspace(query("mlpcg_dot_workspace", x.numel()), x.device)
    call("mlpcg_dot", _p(x), _p(y), _DT[x.dtype], x.numel(), _p(out), _p(ws), ws.numel(), _stream(x.device))
    return out


# ----------------------------------------------------------------------------
# stand-ins for the reference's JIT extension modules (sm_model_3d.py:11-16);
# they take the F.pad'ed tensors exactly like the originals
# ----------------------------------------------------------------------------
class _BlockExt:
    def __init__(self, transpose: bool):
        self._t = transpose

    def inference(self, image, x, weights, bias):
        return [block_forward(image, x, weights, bias, self._t, padded=True)]

    def forward(self, image, x, weights, bias):
        return [block_forward(image, x, weights, bias, self._t, padded=True)]

    def backward(self, grad_output, image, x, weights, bias):
        gx, gw, gb, _ = block_backward(grad_output, image, x, weights, bias, self._t, padded=True)
        return [gx, gw, gb]


class _LinearExt:
    def inference(self, image, weights, bias):
        z, y = linear_forward(image, weights, bias)
        return [z, y]

    forward = inference

    def backward(self, grad_output, y):
        gw, gb = linear_backward(grad_output, y)
        return [gw, gb]


smblock3d = _BlockExt(False)
smblocktrans3d = _BlockExt(True)
smlinear3d = _LinearExt()
