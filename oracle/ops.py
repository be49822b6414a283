"""numpy FP64 restatement of the reference's extension ops (oracle; test infrastructure only).

Conventions: a field is an array (N1, N2, N3) (or (B, N1, N2, N3)); tap
p = 9k + 3l + o has offset off_p = (k-1, l-1, o-1); the image has 3 channels
[air, fluid, non-solid] (lib/read_data.py:28-39) and is zero outside the grid
(the F.pad of sm_model_3d.py:24-26).
"""
from __future__ import annotations

import numpy as np

TAPS = [(p // 9 - 1, (p // 3) % 3 - 1, p % 3 - 1) for p in range(27)]


def _pad1(a: np.ndarray) -> np.ndarray:
    """Zero-pad the last three axes by one cell (F.pad(x, (1,)*6))."""
    pad = [(0, 0)] * (a.ndim - 3) + [(1, 1)] * 3
    return np.pad(a, pad)


def _shift(ap: np.ndarray, d, shape) -> np.ndarray:
    """View of padded ``ap`` at q + d for all interior q (d in {-1,0,1}^3)."""
    n1, n2, n3 = shape
    return ap[..., 1 + d[0]:1 + d[0] + n1, 1 + d[1]:1 + d[1] + n2, 1 + d[2]:1 + d[2] + n3]


def image_patches(img: np.ndarray) -> np.ndarray:
    """(81, N1, N2, N3): patch column s*27 + (9m+3n+o) = img[s, q + (m-1, n-1, o-1)]."""
    img = np.asarray(img, dtype=np.float64)
    shape = img.shape[1:]
    ip = _pad1(img)
    return np.stack([_shift(ip[s], TAPS[o], shape) for s in range(3) for o in range(27)])


def stencil_coeffs(img, weight, bias) -> np.ndarray:
    """K (27, N1, N2, N3): K_p(q) = bias_p + sum_{s,m,n,o} W[p,s,m,n,o] img_zpad[s, q+(m,n,o)-1].

    Follows the coefficient loop of sm_block_3d_cuda_inference_kernel
    (torch_extension/sm_block_3d_kernel.cu:45-65).
    """
    P = image_patches(img)
    W = np.asarray(weight, dtype=np.float64).reshape(27, 81)
    K = np.tensordot(W, P, axes=(1, 0))
    return K + np.asarray(bias, dtype=np.float64).reshape(27, 1, 1, 1)


def stencil_apply(K, x) -> np.ndarray:
    """y(q) = sum_p K_p(q) x(q + off_p), x zero outside (sm_block_3d_kernel.cu:66-70)."""
    x = np.asarray(x, dtype=np.float64)
    shape = K.shape[1:]
    xp = _pad1(x)
    y = np.zeros_like(x)
    for p, d in enumerate(TAPS):
        y += K[p] * _shift(xp, d, shape)
    return y


def stencil_apply_trans(K, x) -> np.ndarray:
    """y(q) = sum_p K_p(q - off_p) x(q - off_p) (sm_block_trans_3d_kernel.cu:45-73)."""
    x = np.asarray(x, dtype=np.float64)
    shape = K.shape[1:]
    y = np.zeros(x.shape[:-3] + tuple(np.array(shape) + 2), dtype=np.float64)
    n1, n2, n3 = shape
    for p, d in enumerate(TAPS):
        # contribution K_p(q') x(q') lands on q = q' + off_p
        y[..., 1 + d[0]:1 + d[0] + n1, 1 + d[1]:1 + d[1] + n2, 1 + d[2]:1 + d[2] + n3] += K[p] * x
    return y[..., 1:-1, 1:-1, 1:-1]


def sm_block(img, x, weight, bias, transpose=False) -> np.ndarray:
    """smblock3d / smblocktrans3d forward on unpadded inputs."""
    K = stencil_coeffs(img, weight, bias)
    return stencil_apply_trans(K, x) if transpose else stencil_apply(K, x)


def coeff_grad(g, x, transpose=False) -> np.ndarray:
    """dK summed over the batch (factors of sm_block_3d_kernel.cu:122-229 and
    sm_block_trans_3d_kernel.cu:173-289)."""
    g = np.asarray(g, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    if g.ndim == 3:
        g, x = g[None], x[None]
    shape = g.shape[1:]
    dK = np.zeros((27,) + shape)
    if not transpose:
        xp = _pad1(x)
        for p, d in enumerate(TAPS):
            dK[p] = (g * _shift(xp, d, shape)).sum(0)
    else:
        gp = _pad1(g)
        for p, d in enumerate(TAPS):
            dK[p] = (_shift(gp, d, shape) * x).sum(0)
    return dK


def weight_grad(dK, img):
    """dW[p, so] = sum_q dK_p(q) patch_so(q); db[p] = sum_q dK_p(q)."""
    P = image_patches(img).reshape(81, -1)
    D = dK.reshape(27, -1)
    return (D @ P.T).reshape(27, 3, 3, 3, 3), D.sum(1)


def image_grad(dK, weight):
    """d/d img(s, c) of sum_p <dK_p, K_p>: sum_{p,o} W[p,s,o] dK_p(c - off_o)."""
    W = np.asarray(weight, dtype=np.float64).reshape(27, 3, 27)
    shape = dK.shape[1:]
    out = np.zeros((3,) + shape)
    n1, n2, n3 = shape
    for o, d in enumerate(TAPS):
        # K_p(q) uses img(q + d): img cell c receives dK_p(c - d)
        contrib = np.tensordot(W[:, :, o], dK, axes=(0, 0))  # (3, N...) at q
        buf = np.zeros((3,) + tuple(np.array(shape) + 2))
        buf[:, 1 + d[0]:1 + d[0] + n1, 1 + d[1]:1 + d[1] + n2, 1 + d[2]:1 + d[2] + n3] += contrib
        out += buf[:, 1:-1, 1:-1, 1:-1]
    return out


def block_backward(g, img, x, weight, bias, transpose=False):
    """smblock3d.backward / smblocktrans3d.backward: (grad_x, grad_W, grad_b, grad_img)."""
    K = stencil_coeffs(img, weight, bias)
    gx = stencil_apply(K, g) if transpose else stencil_apply_trans(K, g)
    dK = coeff_grad(g, x, transpose)
    gw, gb = weight_grad(dK, img)
    return gx, gw, gb, image_grad(dK, weight)


def linear_means(img) -> np.ndarray:
    """y[s,k,l,o] = mean_q img_zpad[s, q + (k-1,l-1,o-1)]  (sm_linear_3d_kernel.cu:43-84, 185)."""
    P = image_patches(img)
    return P.reshape(81, -1).mean(1).reshape(1, 3, 3, 3, 3)


def sm_linear(img, weight, bias):
    """smlinear3d.inference: (z, y) with z = w . y + b (sm_linear_3d_kernel.cu:185-188)."""
    y = linear_means(img)
    z = float(np.dot(np.asarray(weight, np.float64).ravel(), y.ravel())) + float(np.asarray(bias).ravel()[0])
    return np.array([z]), y


def linear_image_grad(g, weight, shape):
    """d z / d img for z = w . linear_means(img) + b."""
    n = np.prod(shape)
    W = np.asarray(weight, dtype=np.float64).reshape(3, 27)
    out = np.zeros((3,) + tuple(shape))
    n1, n2, n3 = shape
    for o, d in enumerate(TAPS):
        buf = np.zeros((3,) + tuple(np.array(shape) + 2))
        buf[:, 1 + d[0]:1 + d[0] + n1, 1 + d[1]:1 + d[1] + n2, 1 + d[2]:1 + d[2] + n3] += W[:, o, None, None, None]
        out += buf[:, 1:-1, 1:-1, 1:-1]
    return out * (float(np.asarray(g).ravel()[0]) / n)


def avg_pool2(x) -> np.ndarray:
    """F.avg_pool3d(x, (2,2,2)) on even sizes (sm_model_3d.py:206)."""
    x = np.asarray(x, dtype=np.float64)
    *lead, n1, n2, n3 = x.shape
    return x.reshape(*lead, n1 // 2, 2, n2 // 2, 2, n3 // 2, 2).mean(axis=(-5, -3, -1))


def _up1(x, axis):
    """Linear x2 along one axis, align_corners=False, source index clamped at 0."""
    n = x.shape[axis]
    f = np.arange(2 * n)
    src = np.maximum(0.5 * (f + 0.5) - 0.5, 0.0)
    i0 = np.floor(src).astype(int)
    i1 = np.minimum(i0 + 1, n - 1)
    l1 = src - i0
    a = np.take(x, i0, axis=axis)
    b = np.take(x, i1, axis=axis)
    shape = [1] * x.ndim
    shape[axis] = 2 * n
    l1 = l1.reshape(shape)
    return (1 - l1) * a + l1 * b


def upsample2(x) -> np.ndarray:
    """F.interpolate(x, scale_factor=2, mode='trilinear') (sm_model_3d.py:230)."""
    x = np.asarray(x, dtype=np.float64)
    return _up1(_up1(_up1(x, -3), -2), -1)


def prolong_nearest8(x) -> np.ndarray:
    """F.interpolate(x, scale_factor=2) / 8 (default 'nearest' mode; sm_model_3d.py:332,378,415):
    every coarse value copied to its 2x2x2 children, divided by 8 -- the adjoint of avg_pool2."""
    x = np.asarray(x, dtype=np.float64)
    for ax in (-3, -2, -1):
        x = np.repeat(x, 2, axis=ax)
    return x / 8.0


def init_block_params(gen_uniform):
    """BaseModel.reset_parameters on a (27,3,3,3,3) weight and (27,) bias (model.py:22-29):
    kaiming_uniform(a=sqrt(5)) gives bound 1/sqrt(fan_in) = 1/9 for both."""
    bound = 1.0 / 9.0
    w = gen_uniform(-bound, bound, (27, 3, 3, 3, 3))
    b = gen_uniform(-bound, bound, (27,))
    return w, b
