"""SmallSMModelDn3D composed from the numpy FP64 ops (oracle; test infrastructure only).

Follows SmallSMModelDn3D.forward (sm_model_3d.py:264-287), including the
``swap_sm_order`` and ``mask`` options (sm_model_3d.py:88,93,245-258).
``params`` is a dict of numpy arrays keyed like the reference state_dict:
``pre.{i}.weight``, ``pre.{i}.bias``, ``post.{i}.*``, ``l.*``, ``c0.{i}.*``,
``c1.{i}.*``.
"""
from __future__ import annotations

import numpy as np

from . import ops


def _blk(params, name):
    return params[f"{name}.weight"], params[f"{name}.bias"]


def forward(params, img, b, n, swap_sm_order=False, mask=False):
    """Preconditioner output for rhs ``b`` of shape (..., N1, N2, N3)."""
    img = np.asarray(img, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)

    def block(name, im, x, masked=False):
        y = ops.sm_block(im, x, *_blk(params, name))
        if masked:
            y = np.where(im[1] == 0, 0.0, y)
        return y

    x = [block("pre.0", img, b, mask)]
    imgs = [img]
    for i in range(1, n):
        x.append(ops.avg_pool2(x[-1]))
        imgs.append(ops.avg_pool2(imgs[-1]))
        x[-1] = block(f"pre.{i}", imgs[-1], x[-1])
    x.append(ops.avg_pool2(x[-1]))
    imgs.append(ops.avg_pool2(imgs[-1]))
    x[-1] = block("l", imgs[-1], x[-1])
    for i in range(n, 0, -1):
        x[i] = ops.upsample2(x[i])
        c0 = ops.sm_linear(imgs[i - 1], *_blk(params, f"c0.{i-1}"))[0][0]
        c1 = ops.sm_linear(imgs[i - 1], *_blk(params, f"c1.{i-1}"))[0][0]
        if swap_sm_order:
            x[i - 1] = c0 * x[i - 1] + c1 * x[i]
            x[i - 1] = block(f"post.{i-1}", imgs[i - 1], x[i - 1], mask and i == 1)
        else:
            x[i] = block(f"post.{i-1}", imgs[i - 1], x[i], mask and i == 1)
            x[i - 1] = c0 * x[i - 1] + c1 * x[i]
    return x[0]


def spd_forward(params, img, b, n):
    """SPDSMModelDn3D.forward (sm_model_3d.py:349-385): a V-cycle with blocks l0 (down), l
    (coarsest) and l1 (up, after the nearest/8 prolongation), then its mirror with the
    transposed blocks l1_t (down), l_t and l0_t (up).  Keys: ``l0.{i}``, ``l1.{i}``, ``l``,
    ``c0.{i}``, ``c1.{i}`` (the ``*_t`` modules share these parameters)."""
    img = np.asarray(img, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)

    def block(name, im, x, transpose=False):
        return ops.sm_block(im, x, *_blk(params, name), transpose=transpose)

    x = [block("l0.0", img, b)]
    imgs = [img]
    for i in range(1, n):
        x.append(ops.avg_pool2(x[-1]))
        imgs.append(ops.avg_pool2(imgs[-1]))
        x[-1] = block(f"l0.{i}", imgs[-1], x[-1])
    x.append(ops.avg_pool2(x[-1]))
    imgs.append(ops.avg_pool2(imgs[-1]))
    x[-1] = block("l", imgs[-1], x[-1])
    c0 = [ops.sm_linear(imgs[i], *_blk(params, f"c0.{i}"))[0][0] for i in range(n)]
    c1 = [ops.sm_linear(imgs[i], *_blk(params, f"c1.{i}"))[0][0] for i in range(n)]
    for i in range(n, 0, -1):
        x[i] = ops.prolong_nearest8(x[i])
        x[i] = block(f"l1.{i-1}", imgs[i - 1], x[i])
        x[i - 1] = c0[i - 1] * x[i - 1] + c1[i - 1] * x[i]
    x = [x[0]]
    for i in range(n):
        x.append(ops.avg_pool2(block(f"l1.{i}", imgs[i], x[i], transpose=True)))
    x[-1] = block("l", imgs[-1], x[-1], transpose=True)
    for i in range(n - 1, -1, -1):
        x[i + 1] = ops.prolong_nearest8(x[i + 1])
        x[i] = c0[i] * x[i] + c1[i] * x[i + 1]
        x[i] = block(f"l0.{i}", imgs[i], x[i], transpose=True)
    return x[0]


def small_spd_forward(params, img, b, n):
    """SmallSPDSMModelDn3D.forward (sm_model_3d.py:404-423): M = S^T S with S the down sweep
    (blocks l0, pooling, coarsest l) -- the up sweep applies the transposed blocks l_t and
    l0_t, the nearest/8 prolongation (the pool's adjoint) and the squared c0, c1."""
    img = np.asarray(img, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)

    def block(name, im, x, transpose=False):
        return ops.sm_block(im, x, *_blk(params, name), transpose=transpose)

    x = [block("l0.0", img, b)]
    imgs = [img]
    for i in range(1, n):
        x.append(ops.avg_pool2(x[-1]))
        imgs.append(ops.avg_pool2(imgs[-1]))
        x[-1] = block(f"l0.{i}", imgs[-1], x[-1])
    x.append(ops.avg_pool2(x[-1]))
    imgs.append(ops.avg_pool2(imgs[-1]))
    x[-1] = block("l", imgs[-1], x[-1])
    x[-1] = block("l", imgs[-1], x[-1], transpose=True)
    for i in range(n, 0, -1):
        x[i] = ops.prolong_nearest8(x[i])
        c0 = ops.sm_linear(imgs[i - 1], *_blk(params, f"c0.{i-1}"))[0][0]
        c1 = ops.sm_linear(imgs[i - 1], *_blk(params, f"c1.{i-1}"))[0][0]
        x[i - 1] = c0 ** 2 * x[i - 1] + c1 ** 2 * x[i]
        x[i - 1] = block(f"l0.{i-1}", imgs[i - 1], x[i - 1], transpose=True)
    return x[0]


def spd_param_names(n, small=False):
    """Parameter names in the reference's creation (RNG) order: per level l0 (and l1 unless
    ``small``), then l, c0[*], c1[*] (sm_model_3d.py:294-311, 389-402)."""
    names = []
    for i in range(n):
        names.append(f"l0.{i}")
        if not small:
            names.append(f"l1.{i}")
    names.append("l")
    for grp in ("c0", "c1"):
        for i in range(n):
            names.append(f"{grp}.{i}")
    return names


def param_names(n):
    """Parameter names in the reference's creation (RNG) order (sm_model_3d.py:165-178)."""
    names = []
    for grp in ("pre", "post"):
        for i in list(range(1, n)) + [0]:
            names.append(f"{grp}.{i}")
    names.append("l")
    for grp in ("c0", "c1"):
        for i in range(n):
            names.append(f"{grp}.{i}")
    return names
