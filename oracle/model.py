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
