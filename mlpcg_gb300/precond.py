"""PrecondPlan: SmallSMModelDn3D.eval_forward (or SmallSPDSMModelDn3D's) with
every block's coefficients precomputed once per (image, weights) and fused
level kernels.

The reference re-evaluates each block's 27 coefficients from the image inside
every call (sm_block_3d_kernel.cu:45-65) and caches only the image pyramid and
c0/c1 (sm_model_3d.py:180-239).  The plan evaluates them once into 27 planes
(BF16 or FP32) per block, so an application is 2n+1 bandwidth-bound kernels
(mlpcg_precond_apply).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._lib import BF16, F32, call
from .ops import _check, _p, _stream

_DT = {torch.float32: F32, torch.bfloat16: BF16}


KIND_SM, KIND_SMALL_SPD, KIND_SPD = 0, 1, 2   # MLPCG_PRECOND_* of the header


def network_kind(model) -> int:
    from .sm_model_3d import SmallSPDSMModelDn3D, SPDSMModelDn3D
    if isinstance(model, SmallSPDSMModelDn3D):
        return KIND_SMALL_SPD
    if isinstance(model, SPDSMModelDn3D):
        return KIND_SPD
    return KIND_SM


def _is_small_spd(model) -> bool:
    return network_kind(model) == KIND_SMALL_SPD


def pack_params(model) -> torch.Tensor:
    """Flat F32 parameter vector in the order mlpcg_precond_setup expects: blocks pre, post, l
    (SmallSPDSMModelDn3D: l0, l; SPDSMModelDn3D: l0, l1, l), then the linear blocks c0, c1."""
    n = model.n
    kind = network_kind(model)
    if kind == KIND_SMALL_SPD:
        blocks = list(model.l0) + [model.l]
    elif kind == KIND_SPD:
        blocks = list(model.l0) + list(model.l1) + [model.l]
    else:
        blocks = list(model.pre) + list(model.post) + [model.l]
    parts = []
    for blk in blocks:
        parts += [blk.weight.detach().reshape(-1), blk.bias.detach().reshape(-1)]
    for lin in list(model.c0) + list(model.c1):
        parts += [lin.weight.detach().reshape(-1), lin.bias.detach().reshape(-1)]
    flat = torch.cat([p.float() for p in parts]).contiguous()
    assert flat.numel() == len(blocks) * 2214 + 2 * n * 82
    return flat


class PrecondPlan:
    """z = M r for one image; ``apply`` is graph-capturable (no host sync, no allocation with ``out``).

    ``model`` is a SmallSMModelDn3D, a SmallSPDSMModelDn3D (M = S^T S) or an
    SPDSMModelDn3D (M = V^T V) -- the last two for textbook PCG;
    ``coefficients()`` returns c0, c1 (the squares for SmallSPDSMModelDn3D)."""

    LAYOUTS = {"dense": 0, "classed": 1}

    def __init__(self, model, image, storage=torch.bfloat16, act_storage=None, layout="classed"):
        if layout not in self.LAYOUTS:
            raise ValueError(f"layout must be one of {sorted(self.LAYOUTS)} (got {layout!r})")
        for dt in (storage, act_storage):
            if dt is not None and dt not in _DT:
                raise ValueError(f"storage dtypes must be torch.float32 or torch.bfloat16 (got {dt})")
        _check(image, "image")
        if image.dim() != 4 or image.shape[0] != 3:
            raise RuntimeError("image must have shape (3, N1, N2, N3)")
        act_storage = storage if act_storage is None else act_storage
        self.shape = tuple(int(s) for s in image.shape[1:])
        self.levels = model.n
        self.storage, self.act_storage, self.layout = storage, act_storage, layout
        self.kind = network_kind(model)
        self.spd = self.kind != KIND_SM
        self.masked = False if self.spd else bool(model.pre[0].mask)
        self.swap = False if self.spd else bool(model.swap_ord)
        self.device = image.device
        lib = _lib.load()
        h = C.c_void_p()
        if self.spd:
            call("mlpcg_precond_create_kind", *self.shape, model.n, self.kind, _DT[storage], _DT[act_storage],
                 self.LAYOUTS[layout], C.byref(h))
        else:
            call("mlpcg_precond_create", *self.shape, model.n, _DT[storage], _DT[act_storage],
                 int(bool(model.swap_ord)), int(bool(model.pre[0].mask)), self.LAYOUTS[layout], C.byref(h))
        self._h = h
        self._lib = lib
        nbytes = lib.mlpcg_precond_workspace(h)
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=image.device)
        self.params = pack_params(model).to(image.device)
        self.image = image
        call("mlpcg_precond_setup", h, _p(self.workspace), nbytes, _p(image), _p(self.params),
             _stream(image.device))

    @property
    def handle(self):
        return self._h

    def coefficients(self) -> torch.Tensor:
        c = torch.empty(2 * self.levels, dtype=torch.float32, device=self.device)
        call("mlpcg_precond_coefficients", self._h, _p(c), _stream(self.device))
        return c

    def _check_vectors(self, r, scale, out):
        """r and out: contiguous F32 with one value per cell of the plan's grid on its device;
        scale: None or an F32 value there.  The kernels index them by the plan's grid alone."""
        n = self.shape[0] * self.shape[1] * self.shape[2]
        for t, name in ((r, "r"), (out, "out")):
            if t is None:
                continue
            _check(t, name)
            if t.numel() != n or t.device != self.device:
                raise RuntimeError(f"{name} must hold {n} values on {self.device} (got {t.numel()} on {t.device})")
        if scale is not None:
            _check(scale, "scale")
            if scale.numel() < 1 or scale.device != self.device:
                raise RuntimeError(f"scale must hold one value on {self.device}")

    def apply(self, r: torch.Tensor, scale: torch.Tensor | None = None, out: torch.Tensor | None = None):
        """z = M(r * scale) on the full grid; r F32 with the grid's numel."""
        self._check_vectors(r, scale, out)
        z = torch.empty(self.shape, dtype=torch.float32, device=r.device) if out is None else out
        call("mlpcg_precond_apply", self._h, _p(r), _p(scale), _p(z), _stream(r.device))
        return z.reshape(r.shape) if out is None else z

    def apply_stages(self, first: int, last: int, r: torch.Tensor, scale=None, out=None):
        """Launch stages [first, last] of an application (see mlpcg_precond_apply_stages)."""
        self._check_vectors(r, scale, out)
        z = torch.empty(self.shape, dtype=torch.float32, device=r.device) if out is None else out
        call("mlpcg_precond_apply_stages", self._h, int(first), int(last), _p(r), _p(scale), _p(z),
             _stream(r.device))
        return z

    def class_counts(self, level: int):
        """(general cells, mixed runs) of a classed level; (-1, -1) on dense levels."""
        g, r = C.c_int64(), C.c_int64()
        call("mlpcg_precond_class_counts", self._h, int(level), C.byref(g), C.byref(r), _stream(self.device))
        return g.value, r.value

    def copy_failed(self) -> bool:
        """True if a level-0 tile copy of an application so far did not complete (mlpcg_precond_check)."""
        v = C.c_int()
        call("mlpcg_precond_check", self._h, C.byref(v), _stream(self.device))
        return bool(v.value)

    def coarse_cluster(self):
        """(first level, CTAs) of the coarse levels run as one thread-block cluster launch, or (-1, 0)
        (mlpcg_precond_coarse_cluster)."""
        lc, c = C.c_int(), C.c_int()
        call("mlpcg_precond_coarse_cluster", self._h, C.byref(lc), C.byref(c))
        return lc.value, c.value

    def set_coarse_cluster(self, on: bool):
        """Run the coarse levels as one cluster launch or as one kernel per stage (the default)
        (mlpcg_precond_set_coarse_cluster); the outputs are the same."""
        call("mlpcg_precond_set_coarse_cluster", self._h, int(bool(on)))

    def set_small_levels(self, tiles_per_sm: int):
        """Levels with at most ``tiles_per_sm`` tiles per SM run the prefetching block kernels
        (mlpcg_precond_set_small_levels; 0 = never); the outputs are the same."""
        call("mlpcg_precond_set_small_levels", self._h, int(tiles_per_sm))

    def set_copy_stall(self, on: bool):
        """Test knob of the bounded TMA waits (mlpcg_precond_set_copy_stall): with ``on`` the level-0
        tile kernels' first wait runs out on an ordinary copy and ``copy_failed()`` turns true; every
        call clears the copy-failed word."""
        call("mlpcg_precond_set_copy_stall", self._h, int(bool(on)), _stream(self.device))

    def class_counts_transposed(self, level: int):
        """(general cells, mixed runs) of the transposed block of a classed level (SPD plans)."""
        g, r = C.c_int64(), C.c_int64()
        call("mlpcg_precond_class_counts_transposed", self._h, int(level), C.byref(g), C.byref(r),
             _stream(self.device))
        return g.value, r.value

    def general_cells(self, level: int) -> int:
        """Cells of a classed level whose neighbourhood is not a single material (-1 on dense levels)."""
        return self.class_counts(level)[0]

    def mixed_runs(self, level: int) -> int:
        """8-cell runs of a classed level that carry a coefficient record (-1 on dense levels)."""
        return self.class_counts(level)[1]

    def level_info(self, level: int):
        n1, n2, n3, fast = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        call("mlpcg_precond_level_info", self._h, int(level), C.byref(n1), C.byref(n2), C.byref(n3),
             C.byref(fast))
        return (n1.value, n2.value, n3.value), bool(fast.value)

    def stage_names(self):
        n = self.levels
        names = [f"pre{l}" for l in range(n)] + [f"l{n}"] + [f"post{2 * n - s}" for s in range(n + 1, 2 * n + 1)]
        if self.kind == KIND_SPD:   # V, then V^T
            names += [f"t_{s}" for s in names]
        return names

    def predict(self, fluid_cells):
        """A model_predict-style callable (test.py:42-51) on compressed FP64 vectors."""
        n = 1
        for s in self.shape:
            n *= s

        def predict(r, timer=None, imgs=None, c0=None, c1=None):
            r32 = r.to(torch.float32)
            g = torch.zeros(n, dtype=torch.float32, device=r.device)
            g[fluid_cells] = r32
            scale = (1.0 / torch.clamp(r32.norm(), min=1e-12)).reshape(1)
            z = self.apply(g, scale)
            return z.reshape(-1)[fluid_cells].double()

        return predict

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.mlpcg_precond_destroy(h)
            except Exception:
                pass
            self._h = None
