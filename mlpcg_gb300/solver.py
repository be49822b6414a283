"""FusedSolver: npsd / npcg with the network preconditioner, entirely on the GPU.

One CUDA graph per solver: a conditional WHILE node wraps one iteration
(the fused preconditioner kernels, the orthogonalisation / SpMV / update
kernels with FP64 cross-thread reductions, a double-float true residual every
``true_every`` iterations, the iteration's control step).  ``solve`` is a
single graph launch; the host synchronises only to read the result.
``solve_host`` is the host-to-host form for a new frame, with the rhs
transfer overlapped with the preconditioner set-up.

The drop-in solvers of ``cg.py`` keep the reference's per-iteration host
round trips (cg_tests.py:90,266); this is the form they are compared with.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import call
from .ops import _check, _p, _stream
from .precond import PrecondPlan, pack_params

METHODS = {"npsd": 0, "npcg": 1}
STATUS = {0: "running", 1: "converged", 2: "max_it", 3: "breakdown", 4: "nonfinite", 5: "copy_failed"}


@dataclass
class SolveResult:
    x: torch.Tensor             # (N1, N2, N3) FP64, zero off-fluid
    iterations: int
    status: str
    rel_res: float              # final FP64 true relative residual
    history: np.ndarray         # relative residual after each iteration (index 0 = initial)


def flags_to_image(flags: torch.Tensor) -> torch.Tensor:
    """[air, fluid, non-solid] F32 channels from uint8 flags on the device."""
    img = torch.empty((3,) + tuple(flags.shape), dtype=torch.float32, device=flags.device)
    call("mlpcg_flags_to_image", _p(flags), _p(img), flags.numel(), _stream(flags.device))
    return img


def _host_mapped(t: torch.Tensor) -> bool:
    """A contiguous FP64 tensor in pinned host memory that kernels reach at its own address."""
    if t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous() or not t.is_pinned():
        return False
    v = C.c_int(0)
    call("mlpcg_host_mapped", C.c_void_p(t.data_ptr()), C.byref(v))
    return bool(v.value)


class FusedSolver:
    def __init__(self, model, flags: torch.Tensor, method="npsd", max_it=100, tol=1e-6, true_every=25,
                 storage=torch.bfloat16, act_storage=None, image=None, plan: PrecondPlan | None = None,
                 layout="classed"):
        if method not in METHODS:
            raise ValueError(f"method must be one of {sorted(METHODS)} (got {method!r})")
        if flags.dtype != torch.uint8 or flags.dim() != 3 or not flags.is_cuda:
            raise ValueError("flags must be a (N1, N2, N3) uint8 CUDA tensor")
        self.flags = flags.contiguous()
        self.shape = tuple(int(s) for s in flags.shape)
        self.method, self.max_it, self.tol, self.true_every = method, int(max_it), float(tol), int(true_every)
        dev = flags.device
        if plan is None:
            image = flags_to_image(self.flags) if image is None else image
            plan = PrecondPlan(model, image, storage=storage, act_storage=act_storage, layout=layout)
        self.plan = plan
        lib = _lib.load()
        self._lib = lib
        h = C.c_void_p()
        call("mlpcg_solver_create", *self.shape, plan.handle, METHODS[method], self.max_it,
             C.c_double(self.tol), self.true_every, C.byref(h))
        self._h = h
        nbytes = lib.mlpcg_solver_workspace(h)
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        self.b = torch.zeros(self.shape, dtype=torch.float64, device=dev)
        self.x = torch.zeros(self.shape, dtype=torch.float64, device=dev)
        call("mlpcg_solver_bind", h, _p(self.workspace), nbytes, _p(self.flags), _p(self.b), _p(self.x))
        self._side = self._order = self._bf = self._xf = None

    def set_image(self, model, image: torch.Tensor, flags: torch.Tensor | None = None):
        """New frame: recompute the plan in place (the captured graph stays valid)."""
        _check(image, "image")
        if tuple(image.shape) != (3,) + self.shape or image.device != self.flags.device:
            raise RuntimeError(f"image must have shape {(3,) + self.shape} on {self.flags.device} "
                               f"(got {tuple(image.shape)} on {image.device})")
        if flags is not None:
            self.flags.copy_(flags)
        if model is not None:
            self.plan.params.copy_(pack_params(model))
        call("mlpcg_precond_setup", self.plan.handle, _p(self.plan.workspace), self.plan.workspace.numel(),
             _p(image), _p(self.plan.params), _stream(self.flags.device))
        self.plan.image = image

    def launch(self, b: torch.Tensor | None = None, x0: torch.Tensor | None = None, use_graph=True):
        """Enqueue a solve (asynchronous with use_graph)."""
        if b is not None and b.data_ptr() != self.b.data_ptr():
            self.b.copy_(b.reshape(self.shape))
        if x0 is None:  # x0 = 0 without a memset: the solve does not read x and writes all of it
            call("mlpcg_solver_solve_zero_guess", self._h, int(bool(use_graph)), _stream(self.flags.device))
            return
        if x0.data_ptr() != self.x.data_ptr():
            self.x.copy_(x0.reshape(self.shape))
        call("mlpcg_solver_solve", self._h, int(bool(use_graph)), _stream(self.flags.device))

    def solve_host(self, flags_h: torch.Tensor, b_h: torch.Tensor, x_out_h: torch.Tensor | None = None,
                   model=None, use_graph=True):
        """A new frame from host memory: flags (uint8) and rhs (FP64) in, the solution into
        ``x_out_h``.  ``b_h`` and ``x_out_h`` are either full grids (N1*N2*N3 values) or fluid-DOF
        vectors -- one value per fluid cell of ``flags_h`` in flat cell order, the compressed vectors
        the reference's solvers take -- told apart by their size; fluid-DOF vectors move only the
        fluid values over the host link.  The rhs is moved on a side stream while the image pyramid
        and the coefficients are built from the flags, so its transfer hides behind the set-up.
        Fluid-DOF vectors in pinned host memory that kernels reach (mlpcg_host_mapped) are read and
        written by the scatter and gather kernels themselves, with no staging copy; other buffers go
        through device copies.  With pinned host buffers every transfer is asynchronous; call
        ``result()`` to wait."""
        dev = self.flags.device
        n = self.b.numel()
        fluid = b_h.numel() != n
        if fluid and x_out_h is not None and x_out_h.numel() != b_h.numel():
            raise ValueError("x_out_h must have the length of b_h")
        main = torch.cuda.current_stream(dev)
        if self._side is None:
            self._side = torch.cuda.Stream(dev)
            self._order = torch.empty(int(self._lib.mlpcg_fluid_order_entries(n)), dtype=torch.int32, device=dev)
        side = self._side
        m = b_h.numel()
        direct_b = fluid and _host_mapped(b_h)
        direct_x = fluid and x_out_h is not None and _host_mapped(x_out_h)
        if fluid and not (direct_b and direct_x) and (self._bf is None or self._bf.numel() < m):
            self._bf = torch.empty(max(m, 1), dtype=torch.float64, device=dev)
            self._xf = torch.empty(max(m, 1), dtype=torch.float64, device=dev)
        side.wait_stream(main)  # the previous solve has finished with these buffers
        if not direct_b:
            with torch.cuda.stream(side):
                if fluid:
                    self._bf[:m].copy_(b_h.reshape(-1), non_blocking=True)
                else:
                    self.b.copy_(b_h.reshape(self.shape), non_blocking=True)
        self.flags.copy_(flags_h.reshape(self.shape), non_blocking=True)
        st = _stream(dev)
        if fluid:
            call("mlpcg_fluid_order", _p(self.flags), n, _p(self._order), st)
        if direct_b:  # the scatter reads the host vector beside the set-up, once the order is known
            side.wait_stream(main)
            call("mlpcg_scatter_fluid", C.c_void_p(b_h.data_ptr()), m, _p(self.flags), _p(self._order), n,
                 _p(self.b), C.c_void_p(side.cuda_stream))
        self.set_image(model, flags_to_image(self.flags))
        main.wait_stream(side)
        if fluid and not direct_b:
            call("mlpcg_scatter_fluid", _p(self._bf), m, _p(self.flags), _p(self._order), n, _p(self.b), st)
        self.launch(None, use_graph=use_graph)
        if x_out_h is not None:
            if direct_x:
                call("mlpcg_gather_fluid", _p(self.x), _p(self.flags), _p(self._order), n,
                     C.c_void_p(x_out_h.data_ptr()), m, st)
            elif fluid:
                call("mlpcg_gather_fluid", _p(self.x), _p(self.flags), _p(self._order), n, _p(self._xf), m, st)
                x_out_h.view(-1).copy_(self._xf[:m], non_blocking=True)
            else:
                x_out_h.view(self.shape).copy_(self.x, non_blocking=True)

    def set_copy_stall(self, on: bool):
        """Test knob of the bounded TMA waits (mlpcg_solver_set_copy_stall): from the next solve the
        npsd SpMV's first tile wait runs out on an ordinary copy and the solve ends 'copy_failed'."""
        call("mlpcg_solver_set_copy_stall", self._h, int(bool(on)))

    def set_dependent_launch(self, on: bool):
        """Programmatic edges between consecutive kernels of the captured iteration (on by default;
        mlpcg_solver_set_dependent_launch): identical results, the launch gaps hidden."""
        call("mlpcg_solver_set_dependent_launch", self._h, int(bool(on)))

    def set_fused_dots(self, on: bool):
        """The solver's products (npsd z . Ap, npcg r . z) summed in the preconditioner's level-0
        post-block (on by default, where the plan allows it; mlpcg_solver_set_fused_dots) or in a
        separate pass."""
        call("mlpcg_solver_set_fused_dots", self._h, int(bool(on)))

    def fused_dots(self) -> bool:
        """Whether the solve sums its products in the preconditioner's epilogue."""
        v = C.c_int()
        call("mlpcg_solver_fused_dots", self._h, C.byref(v))
        return bool(v.value)

    def dependent_edges(self) -> int:
        """Programmatic edges in the current graph (0 before the first graph solve or when off)."""
        n = C.c_int()
        call("mlpcg_solver_dependent_edges", self._h, C.byref(n))
        return n.value

    def result(self, with_history=True) -> SolveResult:
        it, st, rel = C.c_int(), C.c_int(), C.c_double()
        hist = np.zeros(self.max_it + 1, dtype=np.float64)
        call("mlpcg_solver_result", self._h, C.byref(it), C.byref(st), C.byref(rel),
             hist.ctypes.data_as(C.c_void_p) if with_history else None, _stream(self.flags.device))
        return SolveResult(self.x, it.value, STATUS[st.value], rel.value, hist[: it.value + 1])

    def solve(self, b: torch.Tensor, x0: torch.Tensor | None = None, use_graph=True) -> SolveResult:
        self.launch(b, x0, use_graph)
        return self.result()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.mlpcg_solver_destroy(h)
            except Exception:
                pass
            self._h = None


class BatchSolver:
    """Several FusedSolvers -- any grid sizes, methods, tolerances and iteration limits -- solved by
    one graph launch: the loop runs while any system is running, each iteration runs every system as
    a parallel branch, and a system that has converged (or stopped) skips its kernels from then on.
    The solvers must stay bound (no new ``set_image`` flags size change) while batched."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        if not self.solvers:
            raise ValueError("BatchSolver needs at least one solver")
        dev = self.solvers[0].flags.device
        if any(s.flags.device != dev for s in self.solvers):
            raise ValueError("all solvers of a batch must be on one device")
        self._lib = self.solvers[0]._lib
        arr = (C.c_void_p * len(self.solvers))(*[s._h.value for s in self.solvers])
        h = C.c_void_p()
        call("mlpcg_batch_create", arr, len(self.solvers), C.byref(h))
        self._h = h
        self.device = dev

    def launch(self, bs=None, x0s=None):
        """Enqueue the solves of all systems (b: one rhs per system, or None to keep the current)."""
        n = len(self.solvers)
        bs = [None] * n if bs is None else list(bs)
        x0s = [None] * n if x0s is None else list(x0s)
        for s, b, x0 in zip(self.solvers, bs, x0s):
            if b is not None and b.data_ptr() != s.b.data_ptr():
                s.b.copy_(b.reshape(s.shape))
            if x0 is None:
                s.x.zero_()
            elif x0.data_ptr() != s.x.data_ptr():
                s.x.copy_(x0.reshape(s.shape))
        call("mlpcg_batch_solve", self._h, _stream(self.device))

    def solve(self, bs=None, x0s=None):
        self.launch(bs, x0s)
        return [s.result() for s in self.solvers]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.mlpcg_batch_destroy(h)
            except Exception:
                pass
            self._h = None

