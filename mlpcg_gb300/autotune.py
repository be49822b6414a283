"""Schedule autotuning for the fused solver.

Two schedules, each tuned by timing whole solves with CUDA events and cached
in a JSON file so that a later process applies the choice without timing:

* ``tune_solver``: the number of 256-thread CTAs of the solver's grid-stride
  kernels (dot products, q-form, SpMV, update, true residual), candidates 1-8
  per SM; keyed by device name, grid shape and method.
* ``tune_plan``: the preconditioner's block schedule -- from how many tiles per
  SM down a level runs the block kernels that load each run's coefficients up
  front (0, 1, 2, 4 or 8), and whether the coarse levels run as one thread-block
  cluster launch; keyed by device name, grid shape, levels, coefficient dtype
  and method.  Every choice gives the same outputs.

The block kernels' tile shape (2 x 16 x 64) is fixed at build time.
"""
from __future__ import annotations

import json
import os
import statistics
from pathlib import Path

import ctypes as C
import torch

from ._lib import call


def default_cache_path() -> Path:
    root = os.environ.get("MLPCG_AUTOTUNE_CACHE")
    if root:
        return Path(root)
    return Path(os.path.expanduser("~")) / ".cache" / "mlpcg_gb300" / "autotune.json"


def load_cache(path: Path | None = None) -> dict:
    path = Path(path) if path is not None else default_cache_path()
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def save_cache(cache: dict, path: Path | None = None) -> None:
    path = Path(path) if path is not None else default_cache_path()
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(".tmp")
    tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
    os.replace(tmp, path)


def schedule_key(device_name: str, shape, method: str) -> str:
    return f"{device_name}|{'x'.join(str(int(s)) for s in shape)}|{method}"


def candidates(sm_count: int, max_blocks: int = 1216):
    """CTA counts to try: 1, 2, 3, 4, 6 and 8 per SM (within the solver's limit)."""
    out = [k * sm_count for k in (1, 2, 3, 4, 6, 8) if k * sm_count <= max_blocks]
    return out or [max_blocks]


def pick_best(timings: dict) -> int:
    """The candidate with the smallest time (the smaller count on a tie)."""
    return min(sorted(timings), key=lambda k: timings[k])


def set_schedule(solver, blocks: int) -> None:
    call("mlpcg_solver_set_schedule", solver._h, int(blocks))


def get_schedule(solver) -> int:
    v = C.c_int()
    call("mlpcg_solver_get_schedule", solver._h, C.byref(v))
    return v.value


def _time_solve(solver, b, reps: int) -> float:
    for _ in range(2):
        solver.launch(b)
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        solver.launch(b)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    return statistics.median(times)


def tune_solver(solver, b: torch.Tensor | None = None, reps: int = 5, cache_path: Path | None = None,
                retune: bool = False, measure=None) -> int:
    """Apply the fastest CTA count for this solver's grid and method (cached); returns it.
    ``measure(solver, blocks) -> ms`` replaces the CUDA-event timing (for tests)."""
    dev = solver.flags.device
    props = torch.cuda.get_device_properties(dev)
    key = schedule_key(props.name, solver.shape, solver.method)
    cache = load_cache(cache_path)
    if not retune and key in cache:
        set_schedule(solver, cache[key]["blocks"])
        return cache[key]["blocks"]
    b = solver.b if b is None else b
    timings = {}
    for nb in candidates(props.multi_processor_count):
        set_schedule(solver, nb)
        timings[nb] = measure(solver, nb) if measure is not None else _time_solve(solver, b, reps)
    best = pick_best(timings)
    set_schedule(solver, best)
    cache[key] = {"blocks": best, "ms": {str(k): round(v, 4) for k, v in timings.items()}}
    save_cache(cache, cache_path)
    return best


def plan_key(device_name: str, shape, levels: int, dtype: str, method: str) -> str:
    return f"plan|{device_name}|{'x'.join(str(int(v)) for v in shape)}|L{int(levels)}|{dtype}|{method}"


def plan_candidates(cluster_available: bool):
    """(small-level tiles per SM, coarse cluster) pairs to try."""
    out = [(k, 0) for k in (0, 1, 2, 4, 8)]
    if cluster_available:
        out += [(k, 1) for k in (0, 2)]
    return out


def apply_plan_schedule(solver, small: int, cluster: int) -> None:
    solver.plan.set_small_levels(small)
    solver.plan.set_coarse_cluster(bool(cluster))
    set_schedule(solver, get_schedule(solver))  # recapture the solver's graph with the new launches


def tune_plan(solver, b: torch.Tensor | None = None, reps: int = 5, cache_path: Path | None = None,
              retune: bool = False, measure=None):
    """Apply the fastest block schedule of the solver's preconditioner (cached); returns
    (small-level tiles per SM, coarse cluster).  ``measure(solver, choice) -> ms`` replaces the
    CUDA-event timing (for tests)."""
    dev = solver.flags.device
    props = torch.cuda.get_device_properties(dev)
    plan = solver.plan
    key = plan_key(props.name, solver.shape, plan.levels, str(plan.storage).replace("torch.", ""), solver.method)
    cache = load_cache(cache_path)
    if not retune and key in cache:
        choice = tuple(cache[key]["choice"])
        apply_plan_schedule(solver, *choice)
        return choice
    plan.set_coarse_cluster(True)
    cluster_ok = plan.coarse_cluster()[0] > 0
    b = solver.b if b is None else b
    timings = {}
    for choice in plan_candidates(cluster_ok):
        apply_plan_schedule(solver, *choice)
        timings[choice] = measure(solver, choice) if measure is not None else _time_solve(solver, b, reps)
    best = min(sorted(timings), key=lambda c: timings[c])
    apply_plan_schedule(solver, *best)
    cache[key] = {"choice": list(best), "ms": {f"{k[0]},{k[1]}": round(v, 4) for k, v in timings.items()}}
    save_cache(cache, cache_path)
    return best
