"""Time to a 1e-6 relative residual of the neural-preconditioned Poisson solve on one GB300.

Workload (default): one 256^3 synthetic scene (seed 7, 6 solid spheres, one
wall layer, a fluid pool under a wavy height field, air above), the 5-level
SmallSMModelDn3D preconditioner, npsd (the reference's solver) to an FP64
true relative residual of 1e-6, max 100 iterations.

A step = one whole solve of that scene with inputs resident in HBM: flags ->
image channels, the preconditioner plan (image pyramid, the coefficients of
all 11 blocks, c0/c1), then the graph-captured fused iteration.  The L2 is
flushed between steps.  Before the warm-up (untimed) the solver's CTA count is
picked by mlpcg_gb300.autotune (config.solver_schedule).  Also reported:
  * plain_ms   -- the plain FP32 drop-in (reference semantics: coefficients
                  re-evaluated in every block call, FP64 CG vectors, a host
                  round trip per iteration), one solve;
  * setup_ms / solve_ms -- the step split at the end of the plan setup;
  * stages_ms  -- each preconditioner kernel timed alone;
  * roofline   -- the level-0 pre-block kernel (the largest launch of an
                  iteration) against the measured HBM copy bandwidth;
  * e2e        -- the same solve through the public API from pinned host
                  buffers (flags, rhs in; solution out);
  * cpu_baseline -- the reference's CPU path (torch-CPU Conv3d blocks, FP64
                  CSR npsd) on this host, a bounded sample of iterations,
                  extrapolated to the iteration count of the solve;
  * amg_cpu_baseline -- the reference's other host comparator, AMG-
                  preconditioned FP64 CG (smoothed aggregation, SPAI-0), run
                  to the same tolerance on the same scene in a child process
                  (oracle/amg.cpp; setup + solve time, iterations, residual).

``--model small_spd`` / ``--model spd`` run the same harness on the symmetric
networks SmallSPDSMModelDn3D / SPDSMModelDn3D (default solver npcg, textbook
PCG; weights smallspd_l<n>.npz / spd_l<n>.npz when present); their CPU path is
the same torch-CPU blocks composed as that network with the reference's npcg.

``--impl reference`` times only that CPU path and prints its own line.
Multi-GPU (``--gpus N`` under torchrun): N independent replicas, one scene
per rank, no collective in the solve; the reported time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ms to 1e-6 rel. residual at 256³: BF16-fused vs plain FP32 PCG, 1 GB300; %HBM BW"
WEIGHTS_DIR = ROOT / "mlpcg_gb300" / "weights"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--levels", type=int, default=5)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--spheres", type=int, default=6)
    ap.add_argument("--model", default="smallsm", choices=["smallsm", "small_spd", "spd"])
    ap.add_argument("--method", default=None, choices=["npsd", "npcg"],
                    help="default: npsd (smallsm), npcg (small_spd, spd)")
    ap.add_argument("--max-it", type=int, default=100)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--weights", default=None, help="npz state dict (default: committed trained weights)")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default solver CTA count instead of the autotuned one (tuning is untimed)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-reference-solution", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-amg", action="store_true",
                    help="skip the host AMG-preconditioned CG comparator run beside the CPU baseline")
    ap.add_argument("--amg-timeout", type=float, default=240.0)
    ap.add_argument("--no-graph", action="store_true",
                    help="plain launches of the same kernels with a host check per iteration (for profilers)")
    ap.add_argument("--batch", action="store_true",
                    help="the batched workload: 16 scenes (seeds 100-115) of 4 x 64^3, 4 x 96^3 (4 levels), "
                         "4 x 128^3, 4 x 192^3 (5 levels) in one graph launch, against 16 plain solves")
    args = ap.parse_args()
    if args.method is None:
        args.method = "npsd" if args.model == "smallsm" else "npcg"
    return args


MODEL_NAMES = {"smallsm": "SmallSMModelDn3D", "small_spd": "SmallSPDSMModelDn3D", "spd": "SPDSMModelDn3D"}


def weights_path(args):
    if args.weights:
        return Path(args.weights)
    prefix = {"smallsm": "smallsm", "small_spd": "smallspd", "spd": "spd"}[args.model]
    p = WEIGHTS_DIR / f"{prefix}_l{args.levels}.npz"
    return p if p.exists() else None


def load_model(args, device):
    import torch
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D, SmallSPDSMModelDn3D, SPDSMModelDn3D
    torch.manual_seed(0)
    if args.model == "small_spd":
        m = SmallSPDSMModelDn3D(args.levels)
    elif args.model == "spd":
        m = SPDSMModelDn3D(args.levels)
    else:
        m = SmallSMModelDn3D(args.levels, 3, "trilinear")
    wp = weights_path(args)
    meta = {}
    if wp is not None:
        d = np.load(wp)
        m.load_state_dict({k: torch.from_numpy(d[k]) for k in m.state_dict()})
        mp = wp.with_suffix(".json")
        if mp.exists():
            meta = json.loads(mp.read_text())
        meta["weights"] = str(wp.relative_to(ROOT)) if wp.is_relative_to(ROOT) else str(wp)
    else:
        meta["weights"] = "random init (torch.manual_seed(0), reference init order)"
    return m.to(device), meta


# ----------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.path = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        rows = []
        for line in open(self.path):
            f = [c.strip() for c in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5], f[6], f[7], f[8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            for name, v in zip(names, r[2:]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "samples": len(rows), "reasons": sorted(reasons)}


def max_over_ranks(value: float, world: int, device="cpu") -> float:
    """Max of a per-rank time over the replicas (each rank solves its own scene)."""
    if world <= 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t)


def replica_seed(base_seed: int, rank: int) -> int:
    """Scene seed of a replica: rank r solves scene base_seed + r."""
    return base_seed + rank


# ----------------------------------------------------------------------------
# launch accounting
# ----------------------------------------------------------------------------
def precond_launches(plan):
    """Kernel launches of one preconditioner application (mirrors run_apply / run_apply_spd in
    precond.cu)."""
    n = plan.levels
    fast = [plan.level_info(l)[1] for l in range(n + 1)]
    if plan.kind == 2:   # SPDSMModelDn3D: V then V^T
        cnt = 2                                            # coarsest l, l_t
        for l in range(n):
            cnt += 1 if fast[l] else 2 + (1 if l == 0 else 0)  # V down (level 0: scale copy)
            cnt += 2 if fast[l] else 3                          # V up: prolongation + block
            cnt += 1 if fast[l] else 2                          # V^T down
            cnt += 2 if fast[l] else 3 + (1 if l == 0 else 0)  # V^T up (level 0: mask)
        return cnt
    lc, _ = plan.coarse_cluster()                     # levels lc..n: one cluster launch
    cnt = 1 if lc > 0 else 0
    for l in range(n if lc <= 0 else lc):
        cnt += 1 if fast[l] else (2 + (1 if l == 0 else 0))
    if lc <= 0:
        cnt += 2 if plan.spd else 1                   # coarsest l (and l_t)
    for l in range(n - 1 if lc <= 0 else lc - 1, -1, -1):
        if plan.spd:
            cnt += 2 if fast[l] else 3 + (1 if l == 0 else 0)   # prolongation pass + block
        elif fast[l]:
            cnt += 2 if l == 0 else 1                 # level 0: prolongation pass + block
        else:
            cnt += 3 + (2 if l == 0 else 0)
    return cnt


def setup_launches(plan):
    """Kernel launches of flags -> image plus one plan setup (mirrors mlpcg_precond_setup)."""
    n = plan.levels
    cls = [plan.layout == "classed" and plan.level_info(l)[1] for l in range(n + 1)]
    cnt = 1 + n + 1                                # image, pyramid, fluid mask
    cnt += 2 if any(cls) else 0                    # uniform vectors and material records of all blocks
    for l in range(n + 1):
        fast = plan.level_info(l)[1]
        if plan.kind == 2:                         # l0 + l1 (or l), then their transposes gathered
            nb = 2 if l < n else 1
            cnt += (6 + 4 + 2 * nb) if cls[l] else (nb + (nb if fast else 0))
            continue
        if plan.spd:                               # forward block, then its transpose gathered from it
            cnt += 12 if cls[l] else (2 if fast else 1)
            continue
        nb = 2 if l < n else 1
        cnt += 6 if cls[l] else nb                 # classify, 2 tile scans, list, records, fill | dense planes
    cnt += 1 if cls[0] else 0                      # level 0: the pattern table's coefficients
    return cnt + 3 * n + (1 if plan.kind == 1 else 0)   # c0/c1: class sums, reduce, finalize per level (+ squares)


# ----------------------------------------------------------------------------
def run_ours(args, rank, world):
    import torch
    from mlpcg_gb300 import cg
    from mlpcg_gb300.laplacian import FluidLaplacian
    from mlpcg_gb300.scenes import make_scene
    from mlpcg_gb300.solver import FusedSolver, flags_to_image

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    N = args.size
    scene = make_scene(N, replica_seed(args.seed, rank), args.spheres)
    model, meta = load_model(args, dev)
    flags = torch.as_tensor(scene.flags, device=dev)
    b = torch.as_tensor(scene.rhs, device=dev)
    n = N ** 3
    image = flags_to_image(flags)
    solver = FusedSolver(model, flags, method=args.method, max_it=args.max_it, tol=args.tol,
                         storage=torch.bfloat16, image=image)
    plan = solver.plan
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    tuned = None
    if not args.no_autotune:
        # the solver's CTA count for this device / grid / method, timed before the timed region
        from mlpcg_gb300 import autotune
        cache = Path(tempfile.gettempdir()) / f"mlpcg_autotune_{os.getpid()}.json"
        tuned = autotune.tune_solver(solver, b, reps=5, cache_path=cache, retune=True)
        tuned = {"solver_ctas": tuned, "ms_by_ctas": autotune.load_cache(cache)[
            autotune.schedule_key(torch.cuda.get_device_properties(dev).name, solver.shape, solver.method)]["ms"]}
        # the preconditioner's block schedule (small-level kernels, coarse cluster)
        small, cluster = autotune.tune_plan(solver, b, reps=3, cache_path=cache, retune=True)
        pk = autotune.plan_key(torch.cuda.get_device_properties(dev).name, solver.shape, plan.levels, "bfloat16",
                               solver.method)
        tuned.update({"small_level_tiles_per_sm": small, "coarse_cluster": bool(cluster),
                      "ms_by_block_schedule": autotune.load_cache(cache)[pk]["ms"]})
        cache.unlink(missing_ok=True)

    def step(mid=None):
        img = flags_to_image(flags)
        solver.set_image(None, img)
        if mid is not None:
            mid.record()
        solver.launch(b, use_graph=not args.no_graph)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    res0 = solver.result()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    mids = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    its, rels, stats = [], [], []
    with ClockSampler(dev.index) as clk:
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t_wall = time.perf_counter()
        for i in range(args.steps):
            flush.zero_()
            starts[i].record()
            step(mids[i])
            ends[i].record()
            r = solver.result(with_history=(i == args.steps - 1))
            its.append(r.iterations)
            rels.append(r.rel_res)
            stats.append(r.status)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        t_wall = time.perf_counter() - t_wall
    clocks = clk.summary()
    times = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    setup_ms = statistics.mean(s.elapsed_time(m) for s, m in zip(starts, mids))
    solve_ms = statistics.mean(m.elapsed_time(e) for m, e in zip(mids, ends))
    ms = max_over_ranks(statistics.mean(times), world, dev)
    last = r
    x_fused = last.x.clone()

    # ---- per-stage kernel times (roofline of the level-0 pre-block) ----
    reps = 20
    rbuf = torch.randn(n, device=dev)
    zbuf = torch.empty(n, device=dev)
    stage_ms = {}
    names = plan.stage_names()
    for s, name in enumerate(names):
        for _ in range(3):
            plan.apply_stages(s, s, rbuf, None, zbuf)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.zero_()
        e0.record()
        for _ in range(reps):
            plan.apply_stages(s, s, rbuf, None, zbuf)
        e1.record()
        torch.cuda.synchronize()
        stage_ms[name] = e0.elapsed_time(e1) / reps
    lc, ctas = plan.coarse_cluster()
    if lc > 0:
        # what the solve runs for levels lc..n: one cluster launch over their stages
        L_ = plan.levels
        for _ in range(3):
            plan.apply_stages(lc, 2 * L_ - lc, rbuf, None, zbuf)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.zero_()
        e0.record()
        for _ in range(reps):
            plan.apply_stages(lc, 2 * L_ - lc, rbuf, None, zbuf)
        e1.record()
        torch.cuda.synchronize()
        stage_ms[f"cluster{lc}-{L_}"] = e0.elapsed_time(e1) / reps
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    counts = [plan.class_counts(l) for l in range(plan.levels + 1)]
    gen = [c[0] for c in counts]
    mixed = [c[1] for c in counts]
    # coefficients, r in, y out, pooled out (+ the fluid mask)
    bytes_pre0 = coeff_bytes(plan, 0, n, mixed[0]) + n * (4 + 2 + 0.25 + (1 if plan.masked else 0))
    achieved = bytes_pre0 / (stage_ms["pre0"] * 1e-3) / 1e9
    traffic = None
    tp = ROOT / "profiles" / "traffic.json"
    if tp.exists():
        tj = json.loads(tp.read_text())
        if "pre0_bytes_per_cell" in tj:
            traffic = tj["pre0_bytes_per_cell"] * n
    roofline = {"kernel": f"k_pre_fused (level 0, {plan.layout} bf16 coefficients)", "bound": "hbm",
                "achieved": round(achieved, 1), "peak": hbm, "peak_source": peak_src, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "traffic": traffic,
                "algorithmic_bytes": bytes_pre0, "general_cells": gen, "mixed_runs": mixed}
    if not plan.spd and plan.kind != 2:
        # the level-0 post-block stage: prolongation pass (coarse in, u out; with swap also y in), then
        # the block (u in, y in without swap, z out, the fluid mask, the optional block mask)
        y_pass, y_block = (2, 0) if plan.swap else (0, 2)
        m_ = 1 if plan.masked else 0
        bytes_post0 = n * (2 / 8 + 4 + y_pass) + coeff_bytes(plan, 0, n, mixed[0]) + n * (4 + y_block + 4 + 1 + m_)
        a_post = bytes_post0 / (stage_ms["post0"] * 1e-3) / 1e9
        roofline["post0"] = {"kernels": "k_up_fine + k_post_fused (level 0)", "algorithmic_bytes": bytes_post0,
                             "ms": round(stage_ms["post0"], 4), "achieved": round(a_post, 1),
                             "frac": round(a_post / hbm, 4)}
    # whole-iteration bytes (compulsory traffic of the fused algorithm)
    mixed_t = [plan.class_counts_transposed(l)[1] for l in range(plan.levels + 1)] if plan.spd else None
    if plan.spd:
        roofline["mixed_runs_transposed"] = mixed_t
    per_iter_bytes = iteration_bytes(plan, n, mixed, mixed_t, args.method, solver.fused_dots())
    it_mean = statistics.mean(its)

    # ---- e2e: public API from pinned host buffers ----
    # the reference's interface: rhs and solution as fluid-DOF vectors (fluid cells in flat order)
    fluid_h = scene.flags.reshape(-1) == 2
    flags_h = torch.from_numpy(scene.flags).pin_memory()
    b_h = torch.from_numpy(np.ascontiguousarray(scene.rhs.reshape(-1)[fluid_h])).pin_memory()
    x_h = torch.empty(b_h.numel(), dtype=torch.float64).pin_memory()

    def e2e_step():
        solver.solve_host(flags_h, b_h, x_h, use_graph=not args.no_graph)

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    ee = []
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        e2e_step()
        e1.record()
        torch.cuda.synchronize()
        ee.append(e0.elapsed_time(e1))
    e2e = {"value": round(statistics.mean(ee), 3), "unit": "ms", "h2d_bytes_per_step": n + 8 * b_h.numel(),
           "d2h_bytes_per_step": 8 * x_h.numel(), "vectors": "fluid-DOF (the reference's compressed rhs / x)"}

    out = {"its": its, "rels": rels, "status": stats, "ms": ms, "times": times, "stage_ms": stage_ms,
           "dtype": "bf16",  # preconditioner coefficients and activations (CG vectors FP32, reductions FP64)
           "setup_ms": setup_ms, "solve_ms": solve_ms,
           "roofline": roofline, "clocks": clocks, "e2e": e2e, "meta": meta, "history": last.history.tolist(),
           "per_iter_bytes": per_iter_bytes, "launches": setup_launches(plan) + 2 +
           it_mean * (precond_launches(plan) + (5 if args.method == "npsd" else 4)), "x": x_fused, "scene": scene,
           "model": model,
           "flags": flags, "b": b, "wall": t_wall, "tuned": tuned}
    return out


def coeff_bytes(plan, level, n_level, mixed):
    """Coefficient bytes one block application reads at a level (bf16)."""
    if mixed is None or mixed < 0:
        return n_level * 27 * 2                          # dense planes
    tiles = math.ceil(n_level / (2 * 16 * 64))
    return n_level / 8 * 4 + mixed * 27 * 8 * 2 + tiles * 4   # run words, mixed-run records, tile offsets


def iteration_bytes(plan, n0, mixed, mixed_t=None, method="npsd", fused_dots=False):
    """Compulsory HBM bytes of one fused iteration (bf16 coefficients and activations; at level 0
    the input r, the prolongated input u, the output z and, for SPDSMModelDn3D, V's output v0 are
    FP32, and the fluid mask is read once per application; mirrors run_apply / run_apply_spd).
    fused_dots: the npsd products read only Ap1, Ap0 (z is in the post-block's registers)."""
    total = 0.0
    # solver vectors: npsd dots + qform + spmv/dots, or npcg r.z + p/spmv; then the update (r every
    # iteration, 12 B; the double-float iterate with two directions every other one, 24 B)
    dots = 8 if fused_dots else 12
    vec = n0 * (dots + 16 + 18 + 24) if method == "npsd" else n0 * (8 + 17 + 24)
    L = plan.levels
    if plan.kind == 2:   # V (prolongation pass on every level), then V^T
        for l in range(L):
            nl = n0 / 8 ** l
            f = 4 if l == 0 else 2                                       # r, u, v0 at level 0: FP32
            kf, kt = coeff_bytes(plan, l, nl, mixed[l]), coeff_bytes(plan, l, nl, mixed_t[l])
            total += kf + nl * (f + 2 + 2 / 8)                          # V pre: x in, y out, pooled
            total += nl * (2 / 8 + f) + kf + nl * (f + 2 + f)           # V up pass (u out); V post: u, y, out
            total += kt + nl * (f + 2 / 8)                              # V^T pre: w in, pooled (no y)
            total += nl * (2 / 8 + f + f)                               # V^T up pass: coarse, skip, u out
            total += kt + nl * (f + (4 + 1 if l == 0 else 2))           # V^T post: u in, out (+ fluid mask)
        nL = n0 / 8 ** L
        total += coeff_bytes(plan, L, nL, mixed[L]) + coeff_bytes(plan, L, nL, mixed_t[L]) + nL * 8
        return total + vec
    if plan.spd:
        for l in range(L):
            nl = n0 / 8 ** l
            f = 4 if l == 0 else 2
            total += coeff_bytes(plan, l, nl, mixed[l]) + nl * (f + 2 + 2 / 8)   # pre: as below
            # prolongation pass (coarse in, y in, u out), transposed block (u in, out; level 0: z + mask)
            total += nl * (2 / 8 + 2 + f) + coeff_bytes(plan, l, nl, mixed_t[l]) + nl * (f + (4 + 1 if l == 0 else 2))
        nL = n0 / 8 ** L
        total += coeff_bytes(plan, L, nL, mixed[L]) + coeff_bytes(plan, L, nL, mixed_t[L]) + nL * 8
        return total + vec
    m = 1 if plan.masked else 0
    for l in range(L):
        nl = n0 / 8 ** l
        kb = coeff_bytes(plan, l, nl, mixed[l])
        if l == 0:
            total += kb + nl * (4 + 2 + 2 / 8 + m)              # pre: coefficients, r in, y out, pooled out, mask
            # prolongation pass (coarse in, u out; with swap also y in), then the block (u in, y in
            # without swap, z out, the fluid mask and the optional block mask)
            y_pass, y_block = (2, 0) if plan.swap else (0, 2)
            total += nl * (2 / 8 + 4 + y_pass) + kb + nl * (4 + y_block + 4 + 1 + m)
        else:
            total += kb + nl * (2 + 2 + 2 / 8)                  # pre: coefficients, x in, y out, pooled out
            total += kb + nl * (2 / 8 + 2 + 2)                  # post: coefficients, coarse, y, out
    total += coeff_bytes(plan, L, n0 / 8 ** L, mixed[L]) + (n0 / 8 ** L) * (2 + 2)
    return total + vec


def reference_solution(flags, b, tol=1e-12, max_it=20000):
    """FP64 CG (matrix-free kernel, no preconditioner) to ||b - A x|| <= tol ||b||."""
    import torch
    from mlpcg_gb300.laplacian import FluidLaplacian
    A = FluidLaplacian(flags)
    b = torch.where(flags == 2, b, torch.zeros_like(b))
    x = torch.zeros_like(b)
    r = b.clone()
    p = r.clone()
    rr = torch.dot(r.view(-1), r.view(-1))
    nb = math.sqrt(float(rr))
    it = 0
    for it in range(1, max_it + 1):
        Ap = A.matvec_grid(p)
        alpha = rr / torch.dot(p.view(-1), Ap.view(-1))
        x += alpha * p
        r -= alpha * Ap
        rr_new = torch.dot(r.view(-1), r.view(-1))
        if it % 50 == 0:
            if math.sqrt(float(rr_new)) <= tol * nb:
                rt = b - A.matvec_grid(x)
                if float(rt.norm()) <= tol * nb:
                    break
        p = r + (rr_new / rr) * p
        rr = rr_new
    return x, it


def plain_solve(args, model, scene, dev):
    """The plain FP32 GPU drop-in: eval_forward per iteration, FP64 vectors, the drop-in solver."""
    import torch
    from mlpcg_gb300 import cg
    from mlpcg_gb300.laplacian import FluidLaplacian
    flags = torch.as_tensor(scene.flags, device=dev)
    A = FluidLaplacian(flags)
    img = torch.as_tensor(scene.image(), device=dev)
    b = torch.as_tensor(scene.rhs.ravel(), device=dev)[A.fluid_cells]
    solve = getattr(cg, args.method)
    pred = cg.model_predict(model, img, A.fluid_cells)
    solve(b, A, torch.zeros_like(b), pred, 2, tol=args.tol, atol=1e-20)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pred = cg.model_predict(model, img, A.fluid_cells)
    x, it, timer, res = solve(b, A, torch.zeros_like(b), pred, args.max_it, tol=args.tol, atol=1e-20)
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) * 1e3, it, res


# ----------------------------------------------------------------------------
def cpu_baseline(args, model_sd, scene, iterations, budget_s):
    """The reference's CPU path on this host: per-iteration time on a bounded sample."""
    import torch
    from oracle.cpu_path import CPUModel, CPUSPDFullModel, CPUSPDModel, npcg_iterations, npsd_iterations
    threads = torch.get_num_threads()
    cls = {"smallsm": CPUModel, "small_spd": CPUSPDModel, "spd": CPUSPDFullModel}[args.model]
    run = npcg_iterations if args.method == "npcg" else npsd_iterations
    m = cls(model_sd, args.levels)
    img = scene.image()
    # one iteration (includes the pyramid / c0 / c1 cache build) to size the sample
    t0 = time.perf_counter()
    times, _ = run(m, img, scene.flags, scene.rhs, 1)
    first = times[0]
    k = max(1, min(5, int(budget_s / max(first, 1e-3))))
    m2 = cls(model_sd, args.levels)
    times, hist = run(m2, img, scene.flags, scene.rhs, k + 1)
    per_it = statistics.mean(times[1:]) if len(times) > 1 else times[0]
    setup = times[0] - per_it
    total_ms = (setup + per_it * iterations) * 1e3
    return {"value": round(total_ms, 1), "unit": "ms", "cores": threads, "kind": "port",
            "sample": f"{len(times)} {args.method} iterations at {args.size}^3 (torch-CPU Conv3d blocks, "
                      f"{MODEL_NAMES[args.model]}, FP64 CSR), "
                      f"{per_it:.2f} s/iteration, extrapolated to {iterations} iterations",
            "host_cpus": os.cpu_count(), "per_iteration_s": round(per_it, 3)}


def amg_baseline(args, seed):
    """The reference's other host comparator -- AMG-preconditioned CG (cg_tests.py:343-346 with
    cxx_src/lib/AMGCLSolver.h:58-128) -- as restated by oracle/amg.cpp, run to the same tolerance on
    the same scene in a child process on the host cores (its memory and threads stay out of this
    process).  Setup + solve time, measured; the matrix assembly is not timed."""
    cmd = [sys.executable, "-m", "oracle.amg", "--size", str(args.size), "--seed", str(seed),
           "--spheres", str(args.spheres), "--tol", str(args.tol)]
    try:
        p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=args.amg_timeout)
    except subprocess.TimeoutExpired:
        return {"unavailable": f"no result within {args.amg_timeout:.0f} s"}
    if p.returncode != 0:
        tail = (p.stderr.strip().splitlines() or ["no output"])[-1]
        return {"unavailable": f"exit {p.returncode}: {tail[:200]}"}
    try:
        return json.loads(p.stdout.strip().splitlines()[-1])
    except (IndexError, ValueError):
        return {"unavailable": "no JSON line"}


BATCH_SIZES = [64] * 4 + [96] * 4 + [128] * 4 + [192] * 4
BATCH_SEEDS = list(range(100, 116))


def run_batch(args):
    """16 systems of uneven sizes (3 spheres each, seeds 100-115; 4 levels up to 96^3, 5 from 128^3),
    BF16 preconditioner, npsd to 1e-6, solved by one graph launch of a BatchSolver (every system a
    parallel branch, per-system convergence masks).  Timed like the single solve (device time of
    the launch with the plans set up, L2 flushed between steps); the same 16 systems solved one after
    the other by the plain FP32 drop-in are timed once."""
    import torch
    from mlpcg_gb300.scenes import make_scene
    from mlpcg_gb300.solver import BatchSolver, FusedSolver, flags_to_image
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    solvers, rhs, scenes, models, metas = [], [], [], [], []
    for size, seed in zip(BATCH_SIZES, BATCH_SEEDS):
        a = argparse.Namespace(**vars(args))
        a.levels = 4 if size < 128 else 5
        a.size = size
        m, meta = load_model(a, dev)
        sc = make_scene(size, seed, 3)
        flags = torch.as_tensor(sc.flags, device=dev)
        solvers.append(FusedSolver(m, flags, method="npsd", max_it=args.max_it, tol=args.tol,
                                   storage=torch.bfloat16, image=flags_to_image(flags)))
        rhs.append(torch.as_tensor(sc.rhs, device=dev))
        scenes.append(sc)
        models.append((m, a))
        metas.append(meta.get("weights"))
    batch = BatchSolver(solvers)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(max(1, args.warmup)):
        batch.solve(rhs)
    torch.cuda.synchronize()
    times = []
    with ClockSampler(dev.index) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            batch.launch(rhs)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
    res = [s.result(with_history=False) for s in solvers]
    # the same systems one by one through the fused solver, and through the plain drop-in
    seq = []
    for s, b in zip(solvers, rhs):
        s.solve(b)
    torch.cuda.synchronize()
    for s, b in zip(solvers, rhs):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        s.launch(b)
        e1.record()
        torch.cuda.synchronize()
        seq.append(e0.elapsed_time(e1))
    plain = []
    for (m, a), sc in zip(models, scenes):
        a.method = "npsd"
        pm, pit, pres = plain_solve(a, m, sc, dev)
        plain.append({"ms": round(pm, 2), "iterations": pit, "rel_res": pres})
    ms = statistics.mean(times)
    systems = [{"size": sz, "seed": sd, "levels": 4 if sz < 128 else 5, "iterations": r.iterations,
                "status": r.status, "rel_res": r.rel_res, "fused_alone_ms": round(t, 3)}
               for sz, sd, r, t in zip(BATCH_SIZES, BATCH_SEEDS, res, seq)]
    plain_total = sum(p["ms"] for p in plain)
    return {"metric": "ms to 1e-6 rel. residual, 16 uneven systems in one graph launch (BF16 fused npsd) "
                      "vs 16 sequential plain FP32 solves, 1 GB300",
            "value": round(ms, 3), "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16", "data": "synthetic",
            "config": {"workload": "16 scenes, seeds 100-115, 4 x 64^3, 4 x 96^3 (4 levels), 4 x 128^3, "
                                   "4 x 192^3 (5 levels), 3 spheres each, npsd to 1e-6, one BatchSolver launch",
                       "weights": sorted(set(w for w in metas if w)),
                       "l2": "L2 flushed (256 MiB write) between steps"},
            "systems": systems, "sequential_fused_ms": round(sum(seq), 3),
            "plain_sequential_ms": round(plain_total, 2), "plain": plain,
            "speedup_vs_plain_sequential": round(plain_total / ms, 2),
            "all_converged": all(r.status == "converged" for r in res), "clocks": clk.summary(),
            "gpu_launches": None}


def reference_arm(args, world, cfg):
    """The reference's CPU path (torch-CPU blocks composed as the network, FP64 CSR npsd / npcg,
    model_predict's FP32 round trip) run to convergence on this host's cores: one warm-up iteration,
    then one measured solve to the same tolerance and iteration limit as the GPU arm (the
    reference's protocol times npsd's 'Total' clock, test.py:327-331; its two warm-up solves would
    add minutes here).  The solve's own iteration count and final FP64 relative residual (b - A x
    recomputed every iteration) are reported beside the time."""
    import torch
    from mlpcg_gb300.scenes import make_scene
    from oracle.cpu_path import CPUModel, CPUSPDFullModel, CPUSPDModel, npcg_iterations, npsd_iterations
    model, meta = load_model(args, "cpu")
    sd = model.state_dict()
    scene = make_scene(args.size, args.seed, args.spheres)
    cls = {"smallsm": CPUModel, "small_spd": CPUSPDModel, "spd": CPUSPDFullModel}[args.model]
    run = npcg_iterations if args.method == "npcg" else npsd_iterations
    img = scene.image()
    run(cls(sd, args.levels), img, scene.flags, scene.rhs, 1)          # warm-up iteration
    times, hist = run(cls(sd, args.levels), img, scene.flags, scene.rhs, args.max_it, tol=args.tol)
    total_ms = sum(times) * 1e3
    its = len(times)
    per_it = statistics.mean(times[1:]) if its > 1 else times[0]
    cfg = dict(cfg, weights=meta.get("weights"))
    cb = {"value": round(total_ms, 1), "unit": "ms", "cores": torch.get_num_threads(), "kind": "port",
          "sample": f"one {args.method} solve at {args.size}^3 to {args.tol:g} (torch-CPU Conv3d blocks, "
                    f"{MODEL_NAMES[args.model]}, FP64 CSR), run to convergence: {its} iterations, "
                    f"{per_it:.2f} s/iteration after the first",
          "host_cpus": os.cpu_count(), "per_iteration_s": round(per_it, 3), "measured": True}
    return {"impl": "reference", "metric": METRIC, "value": round(total_ms, 1), "unit": "ms",
            "n_gpus": world, "steps": 1, "warmup": 1, "ms_per_step": round(total_ms, 1),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg, "iterations": its,
            "status": "converged" if (hist[-1] < args.tol) else "max_it", "rel_res": hist[-1],
            "history": [round(h, 9) for h in hist], "cpu_baseline": cb,
            "steps_note": "one converged solve (the full CPU solve takes tens of seconds); warm-up = one iteration",
            "e2e": {"value": round(total_ms, 1), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def reference_iterations(meta, args):
    key = f"{args.method}_iterations_{args.size}_seed{args.seed}"
    return int(meta.get(key, args.max_it))


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", 1))
    rank = int(os.environ.get("RANK", 0))
    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl" if args.impl == "ours" else "gloo")
    cfg = {"workload": f"single {args.size}^3 scene (seed {args.seed}, {args.spheres} spheres), "
                       f"{args.levels}-level {MODEL_NAMES[args.model]}, {args.method} to {args.tol:g} FP64 true rel. "
                       f"residual",
           "grid": args.size, "levels": args.levels, "model": MODEL_NAMES[args.model], "method": args.method,
           "max_it": args.max_it,
           "precision": "bf16 coefficients+activations, fp32 CG vectors, fp64 x/b/reductions/true residual",
           "l2": "inputs larger than L2; L2 flushed (256 MiB write) between steps",
           "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        line = reference_arm(args, world, cfg)
        print(json.dumps(line))
        return

    if args.batch:
        if rank == 0:
            print(json.dumps(run_batch(args)))
        return
    r = run_ours(args, rank, world)
    if rank != 0:
        return
    import torch
    dev = r["x"].device
    extra = {}
    if not args.no_reference_solution:
        xr, itr = reference_solution(r["flags"], r["b"])
        fl = r["flags"] == 2
        err = float((r["x"][fl] - xr[fl]).norm() / xr[fl].norm())
        extra["err_vs_fp64_cg"] = err
        extra["fp64_cg_iterations"] = itr
    if not args.no_plain:
        pm, pit, pres = plain_solve(args, r["model"], r["scene"], dev)
        extra.update({"plain_ms": round(pm, 2), "plain_iterations": pit, "plain_rel_res": pres,
                      "speedup_vs_plain": round(pm / r["ms"], 2)})
    cpu = None
    if not args.no_cpu:
        cpu = cpu_baseline(args, r["model"].state_dict(), r["scene"], int(statistics.mean(r["its"])),
                           args.cpu_seconds)
        if not args.no_amg:
            extra["amg_cpu_baseline"] = amg_baseline(args, replica_seed(args.seed, 0))
    it_mean = statistics.mean(r["its"])
    line = {"metric": METRIC, "value": round(r["ms"], 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(r["ms"], 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": r["dtype"], "data": "synthetic",
            "config": dict(cfg, weights=r["meta"].get("weights"),
                           solver_schedule=r["tuned"] or "default (8 CTAs per SM)"),
            "iterations": it_mean, "status": r["status"][-1], "rel_res": r["rels"][-1],
            "history": [round(h, 9) for h in r["history"]],
            "per_iteration_hbm_bytes": r["per_iter_bytes"],
            "setup_ms": round(r["setup_ms"], 3), "solve_ms": round(r["solve_ms"], 3),
            "stages_ms": {k: round(v, 4) for k, v in r["stage_ms"].items()},
            "roofline": r["roofline"], "cpu_baseline": cpu, "e2e": r["e2e"], "clocks": r["clocks"],
            "gpu_launches": int(r["launches"] * args.steps)}
    line.update(extra)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
