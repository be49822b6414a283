"""Training of SmallSMModelDn3D (the reference's train.py) or of the symmetric SmallSPDSMModelDn3D
(train_one_scene.py:176) / SPDSMModelDn3D through the hand-written adjoint kernels.

Loss (per right-hand side b of unit norm, x = f(b) restricted to fluid cells):
  * ``angle`` (default): 1 - cos^2(b, A x), the squared relative residual at
    the best output scale (npsd / npcg do not see the scale of M);
  * ``squared``: ||b - A x||^2 / ||b||^2, averaged over the batch;
  * ``reference``: ||b - A x|| averaged over the batch (residual_loss,
    loss_functions.py:18-23).
Right-hand sides: random combinations of the lowest Lanczos Ritz vectors of
each scene (lanczos.py), plus a fraction of white noise on the fluid cells so
that the high-frequency end of the spectrum is seen as well.  Optimiser:
Adam (train.py:219 of the reference uses lr 1e-4 over far more steps; a
cosine schedule from a larger lr is used here).

    python -m mlpcg_gb300.train --out DIR --size 128 --levels 5 --seeds 10-17 --steps 4000
    python -m mlpcg_gb300.train --out DIR --model small_spd ...   (validated with npcg)
"""
from __future__ import annotations

import argparse
import json
import math
import time
from pathlib import Path

import numpy as np
import torch

from . import ops
from .laplacian import FluidLaplacian
from .lanczos import lanczos_ritz, mix_rhs
from .scenes import make_scene
from .sm_model_3d import SmallSMModelDn3D, SmallSPDSMModelDn3D, SPDSMModelDn3D, set_training_storage

MODELS = {"smallsm": "smallsm", "small_spd": "smallspd", "spd": "spd"}   # --model -> weight file prefix


def make_model(kind, levels):
    if kind == "small_spd":
        return SmallSPDSMModelDn3D(levels)
    if kind == "spd":
        return SPDSMModelDn3D(levels)
    return SmallSMModelDn3D(levels, 3, "trilinear")


def solve_method(model):
    """npcg for the symmetric networks (textbook PCG is valid), npsd otherwise."""
    return "npcg" if isinstance(model, (SmallSPDSMModelDn3D, SPDSMModelDn3D)) else "npsd"
from .solver import FusedSolver, flags_to_image


class LaplacianFunction(torch.autograd.Function):
    """y = A x for a batch of full-grid F32 fields; A is symmetric, so the adjoint is A again."""

    @staticmethod
    def forward(ctx, flags, x):
        ctx.flags = flags
        return _lap_batch(flags, x)

    @staticmethod
    def backward(ctx, g):
        return None, _lap_batch(ctx.flags, g.contiguous())


def _lap_batch(flags, x):
    shp = x.shape
    xb = x.reshape(-1, *flags.shape).contiguous()
    out = torch.stack([ops.laplacian(flags, xb[i]) for i in range(xb.shape[0])])
    return out.reshape(shp)


def residual_loss(model, image, flags, fluid, b, kind="angle"):
    """b: (B, N1, N2, N3) unit-norm on fluid cells, zero elsewhere.

    kind = "squared":   ||b - A x||^2 / ||b||^2
           "reference": ||b - A x||  (residual_loss, loss_functions.py:18-23)
           "angle":     min_s ||b - s A x||^2 / ||b||^2 = 1 - cos^2(b, A x): the
                        squared relative residual at the best scale of the output,
                        in [0, 1]; invariant to the scale of the network output,
                        like npsd and npcg are.
    """
    x = model(image, b[:, None])[:, 0]
    return loss_of_outputs(x * fluid, b, flags, kind)


def loss_of_outputs(x, b, flags, kind="angle"):
    """The loss of network outputs x (B, N1, N2, N3; zero off the fluid cells) for right-hand sides b
    (same shape): see residual_loss.  kind="reference" is loss_functions.py:18-23 with mean=True,
    the mean over the batch of ||b - A x||."""
    Ax = LaplacianFunction.apply(flags, x)
    bf, Af = b.flatten(1), Ax.flatten(1)
    if kind == "angle":
        num = (Af * bf).sum(1).pow(2)
        den = Af.pow(2).sum(1) * bf.pow(2).sum(1)
        return (1.0 - num / den.clamp_min(1e-30)).mean()
    r = bf - Af
    if kind == "reference":
        return r.norm(dim=1).mean()
    return (r.pow(2).sum(1) / bf.pow(2).sum(1)).mean()


def near_identity_(model, eps=0.1):
    """Shrink the random weights by eps and add z = x on the direct path (M ~ I at start; for the
    symmetric network M = S^T S ~ I with S ~ I on the finest level)."""
    with torch.no_grad():
        for p in model.parameters():
            p.mul_(eps)
        first = model.l0[0] if isinstance(model, (SmallSPDSMModelDn3D, SPDSMModelDn3D)) else model.pre[0]
        first.bias[13] += 1.0
        model.c0[0].bias[0] += 1.0


class TrainScene:
    def __init__(self, shape, seed, device, n_ritz=64, lanczos_steps=1600, spheres=3, cache_dir=None):
        s = make_scene(shape, seed, spheres)
        self.seed = seed
        self.flags = torch.as_tensor(s.flags, device=device)
        self.image = flags_to_image(self.flags)
        self.fluid = (self.flags == 2).float()
        self.A = FluidLaplacian(self.flags)
        self.rhs = torch.as_tensor(s.rhs, device=device)
        v0 = self.rhs.reshape(-1)[self.A.fluid_cells]
        t = time.time()
        shp = "x".join(str(d) for d in self.flags.shape)
        cache = Path(cache_dir) / f"ritz_{shp}_s{seed}_k{n_ritz}_m{lanczos_steps}.pt" if cache_dir else None
        if cache is not None and cache.exists():
            d = torch.load(cache, map_location=device)
            self.ritz_vals, ritz = d["vals"].cpu().numpy(), d["vecs"]
        else:
            self.ritz_vals, ritz = lanczos_ritz(self.A, v0, lanczos_steps, n_ritz)
            ritz = ritz.float()
            if cache is not None:
                cache.parent.mkdir(parents=True, exist_ok=True)
                torch.save({"vals": torch.as_tensor(self.ritz_vals), "vecs": ritz}, cache)
        self.lanczos_s = time.time() - t
        self.ritz = ritz.float()
        self.n = self.flags.numel()

        self.harvested = []       # residuals met by npsd with the current network (fluid cells, unit norm)
        self.plan = None
        self.solvers = {}

    def batch(self, B, noise_frac, gen, harvest_frac=0.0):
        nh = min(int(round(B * harvest_frac)), len(self.harvested) and B)
        nb = int(round(B * noise_frac))
        nr = max(B - nb - nh, 0)
        parts = []
        if nr > 0:
            parts.append(mix_rhs(self.ritz, nr, generator=gen))
        if nb > 0:
            w = torch.randn((nb, self.A.n_fluid), device=self.ritz.device, generator=gen)
            parts.append(w / w.norm(dim=1, keepdim=True))
        if nh > 0:
            idx = torch.randint(len(self.harvested), (nh,), generator=gen, device=self.ritz.device).tolist()
            parts.append(torch.stack([self.harvested[i] for i in idx]))
        bf = torch.cat(parts)
        b = torch.zeros((bf.shape[0], self.n), dtype=torch.float32, device=bf.device)
        b[:, self.A.fluid_cells] = bf
        return b.reshape(bf.shape[0], *self.flags.shape)

    def harvest(self, model, gen, depths=(2, 5, 10, 20), keep=48):
        """Residuals after a few fused npsd iterations with the current network, from a random rhs."""
        from .precond import PrecondPlan
        if self.plan is None:
            self.plan = PrecondPlan(model, self.image)
            for d in depths:
                self.solvers[d] = FusedSolver(model, self.flags, method=solve_method(model), max_it=d,
                                              tol=1e-12, plan=self.plan)
        else:
            next(iter(self.solvers.values())).set_image(model, self.image)
        b0 = self.batch(1, 0.5, gen)[0].double()
        for d, s in self.solvers.items():
            res = s.solve(b0)
            r = (b0 - self.A.matvec_grid(res.x)).reshape(-1)[self.A.fluid_cells].float()
            nrm = r.norm()
            if torch.isfinite(nrm) and nrm > 0:
                self.harvested.append(r / nrm)
        self.harvested = self.harvested[-keep:]


class Validator:
    """npsd (npcg for the symmetric network) iterations to 1e-6 on a held-out scene (one solver,
    re-planned with the current weights)."""

    def __init__(self, model, size, seed, spheres, device, max_it=200, tol=1e-6):
        s = make_scene(size, seed, spheres)
        self.flags = torch.as_tensor(s.flags, device=device)
        self.rhs = torch.as_tensor(s.rhs, device=device)
        self.image = flags_to_image(self.flags)
        self.solver = FusedSolver(model, self.flags, method=solve_method(model), max_it=max_it, tol=tol,
                                  image=self.image)

    def __call__(self, model):
        self.solver.set_image(model, self.image)
        r = self.solver.solve(self.rhs)
        return r.iterations, r.status, r.rel_res


def parse_seeds(s):
    if "-" in s:
        a, b = s.split("-")
        return list(range(int(a), int(b) + 1))
    return [int(t) for t in s.split(",")]


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--model", default="smallsm", choices=sorted(MODELS))
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--levels", type=int, default=5)
    ap.add_argument("--seeds", default="10-17")
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--lr-min", type=float, default=1e-4)
    ap.add_argument("--noise-frac", type=float, default=0.25)
    ap.add_argument("--loss", default="angle", choices=["angle", "squared", "reference"])
    ap.add_argument("--init-mode", default="near-identity", choices=["near-identity", "reference"])
    ap.add_argument("--init-eps", type=float, default=0.1)
    ap.add_argument("--lanczos-steps", type=int, default=1600)
    ap.add_argument("--n-ritz", type=int, default=64)
    ap.add_argument("--eval-every", type=int, default=500)
    ap.add_argument("--val-size", type=int, default=256)
    ap.add_argument("--val-seed", type=int, default=19)
    ap.add_argument("--val-spheres", type=int, default=6)
    ap.add_argument("--harvest-every", type=int, default=250, help="0 disables solver-in-the-loop rhs")
    ap.add_argument("--harvest-frac", type=float, default=0.25)
    ap.add_argument("--init", default=None, help="npz state dict to start from")
    ap.add_argument("--storage", default="fp32", choices=["fp32", "bf16"],
                    help="block storage in training: BF16 coefficient planes and saved inputs, FP32 sums")
    ap.add_argument("--recompute", action="store_true",
                    help="recompute per-level activations in the backward pass (large grids, SmallSMModelDn3D)")
    ap.add_argument("--time-limit", type=float, default=1e9, help="seconds of training loop at most")
    ap.add_argument("--ritz-cache", default=None, help="directory caching the Lanczos Ritz vectors")
    args = ap.parse_args(argv)

    dev = torch.device("cuda")
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    torch.manual_seed(0)
    model = make_model(args.model, args.levels).to(dev)
    if args.recompute:
        model.recompute = True
    if args.storage == "bf16":
        set_training_storage(model, torch.bfloat16)
    if args.init:
        d = np.load(args.init)
        model.load_state_dict({k: torch.from_numpy(d[k]) for k in model.state_dict()})
    elif args.init_mode == "near-identity":
        near_identity_(model, args.init_eps)
    t0 = time.time()
    scenes = [TrainScene(args.size, s, dev, args.n_ritz, args.lanczos_steps, cache_dir=args.ritz_cache)
              for s in parse_seeds(args.seeds)]
    val = Validator(model, args.val_size, args.val_seed, args.val_spheres, dev)
    prep_s = time.time() - t0
    print(f"prepared {len(scenes)} scenes in {prep_s:.1f}s (lanczos {[round(s.lanczos_s, 1) for s in scenes]})",
          flush=True)

    opt = torch.optim.Adam(model.parameters(), lr=args.lr)
    gen = torch.Generator(device=dev)
    gen.manual_seed(1234)
    log = {"loss": [], "eval": [], "args": vars(args), "prep_s": prep_s}
    it0, st0, rel0 = val(model)
    log["eval"].append({"step": 0, "iterations": it0, "status": st0, "rel_res": rel0})
    best = (it0 if st0 == "converged" else 10 ** 9, rel0)
    save(model, out, args, log, best=True)
    print(f"step 0 eval: {it0} its ({st0}, {rel0:.2e})", flush=True)
    t_train = time.time()
    ema = None
    step = 0
    for step in range(1, args.steps + 1):
        lr = args.lr_min + 0.5 * (args.lr - args.lr_min) * (1 + math.cos(math.pi * (step - 1) / args.steps))
        for g in opt.param_groups:
            g["lr"] = lr
        if args.harvest_every and (step - 1) % args.harvest_every == 0:
            with torch.no_grad():
                for sc in scenes:
                    sc.harvest(model, gen)
        sc = scenes[(step - 1) % len(scenes)]
        b = sc.batch(args.batch, args.noise_frac, gen, args.harvest_frac if args.harvest_every else 0.0)
        loss = residual_loss(model, sc.image, sc.flags, sc.fluid, b, args.loss)
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
        lv = float(loss.detach())
        ema = lv if ema is None else 0.98 * ema + 0.02 * lv
        if step % 50 == 0:
            log["loss"].append({"step": step, "loss": lv, "ema": ema, "lr": lr})
            print(f"step {step} loss {lv:.4e} ema {ema:.4e} lr {lr:.2e} ({time.time() - t_train:.0f}s)", flush=True)
        if step % args.eval_every == 0 or step == args.steps:
            it, st, rel = val(model)
            log["eval"].append({"step": step, "iterations": it, "status": st, "rel_res": rel})
            score = (it if st == "converged" else 10 ** 9, rel)
            is_best = score < best
            if is_best:
                best = score
            print(f"step {step} eval: {it} its ({st}, {rel:.2e}){' best' if is_best else ''}", flush=True)
            save(model, out, args, log, best=is_best)
        if time.time() - t_train > args.time_limit:
            print(f"time limit reached at step {step}", flush=True)
            break
    log["train_s"] = time.time() - t_train
    log["steps_done"] = step
    log["peak_device_gb"] = round(torch.cuda.max_memory_allocated(dev) / 1e9, 3)
    log["best"] = {"iterations": best[0], "rel_res": best[1]}
    save(model, out, args, log, best=False)


def save(model, out: Path, args, log, best: bool):
    """The best weights so far (by validation iterations) go to <prefix>_l{n}.npz (prefix smallsm or
    smallspd), the latest to *.last.npz."""
    sd = {k: v.detach().float().cpu().numpy() for k, v in model.state_dict().items()}
    stem = f"{MODELS[getattr(args, 'model', 'smallsm')]}_l{args.levels}"
    if best:
        np.savez(out / f"{stem}.npz", **sd)
    np.savez(out / f"{stem}.last.npz", **sd)
    (out / f"{stem}.train.json").write_text(json.dumps(log, indent=1))


if __name__ == "__main__":
    main()
