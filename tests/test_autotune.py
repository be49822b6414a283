"""Schedule autotuner: candidate sets, choice and JSON cache (CPU); applying a schedule to a
real solver (GPU)."""
import json

import pytest

from mlpcg_gb300 import autotune


def test_candidates_and_pick():
    assert autotune.candidates(152) == [152, 304, 456, 608, 912, 1216]
    assert autotune.candidates(1000) == [1000]
    assert autotune.candidates(2000) == [1216]
    assert autotune.pick_best({152: 3.0, 304: 2.0, 608: 2.0}) == 304
    assert autotune.schedule_key("NVIDIA GB300", (256, 256, 256), "npsd") == "NVIDIA GB300|256x256x256|npsd"


def test_cache_round_trip(tmp_path):
    p = tmp_path / "sub" / "tune.json"
    assert autotune.load_cache(p) == {}
    autotune.save_cache({"k": {"blocks": 304}}, p)
    assert autotune.load_cache(p) == {"k": {"blocks": 304}}
    p.write_text("not json")
    assert autotune.load_cache(p) == {}


@pytest.mark.gpu
def test_tune_solver_applies_and_caches(cuda, tmp_path):
    import torch
    from mlpcg_gb300.scenes import make_scene
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D
    from mlpcg_gb300.solver import FusedSolver
    s = make_scene((64, 64, 64), 3)
    torch.manual_seed(0)
    m = SmallSMModelDn3D(3, 3, "trilinear").to(cuda)
    with torch.no_grad():
        for p in m.parameters():
            p.mul_(0.0)
        m.pre[0].bias[13] += 1.0
        m.c0[0].bias[0] += 1.0
    solver = FusedSolver(m, torch.as_tensor(s.flags, device=cuda), method="npcg", max_it=400, tol=1e-6,
                         storage=torch.float32)
    b = torch.as_tensor(s.rhs, device=cuda)
    ref = solver.solve(b)
    seen = []
    cache = tmp_path / "tune.json"
    best = autotune.tune_solver(solver, b, cache_path=cache,
                                measure=lambda sv, nb: (seen.append(nb), abs(nb - 456))[1])
    n_sm = torch.cuda.get_device_properties(cuda).multi_processor_count
    assert seen == autotune.candidates(n_sm) and best == min(seen, key=lambda nb: abs(nb - 456))
    assert autotune.get_schedule(solver) == min(best, 128)  # 64^3: at most 128 CTAs of 512 groups
    res = solver.solve(b)
    assert res.status == "converged" and abs(res.iterations - ref.iterations) <= 2
    # the cached choice is applied without timing
    key = autotune.schedule_key(torch.cuda.get_device_properties(cuda).name, solver.shape, "npcg")
    assert json.loads(cache.read_text())[key]["blocks"] == best
    assert autotune.tune_solver(solver, b, cache_path=cache, measure=lambda *a: 1 / 0) == best
    # the real timing path runs too
    assert autotune.tune_solver(solver, b, cache_path=cache, retune=True, reps=1) in autotune.candidates(n_sm)


def test_plan_candidates_and_key():
    assert autotune.plan_candidates(False) == [(0, 0), (1, 0), (2, 0), (4, 0), (8, 0)]
    assert autotune.plan_candidates(True)[-2:] == [(0, 1), (2, 1)]
    assert autotune.plan_key("NVIDIA GB300", (256, 256, 256), 5, "bfloat16", "npsd") == \
        "plan|NVIDIA GB300|256x256x256|L5|bfloat16|npsd"


@pytest.mark.gpu
def test_tune_plan_applies_caches_and_keeps_results(cuda, tmp_path):
    """Every block schedule gives the same solve bit for bit; the chosen one is applied and cached."""
    import torch
    from mlpcg_gb300.scenes import make_scene
    from mlpcg_gb300.sm_model_3d import SmallSMModelDn3D
    from mlpcg_gb300.solver import FusedSolver
    s = make_scene((128, 128, 128), 3)
    torch.manual_seed(0)
    m = SmallSMModelDn3D(4, 3, "trilinear").to(cuda)
    with torch.no_grad():
        for p in m.parameters():
            p.mul_(0.05)
        m.pre[0].bias[13] += 1.0
        m.c0[0].bias[0] += 1.0
    solver = FusedSolver(m, torch.as_tensor(s.flags, device=cuda), method="npsd", max_it=40, tol=1e-6)
    b = torch.as_tensor(s.rhs, device=cuda)
    ref = solver.solve(b)
    xref = ref.x.clone()
    seen = []

    def measure(sv, choice):
        r = sv.solve(b)
        assert r.iterations == ref.iterations and torch.equal(r.x, xref), choice
        seen.append(choice)
        return 1.0 if choice == (1, 0) else 2.0

    cache = tmp_path / "plan.json"
    best = autotune.tune_plan(solver, b, cache_path=cache, measure=measure)
    assert best == (1, 0) and (2, 0) in seen and (0, 0) in seen
    assert autotune.tune_plan(solver, b, cache_path=cache, measure=lambda *a: 1 / 0) == best
    r = solver.solve(b)
    assert torch.equal(r.x, xref)
