"""bench.py's reference arm (the reference's CPU path on the host cores, run to convergence) prints
exactly one JSON line with the benchmark contract's keys; run at 32^3 on the CPU so that it takes
seconds."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line():
    cmd = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--size", "32", "--levels", "3",
           "--cpu-seconds", "1", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["higher_is_better"] is False
    assert isinstance(d["metric"], str) and d["unit"] == "ms" and d["value"] > 0
    assert d["ms_per_step"] == d["value"] and d["data"] == "synthetic" and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["unit"] == "ms"
    assert cb["value"] == d["value"] and "solve at 32^3" in cb["sample"] and cb["measured"] is True
    # a run to convergence (or to max_it), not an extrapolation: its own count and final residual
    assert d["iterations"] == len(d["history"]) and d["rel_res"] == pytest.approx(d["history"][-1], rel=1e-6)
    assert d["status"] in ("converged", "max_it")
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == "ms"
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_amg_comparator_leg_reports_a_measured_solve():
    """The host AMG comparator beside the CPU baseline: a measured solve of the same scene to the
    bench's tolerance, or an 'unavailable' reason when it does not finish in time."""
    import argparse
    sys.path.insert(0, str(ROOT))
    import bench
    a = argparse.Namespace(size=24, spheres=3, tol=1e-6, amg_timeout=240.0)
    d = bench.amg_baseline(a, bench.replica_seed(7, 0))
    assert d["kind"] == "port" and d["unit"] == "ms" and d["value"] > 0 and d["cores"] >= 1
    assert d["rel_res"] < 1e-6 and 0 < d["iterations"] < 50
    assert d["value"] == pytest.approx(d["setup_ms"] + d["solve_ms"], abs=0.2)
    a.amg_timeout = 1e-3
    assert "unavailable" in bench.amg_baseline(a, 7)
