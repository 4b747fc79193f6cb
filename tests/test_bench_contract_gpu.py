"""The benchmark's one-line JSON contract, on small cases of each workload:
the keys and types every line carries (metric, value, e2e through the host
entry point, roofline, CPU baseline, clocks, kernel launch count), and that
the numbers are consistent with each other. Runs bench.py as a user does,
in a child process."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def bench_line(*args):
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def check_common(d, steps, warmup):
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "clocks", "gpu_launches"):
        assert k in d, k
    assert d["n_gpus"] == 1 and d["steps"] == steps and d["warmup"] == warmup
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["higher_is_better"] is True
    assert "workload" in d["config"]
    e = d["e2e"]
    assert e["value"] > 0 and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert r["achieved"] > 0 and r["peak"] > 0 and abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-3
    c = d["clocks"]
    assert "sm_mhz" in c and "sm_max_mhz" in c and isinstance(c["reasons"], list)
    assert d["gpu_launches"] > 0


def test_suite_line():
    d = bench_line("--only", "star3d2r:float32,box3d1r:float64", "--n", "96", "--T", "6", "--steps", "1",
                   "--warmup", "3", "--cpu-budget", "0.5")
    check_common(d, 1, 3)
    cb = d["cpu_baseline"]
    assert cb["value"] > 0 and cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    # every timed grid is checked against the oracle within the stated bound
    for p in d["per_stencil"]:
        bound = 1e-5 if p["dtype"] == "float32" else 1e-12
        assert p["max_err_vs_oracle"] is not None and p["max_err_vs_oracle"] <= bound
    assert d["gpu_launches"] >= sum(p["launches"] for p in d["per_stencil"])


def test_batched_line():
    d = bench_line("--workload", "batched", "--batch-grids", "24", "--batch-tmax", "24", "--steps", "1",
                   "--warmup", "3", "--no-cpu")
    check_common(d, 1, 3)
    assert d["batched_vs_plain"]["ratio"] > 0
    assert d["config"]["batch_mode"] == "layered" and d["gpu_launches"] == d["config"]["graph_kernels"]


def test_adjoint_line():
    d = bench_line("--workload", "adjoint", "--only", "j2d5pt:float32", "--T", "64", "--steps", "1", "--warmup",
                   "3", "--no-cpu")
    check_common(d, 1, 3)
    (case,) = d["adjoint"]
    assert case["backward_ms"] > 0 and case["forward_ms"] > 0 and case["coef_grad"] is True
