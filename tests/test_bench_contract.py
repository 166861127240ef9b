"""Host checks of bench.py's contract that need no GPU: the reference arm's
JSON line on a tiny workload (the CPU oracle, every host thread), its silence
on ranks other than 0, and the launch bookkeeping behind `gpu_launches`."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TINY = ["--impl", "reference", "--size", "65", "--angles", "24", "--slices", "4", "--steps", "2", "--warmup", "1"]


def run_bench(extra_env=None, wall=None):
    import time
    env = dict(os.environ, **(extra_env or {}))
    t0 = time.perf_counter()
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *TINY], env=env, capture_output=True,
                       text=True, timeout=600, cwd=ROOT)
    if wall is not None:
        wall.append(time.perf_counter() - t0)
    assert r.returncode == 0, r.stderr[-2000:]
    return [l for l in r.stdout.splitlines() if l.startswith("{")]


def test_reference_arm_line(oracle):
    wall = []
    lines = run_bench(wall=wall)
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["unit"] == "slices/s" and d["value"] > 0
    assert d["steps"] == 2 and d["warmup"] == 1 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    # the steps are measured, not modelled: their time fits inside the run
    assert d["steps"] * d["ms_per_step"] / 1000.0 < wall[0]
    # slices/s of the full reconstruction from the measured CG step
    assert abs(d["value"] * 50 * 12 * d["ms_per_step"] / 1000.0 - 1.0) < 1e-9


def test_cpu_baseline_times_a_full_outer_iteration(oracle):
    sys.path.insert(0, ROOT)
    import bench
    v, cores, desc, t_warm, t_outer = bench.cpu_outer_iteration(65, 24)
    assert v > 0 and cores >= 1 and t_warm > 0 and t_outer > 0
    assert abs(v * (t_warm + 50 * t_outer) - 1.0) < 1e-9
    assert "nouter=1" in desc


def test_reference_arm_other_ranks_print_nothing(oracle):
    assert run_bench({"RANK": "1", "WORLD_SIZE": "2"}) == []


def test_launch_bookkeeping():
    sys.path.insert(0, ROOT)
    import bench
    # automatic projector choice (ACU_OPT_PROJECTOR = 7): pixel lines when the
    # 4-slice groups fill their 8-group lines to 8/9 or more
    assert bench.projector_variant(7, 256) == 6
    assert bench.projector_variant(7, 32) == 6
    assert bench.projector_variant(7, 36) == 5      # 9 groups in two lines
    assert bench.projector_variant(7, 4) == 5
    assert bench.projector_variant(5, 256) == 5
    # 2049^2: bands of 126 rows -> 17 band launches plus conversion and finish
    assert bench.radon_launches(6, 2049) == 19
    assert bench.radon_launches(5, 2049) == 2
    assert bench.radon_launches(6, 65) == 3
