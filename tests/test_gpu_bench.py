"""The bench's JSON line on small cases: required keys present and the
figures consistent with each other (value, ms per step, gradients/s,
roofline fraction)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bench(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                         capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-2000:]
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_cube_line():
    d = bench("--n", "48", "--steps", "5", "--warmup", "3", "--no-cpu-baseline", "--no-variants",
              "--no-serving")
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "roofline", "e2e", "clocks", "gpu_launches"):
        assert key in d, key
    cells = 48 ** 3
    assert d["value"] == pytest.approx(cells / (d["ms_per_step"] / 1e3) / 1e9, rel=1e-3)
    r = d["roofline"]
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"], rel=1e-3)
    assert r["achieved"] == pytest.approx(r["alg_bytes_per_launch"] / (r["launch_ms"] / 1e3) / 1e9,
                                          rel=1e-2)
    assert d["e2e"]["h2d_bytes_per_step"] >= 0 and d["e2e"]["value"] > 0
    assert d["gpu_launches"] > 0


@pytest.mark.parametrize("segment,passes", [(0, 2), (45, 3)])
def test_design_line(segment, passes):
    """Recorded history (forward + adjoint) and √N checkpoints (forward,
    recompute, adjoint): the line counts the passes that ran."""
    d = bench("--workload", "design2d", "--n", "160", "--batch", "2", "--steps", "1",
              "--warmup", "1", "--no-cpu-baseline", "--segment", str(segment))
    per = d["forward_s"] + d["backward_s"]
    assert d["ms_per_step"] == pytest.approx(per * 1e3, rel=1e-3)
    assert d["gradients_per_s"] == pytest.approx(2 / per, rel=1e-3)
    cells, steps = 160 * 160, d["config"]["time_steps"]
    assert d["value"] == pytest.approx(passes * cells * steps * 2 / per / 1e9, rel=1e-3)
    assert (d["config"]["checkpoints"] == 0) == (passes == 2)
    assert d["grad_finite"] and d["gpu_launches"] > 0


def test_serving_line():
    """A small serving run: batched against one at a time, latencies, and the
    measured batching bound, consistent with each other."""
    d = bench("--workload", "serving", "--jobs", "6", "--size-scale", "0.3",
              "--max-job-steps", "300")
    sv = d["serving"]
    assert sv["failed"] == 0 and d["value"] == sv["batched_gcells"] > 0
    assert sv["latency_p99_s"] >= sv["latency_p50_s"] > 0
    assert sv["speedup"] == pytest.approx(sv["batched_gcells"] / sv["one_at_a_time_gcells"],
                                          rel=2e-3)
    assert sv["bound"] > 0
    assert sv["speedup_over_bound"] == pytest.approx(sv["speedup"] / sv["bound"], rel=5e-3)
