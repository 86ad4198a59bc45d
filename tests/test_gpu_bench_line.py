"""bench.py's own arm on the GPU at the small case (Ns=40, M=400): the one JSON line it
prints carries the benchmark contract's keys with consistent values -- the roofline of
the memory integrals against the measured copy peak, the end-to-end rate through the C
ABI with host buffers, the launch count, the sampled clocks and the tuning it ran."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_our_arm_line_at_the_small_case():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--config", "small", "--steps", "5",
                        "--warmup", "3", "--no-cpu", "--no-fp64"], cwd=ROOT, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "roofline", "e2e", "gpu_launches", "clocks",
                "tuning"):
        assert key in line, key
    assert line["unit"] == "steps/s" and line["higher_is_better"] is True and line["n_gpus"] == 1
    assert line["steps"] == 5 and line["warmup"] == 3 and line["value"] > 0
    assert abs(line["value"] * line["ms_per_step"] / 1000.0 - 1.0) < 1e-6
    rf = line["roofline"]
    assert rf["bound"] == "hbm" and rf["unit"] == "GB/s" and rf["peak"] > 0
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-9
    # algorithmic bytes of the Ns = 40, M = 400 step: 2 [M(M+1)/2] S 4 + 2 M S 4 + 2 M S 4, S = 1771
    assert rf["algorithmic_bytes"] == 2 * (400 * 401 // 2) * 1771 * 4 + 4 * 400 * 1771 * 4
    assert 0.0 < rf["frac"] < 1.3
    e2e = line["e2e"]
    assert e2e["unit"] == "steps/s" and e2e["value"] > 0
    assert e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    assert line["gpu_launches"] >= 3 * line["steps"]
    assert line["clocks"]["sm_max_mhz"] > 0
    assert line["tuning"]["source"] == "kb_autotune"
    assert line.get("batched_64_runs") is None  # measured beside the Ns=64, M=1000 workload only
