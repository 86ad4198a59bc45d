"""bench.py's reference arm (the CPU oracle port on the host cores) at a tiny
lattice: the one JSON line it prints carries every key of the benchmark
contract, and fewer than three warm-up steps are refused."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*extra):
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *extra],
                          cwd=ROOT, capture_output=True, text=True, timeout=600)


def test_reference_arm_line():
    r = _run("--ns", "8", "--m", "20", "--steps", "1", "--warmup", "3")
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "steps/s" and line["higher_is_better"] is True
    assert line["steps"] == 1 and line["warmup"] == 3 and line["vs_baseline"] is None
    assert "Ns=8" in line["config"]["workload"] and "M=20" in line["config"]["workload"]
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert "Ns=8" in cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_too_few_warmup_steps_are_refused():
    r = _run("--ns", "8", "--m", "20", "--steps", "1", "--warmup", "2")
    assert r.returncode != 0
    assert "warm-up" in r.stderr
