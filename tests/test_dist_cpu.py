"""The N>1 path of bench.py on CPU: two gloo ranks (replicas only: the only
collectives are the barrier and the max-over-ranks of the timed region), and
the reference arm under torchrun, where rank 0 alone runs and prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out_dir):
    os.environ.update(WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), KB_BENCH_GLOO="1")
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    ws, r, local = bench.dist_setup()
    bench.barrier(ws)
    v = bench.max_over_ranks(ws, 10.0 * (rank + 1))
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"ws": ws, "rank": r, "local": local, "max": v}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_barrier_and_max(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = free_port()
    mp.start_processes(_rank_main, args=(port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    for rank in range(2):
        d = json.load(open(tmp_path / f"rank{rank}.json"))
        assert d == {"ws": 2, "rank": rank, "local": rank, "max": 20.0}
    assert torch is not None


def test_reference_arm_under_torchrun_prints_once():
    pytest.importorskip("torch")
    from oracle.pyoracle import build_oracle

    build_oracle()
    env = dict(os.environ, KB_BENCH_GLOO="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3", "--cpu-window", "8"]
    p = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
