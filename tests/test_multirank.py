"""bench.py's multi-process path on CPU (gloo, world size 2, 127.0.0.1):
the barrier and the max-over-ranks / sum-over-ranks reductions that turn the
ranks' timings into one whole-job number, and the reference arm under torchrun
(rank 0 alone replays and prints; the other rank exits 0 without work)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    ws, r, _, dist = bench.dist_setup()
    bench.barrier(dist)
    secs = bench.reduce_max(dist, 1.0 + rank)          # rank 1 is the slowest
    commits = bench.reduce_sum(dist, 1000.0 * (rank + 1))
    bench.barrier(dist)
    with open(os.path.join(out, f"r{rank}.json"), "w") as f:
        json.dump({"ws": ws, "rank": r, "secs": secs, "commits": commits}, f)
    dist.destroy_process_group()


def test_reductions_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    got = [json.load(open(tmp_path / f"r{r}.json")) for r in range(2)]
    for g in got:
        assert g["ws"] == 2
        assert g["secs"] == 2.0          # max over ranks
        assert g["commits"] == 3000.0    # sum over ranks: value = 3000 / 2.0 on every rank
    assert [g["rank"] for g in got] == [0, 1]


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--workload", "ycsb_small", "--steps", "3", "--warmup", "1",
           "--no-reference-gpu"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, timeout=580)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]  # rank 0 only
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 3
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["cores"] >= 1
