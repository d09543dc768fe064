"""bench.py's multi-rank plumbing on the CPU (no GPU): two gloo ranks on
127.0.0.1 through the same helpers the GPU arm uses (barrier, max and sum over
ranks), and the reference arm launched as torch.distributed.run launches it
for N = 2 (rank 0 prints the one line, rank 1 exits 0 without work)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2",
                      RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    world, r, local, dist = bench.dist_setup(None)
    bench.barrier(dist)
    res = {"world": world, "rank": r, "local": local,
           "max": bench.max_over_ranks(dist, float(10 * (rank + 1))),
           "sum": bench.sum_over_ranks(dist, float(rank + 1))}
    bench.barrier(dist)
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)


def test_two_gloo_ranks_reduce_like_the_bench(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    for rank in range(2):
        res = json.load(open(tmp_path / f"rank{rank}.json"))
        assert res["world"] == 2 and res["rank"] == rank and res["local"] == rank
        assert res["max"] == 20.0  # the slowest rank's time is the job's
        assert res["sum"] == 3.0   # units of all ranks add up


def test_reference_arm_under_two_rank_launch():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node",
           "2", "--master-addr", "127.0.0.1", "--master-port", str(port),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["value"] == line["value"]
