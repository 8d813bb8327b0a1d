"""The multi-rank path of bench.py on CPU ranks (gloo, world size 2).

Records shard across ranks with no data-path collective; the only
collectives are the barrier around the timed region and the max-reduce of
the step time over ranks.  These run here on two gloo processes; the GPU arm
itself needs a GPU per rank.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    r, w, local, dist = bench.dist_setup(world)
    assert (r, w, local) == (rank, world, rank) and dist is not None
    assert dist.get_backend() == "gloo"
    bench.barrier(dist)
    step_ms = 10.0 * (rank + 1)  # rank 1 is the slow one
    worst = bench.reduce_max(dist, step_ms)
    bench.barrier(dist)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"worst": worst}, f)
    dist.destroy_process_group()


def test_barrier_and_max_over_ranks(tmp_path):
    port = _free_port()
    torch.multiprocessing.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for rank in range(2):
        got = json.load(open(tmp_path / f"rank{rank}.json"))
        assert got["worst"] == 20.0  # every rank reports the slowest rank's time


def test_reference_arm_under_torchrun_prints_one_line():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--workload", "line", "--gpus", "2", "--steps", "1", "--warmup", "1",
           "--cpu-seconds", "0.5", "--records", "2000"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["metric"] == "GCUPS" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
