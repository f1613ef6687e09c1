"""Multi-rank host logic on CPU (gloo, world size 2).

The pipeline does not shard within a pair, so `bench.py --gpus N` runs N
replicas: each rank processes its own pairs and the process group only aligns
the timed regions and takes the slowest rank's time. These tests run that
logic as two gloo processes, and the reference arm under torchrun, where rank
0 alone measures and prints."""

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


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # Each rank's own time; every rank must see the slowest one.
        local = 10.0 + 5.0 * rank
        got = bench.max_over_ranks(local, dist)
        shard = bench.shard_pairs(rank, 5, distinct=16)
        dist.barrier()
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as fh:
            json.dump({"max": got, "shard": shard}, fh)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_shards_with_gloo(tmp_path):
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    assert [r["max"] for r in res] == [15.0, 15.0]
    assert res[0]["shard"] == [0, 1, 2, 3, 4]
    assert res[1]["shard"] == [5, 6, 7, 8, 9]


def test_max_over_ranks_without_a_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.shard_pairs(3, 4, distinct=16) == [12, 13, 14, 15]
    assert bench.shard_pairs(1, 20, distinct=16)[:6] == [4, 5, 6, 7, 8, 9]


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_prints_once(tmp_path):
    """`bench.py --impl reference` launched as two ranks: rank 0 times the CPU
    restatement of the reference and prints one JSON line; rank 1 exits 0
    without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    env = dict(os.environ)
    env["OMP_NUM_THREADS"] = "1"
    r = subprocess.run(cmd, cwd=str(tmp_path), capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["unit"] == "pairs/s"
    assert line["cpu_baseline"]["kind"] == "port"
