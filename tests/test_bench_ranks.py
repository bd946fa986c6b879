"""bench.py's multi-process handling, on CPU with the gloo backend.

The path does not shard (replicas only): each rank times its own replica and
rank 0 reports the whole job from the slowest rank's time; under torchrun the
reference arm runs on rank 0 alone while the other ranks exit without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(1.5 + rank, "cpu")  # each rank's own step time
        with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
            json.dump({"rank": rank, "max": got}, f)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gives_every_rank_the_slowest_time(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    got = [json.load(open(tmp_path / f"r{r}.json")) for r in range(world)]
    assert [g["max"] for g in got] == [1.5 + world - 1] * world


def test_max_over_ranks_without_a_process_group_is_the_value():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.25, "cpu") == 3.25


@pytest.mark.parametrize("rank", [1, 3])
def test_reference_arm_other_ranks_exit_without_work(rank):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="4", LOCAL_RANK=str(rank))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_reference_arm_prints_the_contract_line():
    """Rank 0 (or a single process) times the oracle on the headline workload
    and prints one JSON line keyed like the repository arm's, with a CPU
    baseline record and an end-to-end figure that moves no bytes."""
    sys.path.insert(0, ROOT)
    import bench

    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["config"]["workload"] == bench.CONFIG["workload"]
    assert d["unit"] == "queries/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["value"] > 0 and abs(d["ms_per_step"] - 16000.0 / d["value"]) < 1e-6 * d["ms_per_step"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
