"""The multi-GPU form of bench.py on CPU: one replica per rank, and no
data-path collective.  Two gloo ranks with different step times must agree
on the slowest one (the job's time), and the job's rate must count both
replicas' units over it.  The reference arm under several ranks runs on rank
0 alone; the others exit without work.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

import bench

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out_dir: str):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank  # rank 1 is the slow replica
        slowest = bench.max_over_ranks(ms, dist, "cpu")
        rate = bench.job_rate(world, 1000.0, slowest * 1e-3)
        Path(out_dir, f"rank{rank}.json").write_text(json.dumps({"slowest": slowest, "rate": rate}))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_and_count_both_replicas(tmp_path):
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    got = [json.loads(Path(tmp_path, f"rank{r}.json").read_text()) for r in range(world)]
    for g in got:
        assert g["slowest"] == 15.0
        assert abs(g["rate"] - 2 * 1000.0 / 15e-3) < 1e-6


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(7.5) == 7.5
    assert bench.job_rate(1, 300.0, 2.0) == 150.0


def test_reference_arm_on_a_second_rank_exits_without_work():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "3"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
