"""The multi-GPU form of the benchmark is replicas only: every rank runs independent
chains (its own Philox key) and the ranks meet once, to combine the timed work. Tested on
CPU with two gloo ranks (127.0.0.1): the whole-job value is the work summed over ranks
divided by the slowest rank's time, identical on both ranks; keys differ per rank; the
reference arm's non-zero ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    work = [1000.0, 3000.0][rank]
    seconds = [2.0, 5.0][rank]
    value, w, s = bench.aggregate(torch, dist, work, seconds, "cpu")
    out[rank] = (value, w, s, bench.rank_seed(rank))
    dist.barrier()
    dist.destroy_process_group()


def test_aggregate_over_two_gloo_ranks():
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
    assert out[0][:3] == out[1][:3] == (4000.0 / 5.0, 4000.0, 5.0)
    assert out[0][3] != out[1][3]


def test_single_process_aggregate():
    assert bench.aggregate(torch, None, 600.0, 3.0, "cpu") == (200.0, 600.0, 3.0)


def test_reference_arm_nonzero_rank_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0 and r.stdout.strip() == ""
