"""Host side of bench.py's multi-GPU path on CPU (gloo, world size 2): the
path runs independent replicas, so ranks only meet at barriers and at the
max-over-ranks of the timed region; the reference arm runs on rank 0 alone."""
import importlib
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    assert bench._dist() == (world, rank, rank)
    bench._barrier(world)
    # Each rank's timed region; the job's time is the slowest rank's.
    out[rank] = bench._barrier_max(10.0 + 5.0 * rank, world)
    dist.destroy_process_group()


def test_barrier_and_max_over_ranks():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
        assert dict(out) == {0: 15.0, 1: 15.0}


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    assert bench._barrier_max(3.5, 1) == 3.5
    bench._barrier(1)
    assert not dist.is_initialized()


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
