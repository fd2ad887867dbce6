"""bench.py with more than one rank, on the CPU: two gloo ranks (the way
torchrun starts them, rendezvous on 127.0.0.1) take the job's time as the
slowest rank's, and the reference arm's other ranks leave without work or
output.  Each rank steps its own replica of the workload, so the data path
itself has no exchange to test."""
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench._dist() == (world, rank, rank)
        # rank r timed 10 + r ms: every rank reports the slowest
        out[rank] = bench._max_over_ranks(10.0 + rank, world, device="cpu")
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        assert dict(out) == {0: 11.0, 1: 11.0}


def test_reference_arm_other_ranks_leave_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "2", "--warmup", "3"], env=env, capture_output=True, text=True,
                       timeout=120, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
