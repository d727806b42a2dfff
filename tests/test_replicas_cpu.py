"""The multi-GPU path is replicas only: each rank steps its own grid and the
ranks share nothing but bench.py's barrier and the max-over-ranks time
(gloo).  Checked here with world size 2 on CPU processes."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys
sys.path.insert(0, sys.argv[1])
import bench
rank, local, world = bench.rank_info()
assert world == 2
d = bench.Dist(world)
d.barrier()
# Each rank reports its own elapsed time; every rank must see the maximum.
t = d.max(1.5 if rank == 0 else 4.25)
assert t == 4.25, t
# The job's throughput counts the units of every rank over that time.
cells, steps = 64 ** 3, 10
value = cells * steps * world / t
assert abs(value - 2 * 64 ** 3 * 10 / 4.25) < 1e-6
d.barrier()
d.close()
print("rank", rank, "ok")
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replica_ranks_share_only_barrier_and_max():
    pytest.importorskip("torch.distributed")
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.STDOUT, text=True))
    outs = []
    for p in procs:
        try:
            out, _ = p.communicate(timeout=240)
        except subprocess.TimeoutExpired:
            p.kill()
            out, _ = p.communicate()
        outs.append(out)
    for rank, (p, out) in enumerate(zip(procs, outs)):
        assert p.returncode == 0, out
        assert f"rank {rank} ok" in out


def test_reference_arm_other_ranks_exit_without_work():
    # Under torchrun only rank 0 times the CPU path and prints; others exit 0.
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=240)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
