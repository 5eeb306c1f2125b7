"""The multi-GPU form of the benchmark: replicas only (independent scenes shard trivially; the step
has no exchange between GPUs).  Two gloo ranks on the CPU check the cross-rank part of bench.py: the
timed region is the slowest rank's, and the whole-job value counts every rank's bodies over it."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        own_ms = 100.0 + 25.0 * rank                     # rank 1 is the slow one
        slowest = bench.max_over_ranks(own_ms, dist)
        dist.barrier()
        q.put((rank, slowest))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    assert got == [(0, 125.0), (1, 125.0)]


def test_replica_value_counts_every_rank():
    # 501,361 bodies per replica, 20 steps, slowest rank 200 ms: one replica's rate times the replicas
    one = bench.replica_value(501361, 20, 1, 200.0)
    assert one == pytest.approx(501361 * 20 / 0.2)
    assert bench.replica_value(501361, 20, 4, 200.0) == pytest.approx(4 * one)


def test_roofline_traffic_reads_the_committed_launch_list():
    # roofline.traffic and phases_dram_bytes_ncu come from the committed ncu summary of one batched step
    for phase in ("integrate", "broadphase", "narrowphase", "solver"):
        v = bench.ncu_traffic(phase)
        assert v is not None and v > 0, phase
    assert bench.ncu_traffic("narrowphase") > bench.ncu_traffic("solver") > bench.ncu_traffic("integrate")
