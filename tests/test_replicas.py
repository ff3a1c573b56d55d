"""Multi-GPU runs are replicas (no data-path collective): bench.py's only collective is the
max-over-ranks timing reduction, and the whole-job value is the sum over replicas.  Checked
here with world_size-2 gloo process groups on the CPU."""

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, values, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.max_over_ranks(values[rank])
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("values", [(3.5, 7.25), (9.0, 1.0)])
def test_max_over_ranks_with_two_gloo_ranks(values):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    assert out[0] == out[1] == max(values)


def test_single_process_needs_no_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(2.5) == 2.5


def test_replica_throughput_is_the_sum_over_replicas():
    sys.path.insert(0, str(ROOT))
    import bench

    # 4 replicas of 100k particles x 50 steps, the slowest taking 5 ms: 4e9 particle-steps/s
    assert bench.replica_throughput(100_000 * 50, 5.0, 4) == pytest.approx(4e9)
    assert bench.replica_throughput(100_000 * 50, 5.0, 1) == pytest.approx(1e9)
