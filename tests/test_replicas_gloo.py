"""CPU: the multi-GPU path of bench.py (replicas only) on two gloo ranks.

The solve does not shard (no exchange on the solve path), so N GPUs run N
independent replicas; bench.py takes the slowest replica's time (maximum
over ranks) and reports N x steps / that time.  Two CPU processes with the
gloo backend check the aggregation (no GPU).
"""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r took (r + 1) seconds for 3 steps, wall (r + 2) seconds
    total, wall = bench.max_over_ranks([rank + 1.0, rank + 2.0], dist, torch.device("cpu"))
    value = bench.replica_throughput(world, 3, total)
    out[rank] = (total, wall, value)
    dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        total, wall, value = out[r]
        assert total == 2.0 and wall == 3.0
        assert value == 2 * 3 / 2.0


def test_single_rank_is_identity():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks([1.5, 2.5], None, None) == [1.5, 2.5]
    assert bench.replica_throughput(1, 4, 2.0) == 2.0
