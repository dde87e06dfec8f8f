"""bench.py at N > 1 runs independent replicas (the path does not shard): the
job's throughput is N x per-rank work over the slowest rank's time.  Checked with
two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as td
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    td.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = 100.0 * (rank + 1)          # rank 1 is the slow one
    value, ms = bench.replica_throughput(local_ms, units_per_rank=50, world=world)
    out.put((rank, value, ms))
    td.destroy_process_group()


def test_replica_throughput_uses_slowest_rank():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    results = sorted(q.get(timeout=10) for _ in range(world))
    for rank, value, ms in results:
        assert ms == pytest.approx(200.0)
        assert value == pytest.approx(2 * 50 / 0.2)


def test_single_rank_is_local():
    import bench
    value, ms = bench.replica_throughput(250.0, 100, 1)
    assert ms == 250.0 and value == pytest.approx(400.0)
