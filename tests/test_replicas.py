"""Multi-rank path of bench.py (replicas only): the whole-job figure sums the units of all
ranks and divides by the slowest rank's time; ranks must agree on the count.  Runs as two
gloo ranks on the CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, counts, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 100.0 * (rank + 1)
    units = 1000 * (rank + 1)
    res = bench.replica_throughput(units, ms, counts[rank], dist, "cpu")
    q.put((rank, res))
    dist.barrier()
    dist.destroy_process_group()


def _run(counts):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, counts, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    return out


def test_two_replicas_sum_units_and_take_slowest_time():
    out = _run([12345678901, 12345678901])
    for rank in (0, 1):
        total, worst, value, same = out[rank]
        assert total == 3000 and worst == 200.0 and same
        assert value == pytest.approx(3000 / 0.2)


def test_two_replicas_detect_disagreeing_counts():
    out = _run([7, 8])
    assert not out[0][3] and not out[1][3]


def test_single_process_path():
    import bench
    assert bench.replica_throughput(500, 250.0, 3) == (500, 250.0, 2000.0, True)
