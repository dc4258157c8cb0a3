"""Multi-rank path of bench.py: the count is sharded, each rank counting one part of the
same graph (atc_tc_part) and the parts summed over the ranks.  The whole-job figure
counts the graph's units once over the slowest rank's time.  Runs as two gloo ranks on
the CPU, with a stand-in for the library's part count (no GPU here)."""
import os
import socket
import types

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class _FakeStats:
    kernel_ms = 1.0
    launches = 3


def _fake_atc(part_counts):
    """Stand-in for the binding: part p of n counts part_counts[p] (n must match)."""
    def tc_part(csr, part, nparts, kernel, stream=None):
        assert nparts == len(part_counts) and 0 <= part < nparts
        return part_counts[part], (part, part + 1), _FakeStats()

    def tc(csr, kernel, stream=None):
        return sum(part_counts), _FakeStats()

    return types.SimpleNamespace(tc_part=tc_part, tc=tc)


def _worker(rank, world, port, part_counts, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    res = bench.sharded_throughput(3000, 100.0 * (rank + 1), part_counts[rank], dist, "cpu")
    total, _ = bench.count_step(_fake_atc(part_counts), None, 0, rank, world, None, dist, "cpu")
    q.put((rank, (res, total)))
    dist.barrier()
    dist.destroy_process_group()


def _run(part_counts):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    world = len(part_counts)
    ps = [ctx.Process(target=_worker, args=(r, world, port, part_counts, q)) for r in range(world)]
    for p in ps:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(world))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    return out


def test_two_shards_count_units_once_take_slowest_time_and_sum_parts():
    parts = [12345678901, 987654321]
    out = _run(parts)
    for rank in (0, 1):
        (units, worst, value, total), step_total = out[rank]
        assert units == 3000 and worst == 200.0
        assert value == pytest.approx(3000 / 0.2)
        assert total == sum(parts) and step_total == sum(parts)


def test_single_process_path():
    import bench
    assert bench.sharded_throughput(500, 250.0, 3) == (500, 250.0, 2000.0, 3)
    total, st = bench.count_step(_fake_atc([5, 6]), None, 0, 0, 1, None)
    assert total == 11 and st.launches == 3
