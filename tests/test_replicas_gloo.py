"""Multi-rank replica logic on CPU with the gloo backend (world size 2)."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from fullwave25_gb300.replicas import aggregate_throughput, rank_instances

    ids = rank_instances(rank, world, 3)
    # rank r processed 10 * (r + 1) units in (r + 1) seconds
    total, tmax, value = aggregate_throughput(10.0 * (rank + 1), float(rank + 1))
    gathered = [None] * world
    dist.all_gather_object(gathered, ids)
    out.put((rank, ids, total, tmax, value, gathered))
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_and_own_disjoint_instances():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ids, total, tmax, value, gathered in res:
        assert total == 30.0 and tmax == 2.0 and value == 15.0
        assert ids == [rank * 3 + i for i in range(3)]
        assert set(gathered[0]).isdisjoint(gathered[1])


def test_single_process_aggregate_is_local():
    from fullwave25_gb300.replicas import aggregate_throughput, rank_instances

    assert aggregate_throughput(12.0, 3.0) == (12.0, 3.0, 4.0)
    with pytest.raises(ValueError):
        rank_instances(2, 2, 1)
