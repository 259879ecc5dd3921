"""Replica bookkeeping for multi-GPU runs: one process per GPU, independent simulations per rank.

The engine does not shard a single solve (one GB300 holds every benchmark configuration); across
GPUs it runs independent replicas: rank r owns simulations ``r * n_per_rank + i``. Throughput is
the cell-updates of all ranks divided by the slowest rank's time (weak scaling), with no
collective on the data path: only these two scalars are reduced once, after the timed region.
"""

from __future__ import annotations


def rank_instances(rank: int, world: int, n_per_rank: int) -> list:
    """Simulation ids owned by ``rank`` (disjoint across ranks, seeds of the batched workload)."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    return [rank * n_per_rank + i for i in range(n_per_rank)]


def aggregate_throughput(units: float, seconds: float, group=None) -> tuple:
    """Whole-job throughput: (sum of units over ranks) / (max of seconds over ranks).

    Returns ``(units_total, seconds_max, units_total / seconds_max)``. With ``group`` None or a
    single rank the local values are used.
    """
    import torch  # noqa: PLC0415
    import torch.distributed as dist  # noqa: PLC0415

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
        u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
        t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
        dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
        dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
        units, seconds = float(u.item()), float(t.item())
    return units, seconds, units / seconds
