"""Replica runs on several GPUs of one node.

Fragmentation jobs are independent, so the path shards by job and needs no
collective on the data path: every rank runs its whole workload on its own GPU
(weak scaling).  The only exchange is host-side bookkeeping over gloo: a
barrier before the timed region and the maximum of the ranks' timings after
it, so that whole-job throughput is (units processed by all ranks) / (slowest
rank's time).
"""
import os


def world() -> int:
    return int(os.environ.get("WORLD_SIZE", "1"))


def rank() -> int:
    return int(os.environ.get("RANK", "0"))


def init() -> int:
    """Joins the gloo process group when WORLD_SIZE > 1 (rendezvous from
    MASTER_ADDR / MASTER_PORT); returns the world size."""
    n = world()
    if n > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("gloo")
    return n


def barrier() -> None:
    if world() > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float) -> float:
    """The maximum of x over all ranks (x itself on one rank)."""
    if world() <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, ms_per_rank: float) -> float:
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    ms = max_over_ranks(ms_per_rank)
    return units_per_rank * world() / (ms / 1000.0) if ms > 0 else 0.0


def finalize() -> None:
    if world() > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()
