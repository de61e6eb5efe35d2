"""Replicas across ranks for the multi-GPU runs of the hot path.

The path has no exchange step between GPUs at the sizes here (one box has one GPU, and a row-band decomposition
is not built), so N GPUs run N independent replicas of the workload, one process per GPU. What the ranks share
is only the measurement: a barrier before and after the timed region, the maximum of the ranks' times, and the
whole-job throughput = the units all ranks processed / that maximum. No collective touches the data path.
"""
import os


def rank_info():
    """(rank, world_size, local_rank) from the launcher's environment (torchrun), (0, 1, 0) when absent."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(world: int, backend: str):
    """The process group of a multi-rank run, or None for one rank. MASTER_ADDR/MASTER_PORT come from the
    launcher (127.0.0.1 on these boxes)."""
    if world <= 1:
        return None
    import torch.distributed as dist

    if not dist.is_initialized():
        dist.init_process_group(backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(value: float, dist, device: str = "cpu") -> float:
    """The maximum of `value` over all ranks (every rank gets it)."""
    if dist is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, elapsed_ms: float) -> float:
    """Units per second of the whole job: every rank processed `units_per_rank` in at most `elapsed_ms`."""
    return units_per_rank * world / (elapsed_ms / 1e3)


def finish(dist):
    if dist is not None:
        dist.destroy_process_group()
