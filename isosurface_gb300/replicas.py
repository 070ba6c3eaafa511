"""Multi-GPU layout of the extraction path: independent replicas.

Extraction of one volume is a single pass over one GPU's memory with no
exchange step, so N GPUs run N independent extractions (one process per GPU,
each on its own volume or its own share of a chunk batch). The only
cross-rank traffic is on the host side of a measurement: a barrier around the
timed region and a max over ranks of the per-rank time. These helpers hold
that logic so it can be exercised with the ``gloo`` backend on CPU.
"""
import os


def rank_env():
    """(world, rank, local_rank) from the torchrun environment (1, 0, 0 when absent)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend="nccl"):
    """Join the process group when launched with WORLD_SIZE > 1; returns the
    ``torch.distributed`` module or None for a single process."""
    world, _, _ = rank_env()
    if world <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend)
    return dist


def max_over_ranks(x, dist, device="cpu"):
    """Largest value of ``x`` over all ranks (``x`` itself without a group).
    ``device`` is where the reduction tensor lives: "cuda" for NCCL, "cpu" for gloo."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard(n_units, rank, world):
    """Half-open range [lo, hi) of ``n_units`` independent units (chunks,
    volumes) owned by ``rank``: contiguous, sizes differing by at most one."""
    base, extra = divmod(n_units, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def whole_job_rate(units_per_rank, world, seconds_max):
    """Throughput of the whole job: every rank's units over the slowest rank's time."""
    return world * units_per_rank / seconds_max
