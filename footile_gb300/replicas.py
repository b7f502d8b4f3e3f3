"""Multi-GPU host logic: paths are independent, so ranks work on separate path
sets (no collective on the data path).  Weak scaling gives every rank its own batch;
`shard` splits one batch when the total is fixed.  Reductions use torch.distributed
when a process group is initialised (NCCL on GPUs, gloo on CPUs) and are identities
otherwise."""


def shard(n, rank, world):
    """Contiguous slice of n paths owned by `rank` of `world` (a partition of range(n))."""
    return range(rank * n // world, (rank + 1) * n // world)


def _dist():
    try:
        import torch.distributed as dist
        return dist if dist.is_available() and dist.is_initialized() else None
    except Exception:
        return None


def _reduce(x, op_name, device):
    dist = _dist()
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def reduce_max(x, device="cpu"):
    """Max over ranks (the slowest rank's time bounds the job)."""
    return _reduce(x, "MAX", device)


def reduce_sum(x, device="cpu"):
    """Sum over ranks (pixels or paths processed by the whole job)."""
    return _reduce(x, "SUM", device)


def barrier():
    dist = _dist()
    if dist is not None:
        dist.barrier()
