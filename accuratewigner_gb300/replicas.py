"""Whole-job throughput of independent replicas, one per GPU (no reference counterpart).

A single propagator grid is never split across GPUs (the largest, a 4096^2 density matrix with
its 8192^2 Wigner grid, fits one GPU), and batches and served requests are independent, so
several GPUs run replicas: every rank advances its own instances with no collective on the data
path.  The only exchange is this bookkeeping after the timed region: the slowest rank's time and
the sum of the work units, over any torch.distributed process group (NCCL on the GPU machine, gloo
in the CPU tests).
"""


def job_throughput(seconds, units, group=None, device=None):
    """(max seconds over ranks, total units over ranks, units / second) of a weak-scaling run."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return seconds, units, units / seconds
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    sec, tot = float(t.item()), float(u.item())
    return sec, tot, tot / sec
