"""Several GPUs: one process per GPU, each with its own handle and a contiguous
range of the slices.

Slices are independent, so the only exchange is the host-side collection of
results (the reference's tests/test_gpus_many.py:58-85 runs one thread per GPU
on disjoint slice ranges and writes into one host array).  There is no
collective on the data path; `gather_slices` and `max_over_ranks` are the
host-side steps of a sharded run (result collection and the timing
reduction), over whatever torch.distributed backend is initialised (NCCL on
GPUs, gloo on CPU).
"""
import numpy as np


def slice_range(S, world, rank):
    """Contiguous [start, stop) of S slices for `rank` of `world`; sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside world of %d" % (rank, world))
    base, extra = divmod(int(S), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(value, device=None):
    """Largest `value` over all ranks (the job's time is its slowest rank's)."""
    dist = _dist()
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_slices(local, S, dst=0):
    """Collect every rank's slice range of a [S, ...] result on rank `dst`.

    `local` is this rank's [stop - start, ...] host array (slice_range order).
    Returns the full [S, ...] array on `dst` and None elsewhere."""
    dist = _dist()
    local = np.ascontiguousarray(local)
    if dist is None:
        return local
    import torch
    world, rank = dist.get_world_size(), dist.get_rank()
    shape = local.shape[1:]
    n_max = max(b - a for a, b in (slice_range(S, world, r) for r in range(world)))
    buf = torch.zeros((n_max,) + shape, dtype=torch.from_numpy(local[:0]).dtype)
    buf[:local.shape[0]] = torch.from_numpy(local)
    parts = [torch.zeros_like(buf) for _ in range(world)] if rank == dst else None
    dist.gather(buf, parts, dst=dst)
    if rank != dst:
        return None
    out = np.empty((S,) + shape, dtype=local.dtype)
    for r in range(world):
        a, b = slice_range(S, world, r)
        out[a:b] = parts[r][:b - a].numpy()
    return out
