"""Sharding of independent OS-EM work units (slices, energy points) over ranks.

The path has no exchange step: every slice is reconstructed from its own sinogram, so N
processes (one per GPU) each take a share of the units and no collective touches the data
path -- the reference does the same across the devices of one process (CT_reconstruction/
GPU.cpp:634-648).  Units of one shape are split into contiguous slabs; units of different
shapes (a CT-XAFS stack: widths w, angle counts A) are balanced by their cost, which grows as
w^2 * A (every pixel meets every angle once per iteration in each projector).  The only
collective is the timing's maximum over ranks.
"""


def slice_range(n, rank, world):
    """Contiguous [start, end) of n equal-cost slices for rank (sizes differ by at most 1)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank %d outside world %d" % (rank, world))
    q, r = divmod(n, world)
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


def item_cost(width, angles):
    """Relative cost of one slice-iteration of a w x w slice with `angles` projections."""
    return float(width) * float(width) * float(angles)


def balance(costs, world):
    """Longest-processing-time assignment: items sorted by decreasing cost, each given to the
    least-loaded rank (ties to the lowest rank).  Returns one sorted index list per rank."""
    if world <= 0:
        raise ValueError("world must be > 0")
    loads = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda k: (loads[k], k))
        parts[r].append(i)
        loads[r] += costs[i]
    return [sorted(p) for p in parts]


def max_over_ranks(value, device=None):
    """The maximum of a float over the ranks of the default process group (the value itself
    when torch.distributed is not initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
