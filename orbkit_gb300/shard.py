"""Point sharding across GPUs (one process per GPU).

Grid points are independent (orbkit's slice_rho works on any slice,
orbkit/core.py:179-308), so N ranks each take one contiguous block of the
flattened grid and no data-path collective is needed; the blocks are
concatenated on the host.  ``point_range`` is the partition, ``gather_blocks``
the host-side concatenation over torch.distributed (any backend).
"""


def point_range(npts, rank, world):
    """[start, end) of rank's block: sizes differ by at most one point."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("rank %d outside world of size %d" % (rank, world))
    base, extra = divmod(int(npts), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_blocks(block, group=None):
    """Concatenate every rank's block (numpy arrays, points on the last axis) on all ranks."""
    import numpy
    import torch.distributed as dist
    world = dist.get_world_size(group)
    out = [None] * world
    dist.all_gather_object(out, block, group=group)
    return numpy.concatenate(out, axis=-1)
