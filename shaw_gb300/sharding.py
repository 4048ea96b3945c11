"""Forcing-column sharding across GPUs (one process per GPU).

Rank-2 columns are independent for the whole run: the forcing couples only within a
column (AddForcingRank2, src/kokkos/fom_update_kernels.hpp:106-129) and the updates are
column-wise (updateVelocity / updateStress rank 2, :132-181).  A job of M forcings is
therefore split into contiguous column ranges, one per rank, with no communication in
the time loop; the per-rank outputs (seismograms R x T x m, snapshots N x T x m,
final states N x m -- forcing index last) are concatenated on rank 0 at the end.
"""
import numpy as np


def shard_range(total, rank, world):
    """Contiguous, balanced [start, stop) of `total` columns for `rank` of `world`
    (the first total % world ranks hold one extra column; a rank may hold none)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    if total < 0:
        raise ValueError("negative column count")
    base, extra = divmod(total, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_columns(local, total, dist, group=None, dst=0):
    """Concatenate each rank's column block (last axis) on rank `dst`, in rank order.

    `local` is this rank's array (..., m) with m = its shard size; every rank passes the
    same leading shape.  Runs over a host (gloo) process group; returns the full array
    (..., total) on `dst` and None elsewhere.  Outside any timed region: it is the
    host gather of the outputs, not part of the time loop."""
    import torch

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    start, stop = shard_range(total, rank, world)
    local = np.asarray(local, np.float64)
    if local.shape[-1] != stop - start:
        raise ValueError("rank %d holds %d columns, its shard is %d" % (rank, local.shape[-1], stop - start))
    lead = local.shape[:-1]
    width = -(-total // world)  # the largest shard
    buf = np.zeros(lead + (width,))
    buf[..., : stop - start] = local
    t = torch.from_numpy(np.ascontiguousarray(buf))
    parts = [torch.zeros_like(t) for _ in range(world)] if rank == dst else None
    dist.gather(t, parts, dst=dst, group=group)
    if rank != dst:
        return None
    cols = []
    for r in range(world):
        a, b = shard_range(total, r, world)
        cols.append(parts[r].numpy()[..., : b - a])
    return np.concatenate(cols, axis=-1)
