"""Multi-GPU: replicas over row shards of the point table, one process per GPU.

The join shards naturally: points are independent, so each rank joins its own
contiguous row range of the table and the per-polygon partial results are
summed.  This is the only exchange: one all-reduce of 2P values (count as
int64, sum as float64), plus 4P bound terms for the error-bounds join.  The
raster join's canvas counts are additive too, so partial raster results sum
to the single-GPU result exactly.

`executor(shard_columns) -> (count, sum[, bounds])` runs the local join (a
GLHandler on this rank's GPU in production).
"""
import numpy as np


def shard_range(n, rank, world):
    """Contiguous row range [lo, hi) of rank in a table of n rows."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def shard_columns(columns, rank, world):
    n = len(next(iter(columns.values())))
    lo, hi = shard_range(n, rank, world)
    return {k: v[lo:hi] for k, v in columns.items()}


def join_replicated(executor, columns, rank, world, group=None):
    """Run executor on this rank's shard and sum the partial results over ranks."""
    import torch
    import torch.distributed as dist

    part = executor(shard_columns(columns, rank, world))
    count = torch.from_numpy(np.asarray(part[0], dtype=np.int64).copy())
    s = torch.from_numpy(np.asarray(part[1], dtype=np.float64).copy())
    out = [count, s]
    if len(part) > 2 and part[2] is not None:
        out.append(torch.from_numpy(np.asarray(part[2], dtype=np.int64).copy()))
    if world > 1:
        for t in out:
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    res = [out[0].numpy().astype(np.uint64), out[1].numpy()]
    if len(out) > 2:
        res.append(out[2].numpy())
    return tuple(res)
