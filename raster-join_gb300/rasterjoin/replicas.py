"""Multi-GPU: replicas over row shards of the point table, one process per GPU.

The join shards naturally: points are independent, so each rank joins its own
contiguous row range of the table and the per-polygon partial results are
summed.  This is the only exchange: one all-reduce each of the counts (int64),
the exact fixed-point sums (int64), the fp64 sums of non-finite values and,
for the error-bounds join, the 4P bound terms.

Sums stay exact across ranks.  The library sums round(v * 2^shift) as int64
per polygon (order-independent) and decodes once.  Replicas first agree on the
shift the whole table would get (largest |value| over all shards, total rows:
`agree_shift`), each rank joins its shard with that shift, the int64 partials
are all-reduced (two's complement, wrapping like the kernels' atomics) and
decoded once: N ranks give the bits of one GPU.  Non-finite values are summed
apart in fp64, where the result does not depend on the order (any NaN gives
NaN, infinities of one sign their infinity, of both signs NaN).

`executor(shard_columns) -> Partial` runs the local join (a GLHandler on this
rank's GPU in production, `handler_executor`).
"""
from collections import namedtuple

import numpy as np

# count: uint64[P]; fixed: int64[P]; nonfinite: float64[P]; shift: int;
# bounds: int64[4P] or None
Partial = namedtuple("Partial", "count fixed nonfinite shift bounds")


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


def sum_shift_for(max_abs, rows):
    """The library's fixed-point shift for |values| <= max_abs over `rows` rows
    (rj_sum_shift_for): |v| * 2^s * rows < 2^62 for every subset."""
    amax = max(abs(float(max_abs)) if np.isfinite(max_abs) else 0.0, 1e-30)
    s = int(np.floor(62.0 - np.log2(amax) - np.log2(float(rows) + 1.0)))
    return max(-90, min(150, s))


def agree_shift(local_max_abs, local_rows, world, group=None):
    """Shift of the whole table: max over ranks of the largest |value|, sum of rows."""
    import torch
    import torch.distributed as dist

    m = torch.tensor([float(local_max_abs)], dtype=torch.float64)
    r = torch.tensor([int(local_rows)], dtype=torch.int64)
    if world > 1:
        dist.all_reduce(m, op=dist.ReduceOp.MAX, group=group)
        dist.all_reduce(r, op=dist.ReduceOp.SUM, group=group)
    return sum_shift_for(m.item(), r.item())


def decode_sums(fixed, nonfinite, shift):
    """fixed * 2^-shift + nonfinite, as the library decodes a single join."""
    return np.ldexp(np.asarray(fixed, np.int64).astype(np.float64), -int(shift)) + np.asarray(nonfinite, np.float64)


def join_replicated(executor, columns, rank, world, group=None):
    """Run executor on this rank's shard and reduce the exact partials over
    ranks; returns (count uint64[P], sum float64[P], bounds int64[4P] or None)."""
    import torch
    import torch.distributed as dist

    part = executor(shard_columns(columns, rank, world))
    shifts = torch.tensor([int(part.shift), -int(part.shift)], dtype=torch.int64)
    count = torch.from_numpy(np.asarray(part.count, dtype=np.uint64).astype(np.int64))
    fixed = torch.from_numpy(np.asarray(part.fixed, dtype=np.int64).copy())
    nonfinite = torch.from_numpy(np.asarray(part.nonfinite, dtype=np.float64).copy())
    out = [count, fixed, nonfinite]
    if part.bounds is not None:
        out.append(torch.from_numpy(np.asarray(part.bounds, dtype=np.int64).copy()))
    if world > 1:
        dist.all_reduce(shifts, op=dist.ReduceOp.MAX, group=group)
        if int(shifts[0]) != -int(shifts[1]):
            raise ValueError("replicas joined with different sum shifts (%d..%d): agree on one first"
                             % (-int(shifts[1]), int(shifts[0])))
        for t in out:
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    sums = decode_sums(out[1].numpy(), out[2].numpy(), part.shift)
    bounds = out[3].numpy() if len(out) > 3 else None
    return out[0].numpy().astype(np.uint64), sums, bounds


def handler_executor(handler, fn, shift):
    """Executor over a GLHandler: loads the shard's columns (attrib id -> (type,
    array); the location column under the DataHandler's location id), joins
    with the agreed shift and returns the exact partials."""
    import rasterjoin as rj

    def run(shard):
        dh = handler.dataHandler
        for aid, arr in shard.items():
            dh.add_column(aid, dh.attr_type(aid), arr)
        handler.setSumShift(shift)
        r = handler.execute(fn)
        fixed, nf, sh = handler.sumPartials()
        b = r.bounds.astype(np.int64) if (fn == rj.RasterJoinBoundFn and r.bounds is not None) else None
        return Partial(r.count, fixed, nf, sh, b)

    return run
