"""Replica sharding over 2 CPU ranks (gloo): the reduced partial joins equal the
single-process join bit for bit -- counts, exact fixed-point sums (including
non-finite values) and the raster join's counts; bound terms are additive
upper bounds."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N = 50_001


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _values(n, seed):
    """Lognormal aggregate values with a few non-finite ones (NaN, +inf)."""
    rng = np.random.default_rng(seed)
    a = np.exp(rng.normal(2.5, 0.8, n)).astype(np.float32)
    a[rng.choice(n, 5, replace=False)] = np.inf
    a[rng.choice(n, 3, replace=False)] = np.nan
    return a


def _toy_partial(shard, shift, P=30):
    """Exact partials of a stand-in join: polygon = cell of a 5 x 6 grid over
    the box; fixed = sum of round(a * 2^shift) per polygon (int64)."""
    from rasterjoin import replicas
    xy, a = shard["xy"], shard["a"]
    label = (np.clip((xy[:, 0] / 8000.0).astype(int), 0, 4) * 6 + np.clip((xy[:, 1] / 6667.0).astype(int), 0, 5))
    count = np.bincount(label, minlength=P).astype(np.uint64)
    fin = np.isfinite(a)
    q = np.round(np.ldexp(a[fin].astype(np.float64), shift)).astype(np.int64)
    fixed = np.zeros(P, np.int64)
    np.add.at(fixed, label[fin], q)
    nf = np.zeros(P, np.float64)
    np.add.at(nf, label[~fin], a[~fin].astype(np.float64))
    return replicas.Partial(count, fixed, nf, shift, None)


def _worker(rank, world, port, outq):
    import sys
    for p in (os.path.join(ROOT, "raster-join_gb300"), os.path.join(ROOT, "oracle")):
        sys.path.insert(0, p)
    import torch.distributed as dist
    import oracle
    from rasterjoin import replicas, synth

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pts = synth.points(N, seed=9, columns=True)
    verts, pidx = synth.voronoi_polygons(30, seed=9)
    cols = {"xy": pts["xy"], "a": _values(N, 9)}
    mine = replicas.shard_columns(cols, rank, world)
    a = mine["a"]
    shift = replicas.agree_shift(np.max(np.abs(a[np.isfinite(a)])), len(a), world)

    r1 = replicas.join_replicated(lambda sh: _toy_partial(sh, shift), cols, rank, world)

    def raster(sh):
        c, _, b = oracle.raster_join(sh["xy"], verts, pidx, 100.0, bounds=True, nthreads=1,
                                     bbox=np.array([0, 0, 40000.0, 40000.0]))
        P = len(c)
        return replicas.Partial(c, np.zeros(P, np.int64), np.zeros(P), 0, b)

    r2 = replicas.join_replicated(raster, cols, rank, world)
    # shards that do not agree on the shift are refused
    refused = False
    try:
        replicas.join_replicated(lambda sh: _toy_partial(sh, shift + rank), cols, rank, world)
    except ValueError:
        refused = True
    dist.barrier()
    dist.destroy_process_group()
    if rank == 0:
        outq.put((r1[0].tolist(), r1[1].tobytes(), r2[0].tolist(), r2[2].tolist(), shift, refused))


def test_two_rank_replicas_match_single():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import oracle
    from rasterjoin import replicas, synth

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    pts = synth.points(N, seed=9, columns=True)
    a = _values(N, 9)
    shift = replicas.sum_shift_for(np.max(np.abs(a[np.isfinite(a)])), N)
    assert got[4] == shift
    assert got[5], "shards with different shifts must be refused"
    one = _toy_partial({"xy": pts["xy"], "a": a}, shift)
    np.testing.assert_array_equal(np.array(got[0], np.uint64), one.count)
    single = replicas.decode_sums(one.fixed, one.nonfinite, shift)
    assert np.frombuffer(got[1], np.float64).tobytes() == single.tobytes()   # bit equality, NaNs included
    verts, pidx = synth.voronoi_polygons(30, seed=9)
    c, _, b = oracle.raster_join(pts["xy"], verts, pidx, 100.0, bounds=True, bbox=np.array([0, 0, 40000.0, 40000.0]))
    np.testing.assert_array_equal(np.array(got[2], np.uint64), c)
    # bounds terms involve per-pixel ceil(): shard sums are >= the global ones
    assert np.all(np.array(got[3]) >= b)
    assert replicas.shard_range(10, 0, 3) == (0, 4) and replicas.shard_range(10, 2, 3) == (7, 10)


def test_shift_formula_matches_library():
    """replicas.sum_shift_for restates rj_sum_shift_for."""
    import rasterjoin as rj
    from rasterjoin import replicas
    try:
        rj.load_library()
    except RuntimeError:
        pytest.skip("librj.so not built")
    for amax, rows in ((1.0, 1), (50.0, 100_000_000), (3.4e38, 2_000_000_000), (1e-20, 5), (0.0, 0),
                       (float("inf"), 10), (7.5, 1 << 40)):
        assert replicas.sum_shift_for(amax, rows) == rj.sum_shift_for(amax, rows), (amax, rows)
