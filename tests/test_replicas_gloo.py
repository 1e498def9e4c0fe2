"""Replica sharding over 2 CPU ranks (gloo): the summed partial joins equal the
single-process join, for the exact join and the raster join with bounds."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


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
    pts = synth.points(50_001, seed=9, columns=True)
    verts, pidx = synth.voronoi_polygons(30, seed=9)
    cols = {"xy": pts["xy"], "a": pts["a"]}

    def exact(sh):
        f = oracle.Columns({3: (oracle.Float, sh["a"])}).filt([], aggr_attrib=3)
        c, s = oracle.index_join(sh["xy"], verts, pidx, 64, f=f, nthreads=1)
        return c, s

    def raster(sh):
        c, s, b = oracle.raster_join(sh["xy"], verts, pidx, 100.0, bounds=True, nthreads=1,
                                     bbox=np.array([0, 0, 40000.0, 40000.0]))
        return c, s, b

    r1 = replicas.join_replicated(exact, cols, rank, world)
    r2 = replicas.join_replicated(raster, cols, rank, world)
    dist.barrier()
    dist.destroy_process_group()
    if rank == 0:
        outq.put((r1[0].tolist(), r1[1].tolist(), r2[0].tolist(), r2[2].tolist()))


def test_two_rank_replicas_match_single():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import oracle
    from rasterjoin import synth, replicas

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
    pts = synth.points(50_001, seed=9, columns=True)
    verts, pidx = synth.voronoi_polygons(30, seed=9)
    f = oracle.Columns({3: (oracle.Float, pts["a"])}).filt([], aggr_attrib=3)
    c, s = oracle.index_join(pts["xy"], verts, pidx, 64, f=f)
    np.testing.assert_array_equal(np.array(got[0], np.uint64), c)
    np.testing.assert_allclose(np.array(got[1]), s, rtol=1e-12)
    c, _, b = oracle.raster_join(pts["xy"], verts, pidx, 100.0, bounds=True, bbox=np.array([0, 0, 40000.0, 40000.0]))
    np.testing.assert_array_equal(np.array(got[2], np.uint64), c)
    # bounds terms involve per-pixel ceil(): shard sums are >= the global ones
    assert np.all(np.array(got[3]) >= b)
    assert replicas.shard_range(10, 0, 3) == (0, 4) and replicas.shard_range(10, 2, 3) == (7, 10)
