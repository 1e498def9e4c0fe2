"""Batched raster joins, the time index of the resident table and the
serving loop.

Every query of a batch must give exactly the result it gives alone through
rj_execute (counts and fixed-point sums are order-independent integers, so
the comparison is bit-exact), and alone it matches the CPU oracle.  The time
index reorders the table: results before and after must be identical."""
import ctypes as C

import numpy as np
import pytest

import oracle
import rasterjoin as rj
from rasterjoin import synth

pytestmark = pytest.mark.gpu

T0 = synth.T0
DAY = 86400


@pytest.fixture(scope="module")
def table():
    return synth.points(1_500_003, seed=77, columns=True)


def make_dh(pts, verts, pidx):
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, pts["xy"])
    dh.add_column(2, rj.Uint, pts["t"])
    dh.add_column(3, rj.Float, pts["a"])
    dh.add_column(4, rj.Int, pts["f1"])
    dh.add_column(5, rj.Int, pts["f2"])
    dh.setPolygons(verts, pidx)
    return dh


def poly_sets():
    return [
        synth.voronoi_polygons(260, seed=3),                                                 # tessellation
        synth.star_polygons(60, seed=4, vmin=8, vmax=300, rmin=300, rmax=5000),             # overlapping
        synth.star_polygons(1, seed=5, vmin=40, vmax=40, rmin=6000, rmax=6000),             # one polygon
        synth.star_polygons(7, seed=6, vmin=4, vmax=40, rmin=200, rmax=3000),
        synth.star_polygons(4500, seed=7, vmin=4, vmax=12, rmin=60, rmax=400),              # > shared histogram
    ]


def make_query(cell, aggr=False, window=None, preds=(), max_fbo=8192, fn=rj.RasterJoinFn, flags=0):
    q = rj.default_query()
    q.function_type = fn
    q.cell_size = cell
    q.max_fbo_size = max_fbo
    q.flags = flags
    if aggr:
        q.aggregation = rj.Avg
        q.aggr_attrib = 3
    types = {3: rj.Float, 4: rj.Int, 5: rj.Int, 2: rj.Uint}
    q.n_constraints = len(preds)
    for i, (aid, op, val) in enumerate(preds):
        q.constraints[i] = rj.constraint(aid, op, val, types[aid])
    if window is not None:
        q.time_attrib = 2
        q.t_start, q.t_end = window
    return q


def query_mix():
    """(polygon set, query) pairs of uneven size: canvases from 40 m down to
    multi-tile, count and avg, time windows from a day to the whole year."""
    mix = [
        (0, make_query(40.0)),
        (0, make_query(10.0, aggr=True, window=(T0, T0 + 182 * DAY), preds=((4, rj.GT, 2), (5, rj.LT, 8), (3, rj.LT, 50.0)))),
        (1, make_query(25.0, aggr=True, window=(T0 + 30 * DAY, T0 + 40 * DAY))),
        (2, make_query(5.0, window=(T0 + 100 * DAY, T0 + 101 * DAY))),
        (3, make_query(8.0, aggr=True, preds=((4, rj.EQ, 7),))),
        (4, make_query(20.0, window=(T0, T0 + 300 * DAY))),
        (0, make_query(12.0, max_fbo=1500)),                                                  # 3 x 3 tiles
        (1, make_query(60.0, preds=((3, rj.GTE, 12.5),), window=(T0 + 200 * DAY, T0 + 365 * DAY))),
        (3, make_query(100.0, preds=((4, rj.LT, 0),))),                                       # empty filter
        (2, make_query(30.0, aggr=True, window=(T0 + 400 * DAY, T0 + 500 * DAY))),            # no rows
    ]
    return mix


@pytest.fixture(scope="module")
def setup(table, built):
    h = rj.GLHandler()
    sets_raw = poly_sets()
    v0, p0 = sets_raw[0]
    h.setDataHandler(make_dh(table, v0, p0))
    h.upload()
    sets = [h.polyset(v, p) for v, p in sets_raw]
    yield h, sets, sets_raw
    for s in sets:
        s.close()
    h.close()


def single(h, ps, q):
    h.usePolySet(ps)
    r = h.execute(q.function_type, query=q)
    return r.count.copy(), r.sum.copy()


def test_batch_equals_single_and_oracle(setup, table):
    h, sets, raw = setup
    mix = query_mix()
    alone = [single(h, sets[s], q) for s, q in mix]
    res, status, stats = h.execute_batch([q for _, q in mix], [sets[s] for s, _ in mix], flags=rj.BATCH_FUSE)
    assert (status == 0).all()
    assert stats["fused"] == len(mix) and stats["fallback"] == 0
    for (c, s), r in zip(alone, res):
        np.testing.assert_array_equal(r.count, c)
        np.testing.assert_array_equal(r.sum, s)
    # alone == oracle for a few of them
    cols = oracle.Columns({2: (oracle.Uint, table["t"]), 3: (oracle.Float, table["a"]),
                           4: (oracle.Int, table["f1"]), 5: (oracle.Int, table["f2"])})
    for k in (1, 2, 3, 6):
        s, q = mix[k]
        v, p = raw[s]
        preds = []
        for i in range(q.n_constraints):
            c = q.constraints[i]
            preds.append((c.attribId, c.type, c.val.fval if c.attribId == 3 else c.val.ival))
        f = cols.filt(preds, aggr_attrib=3 if q.aggregation else None,
                      time_range=(2, q.t_start, q.t_end) if q.time_attrib >= 0 else None)
        want = oracle.raster_join(table["xy"], v, p, q.cell_size, f=f, max_res=q.max_fbo_size)
        np.testing.assert_array_equal(res[k].count, want[0])
        if q.aggregation:
            np.testing.assert_allclose(res[k].sum, want[1], rtol=1e-6, atol=1e-9 * max(1.0, float(np.abs(want[1]).max())))


def test_batch_mixed_join_types_fall_back(setup):
    h, sets, _ = setup
    qs = [make_query(20.0), make_query(20.0, fn=rj.HybridJoinFn), make_query(20.0, fn=rj.IndexJoinFn),
          make_query(20.0, fn=rj.RasterJoinBoundFn),
          make_query(20.0, preds=((4, rj.GTE, 3),), flags=rj.FLAG_COMPAT_FLOAT_EQ)]
    ss = [sets[0], sets[3], sets[0], sets[3], sets[1]]
    alone = [single(h, s, q) for s, q in zip(ss, qs)]
    res, status, stats = h.execute_batch(qs, ss, flags=rj.BATCH_FUSE)
    assert (status == 0).all()
    assert stats["fused"] == 1 and stats["fallback"] == 4
    for (c, s), r in zip(alone, res):
        np.testing.assert_array_equal(r.count, c)
        np.testing.assert_array_equal(r.sum, s)


def test_batch_autotune_same_result(setup):
    h, sets, _ = setup
    mix = query_mix()
    base, _, _ = h.execute_batch([q for _, q in mix], [sets[s] for s, _ in mix], flags=rj.BATCH_FUSE)
    tuned, status, stats = h.execute_batch([q for _, q in mix], [sets[s] for s, _ in mix],
                                           flags=rj.BATCH_FUSE | rj.BATCH_AUTOTUNE)
    assert (status == 0).all() and stats["tuned"] == 1
    for a, b in zip(base, tuned):
        np.testing.assert_array_equal(a.count, b.count)
        np.testing.assert_array_equal(a.sum, b.sum)


def test_batch_no_fuse_equals_fused(setup):
    h, sets, _ = setup
    mix = query_mix()
    fused, _, _ = h.execute_batch([q for _, q in mix], [sets[s] for s, _ in mix], flags=rj.BATCH_FUSE)
    plain, status, stats = h.execute_batch([q for _, q in mix], [sets[s] for s, _ in mix], flags=rj.BATCH_NO_FUSE)
    assert (status == 0).all() and stats["fused"] == 0
    for a, b in zip(fused, plain):
        np.testing.assert_array_equal(a.count, b.count)
        np.testing.assert_array_equal(a.sum, b.sum)


def test_time_index_preserves_results(table, built):
    """Reordering the table by time bucket changes no result of any join."""
    v, p = synth.voronoi_polygons(260, seed=3)
    h = rj.GLHandler()
    try:
        h.setDataHandler(make_dh(table, v, p))
        cases = [(fn, make_query(25.0, aggr=True, window=w, fn=fn)) for fn in
                 (rj.RasterJoinFn, rj.IndexJoinFn, rj.HybridJoinFn, rj.RasterJoinBoundFn)
                 for w in ((T0 + 10 * DAY, T0 + 11 * DAY), (T0, T0 + 365 * DAY), None)]
        before = []
        for fn, q in cases:
            r = h.execute(fn, query=q)
            before.append((r.count.copy(), r.sum.copy(), None if r.bounds is None else r.bounds.copy()))
        h.buildTimeIndex(2, 1000)
        for (fn, q), (c, s, b) in zip(cases, before):
            r = h.execute(fn, query=q)
            np.testing.assert_array_equal(r.count, c)
            np.testing.assert_array_equal(r.sum, s)
            if b is not None:
                np.testing.assert_array_equal(r.bounds, b)
    finally:
        h.close()


@pytest.mark.parametrize("batch_flags", [0, rj.BATCH_FUSE])
def test_server_results_alone_and_in_mix(setup, batch_flags):
    """Requests submitted while others run give the result they give alone,
    on the lanes (default) and through the fused pass."""
    h, sets, _ = setup
    mix = query_mix()
    alone = [single(h, sets[s], q) for s, q in mix]
    srv = h.server(slots=2, canvas_mb=2048, max_batch=8, batch_flags=batch_flags)
    try:
        tickets = []
        for rep in range(3):
            for i, (s, q) in enumerate(mix):
                tickets.append((i, srv.submit(q, sets[s])))
        sizes = set()
        for i, t in tickets:
            r, info = srv.poll(t, -1)
            assert info["status"] == 0
            sizes.add(info["batch_size"])
            np.testing.assert_array_equal(r.count, alone[i][0])
            np.testing.assert_array_equal(r.sum, alone[i][1])
        assert max(sizes) > 1      # requests were batched together
    finally:
        srv.close()
    # the context is usable again once the server is gone
    c, s = single(h, sets[0], mix[0][1])
    np.testing.assert_array_equal(c, alone[0][0])


def test_server_rejects_context_calls_while_running(setup):
    h, sets, _ = setup
    srv = h.server(slots=1, canvas_mb=512)
    try:
        with pytest.raises(rj.RJError) as e:
            h.buildTimeIndex(2)
        assert e.value.code == -8
    finally:
        srv.close()


@pytest.mark.parametrize("time_attrib,nb,bits", [(2, 512, 6), (-1, 0, 8)])
def test_clustered_order_preserves_results(table, built, time_attrib, nb, bits):
    """Rows ordered by (time bucket, Z-order cell) or by cell alone: every
    join returns what it returned on the original order, and batches too."""
    v, p = synth.voronoi_polygons(260, seed=3)
    sv, sp = synth.star_polygons(40, seed=12, vmin=8, vmax=200, rmin=300, rmax=5000)
    h = rj.GLHandler()
    try:
        h.setDataHandler(make_dh(table, v, p))
        cases = [(fn, make_query(25.0, aggr=True, window=w, fn=fn)) for fn in
                 (rj.RasterJoinFn, rj.IndexJoinFn, rj.HybridJoinFn, rj.RasterJoinBoundFn)
                 for w in ((T0 + 10 * DAY, T0 + 11 * DAY), None)]
        before = []
        for fn, q in cases:
            r = h.execute(fn, query=q)
            before.append((r.count.copy(), r.sum.copy(), None if r.bounds is None else r.bounds.copy()))
        stars = h.polyset(sv, sp)
        mix = [make_query(12.0, aggr=True, window=(T0, T0 + 90 * DAY)), make_query(30.0),
               make_query(60.0, aggr=True, preds=((4, rj.GT, 4),))]
        bres, _, _ = h.execute_batch(mix, [stars] * len(mix))
        b_before = [(r.count.copy(), r.sum.copy()) for r in bres]
        h.clusterPoints(time_attrib, nb, bits)
        for (fn, q), (c, s, b) in zip(cases, before):
            r = h.execute(fn, query=q)
            np.testing.assert_array_equal(r.count, c)
            np.testing.assert_array_equal(r.sum, s)
            if b is not None:
                np.testing.assert_array_equal(r.bounds, b)
        bres, status, _ = h.execute_batch(mix, [stars] * len(mix))
        assert (status == 0).all()
        for r, (c, s) in zip(bres, b_before):
            np.testing.assert_array_equal(r.count, c)
            np.testing.assert_array_equal(r.sum, s)
        stars.close()
    finally:
        h.close()


def test_batch_tiered_canvases(setup):
    """Large canvases (>= 2^24 pixels) take the tiered form inside the fused
    batch: label form, canvas form after an overlap check, several tiles;
    each equals the flat single-query result."""
    h, sets, _ = setup
    qs = [make_query(5.0, aggr=True), make_query(4.0, aggr=True, window=(T0, T0 + 200 * DAY)),
          make_query(2.5, max_fbo=6000), make_query(6.0, preds=((4, rj.GT, 3),))]
    ss = [sets[0], sets[1], sets[0], sets[4]]
    flat = []
    for s, q in zip(ss, qs):
        q2 = rj.Query()
        C.pointer(q2)[0] = q
        q2.flags = rj.FLAG_FLAT_CANVAS
        flat.append(single(h, s, q2))
    res, status, stats = h.execute_batch(qs, ss, flags=rj.BATCH_FUSE)
    assert (status == 0).all() and stats["fused"] == len(qs) and stats["fallback"] == 0
    for (c, sm), r in zip(flat, res):
        np.testing.assert_array_equal(r.count, c)
        np.testing.assert_array_equal(r.sum, sm)


def test_point_heavy_label_queries_leave_the_fused_pass(built):
    """With RJ_BATCH_FUSE, single-tile queries over >= 2^22 rows leave the
    fused pass for rj_execute's lean passes on the lanes (counted as
    fallback); RJ_BATCH_FUSE_ALL keeps them fused.  Both give the
    single-query results bit for bit."""
    big = synth.points(5_000_001, seed=78, columns=True)
    v, p = poly_sets()[0]
    h = rj.GLHandler()
    try:
        h.setDataHandler(make_dh(big, v, p))
        h.upload()
        ps = h.polyset(v, p)
        qs = [make_query(20.0), make_query(30.0, aggr=True, preds=((4, rj.GT, 2),)),
              make_query(20.0, max_fbo=1000)]                     # a multi-tile canvas stays fused
        alone = [single(h, ps, q) for q in qs]
        res, status, stats = h.execute_batch(qs, [ps] * 3, flags=rj.BATCH_FUSE)
        assert (status == 0).all() and stats["fused"] == 1 and stats["fallback"] == 2
        res2, status2, stats2 = h.execute_batch(qs, [ps] * 3, flags=rj.BATCH_FUSE_ALL)
        assert (status2 == 0).all() and stats2["fused"] == 3 and stats2["fallback"] == 0
        for (c, s), r, r2 in zip(alone, res, res2):
            np.testing.assert_array_equal(r.count, c)
            np.testing.assert_array_equal(r.sum, s)
            np.testing.assert_array_equal(r2.count, c)
            np.testing.assert_array_equal(r2.sum, s)
        ps.close()
    finally:
        h.close()


def test_lanes_equal_single(setup):
    """The default route: every raster query (and the error-bounds query)
    runs rj_execute's device path on the lanes -- eight streams with their own
    scratch -- and gives the single-query results bit for bit, bounds
    included; the other join types still run through rj_execute in turn."""
    h, sets, _ = setup
    mix = query_mix() + [(3, make_query(20.0, fn=rj.RasterJoinBoundFn)), (0, make_query(20.0, fn=rj.IndexJoinFn)),
                         (1, make_query(6.0, fn=rj.RasterJoinBoundFn, window=(T0, T0 + 90 * DAY)))]
    alone = []
    for s, q in mix:
        h.usePolySet(sets[s])
        r = h.execute(q.function_type, query=q)
        alone.append((r.count.copy(), r.sum.copy(), None if r.bounds is None else r.bounds.copy()))
    for rnd in range(2):                                   # the second round reuses the lanes' scratch
        res, status, stats = h.execute_batch([q for _, q in mix], [sets[s] for s, _ in mix])
        assert (status == 0).all() and stats["fused"] == 0 and stats["fallback"] == len(mix)
        for (c, sm, b), r in zip(alone, res):
            np.testing.assert_array_equal(r.count, c)
            np.testing.assert_array_equal(r.sum, sm)
            if b is not None:
                np.testing.assert_array_equal(r.bounds, b)


def test_lanes_retry_queries_the_budget_cannot_hold_at_once(built):
    """Under a device-memory budget too small for several lanes' label maps at
    once, the queries whose lane ran out of memory run again alone after the
    lanes' scratch is released: every status is RJ_OK and every result equals
    the single-query result."""
    pts = synth.points(500_001, seed=91, columns=True)
    h = rj.GLHandler(gpu_mem_mb=48)
    try:
        dh = rj.DataHandler()
        dh.add_column(1, rj.Location, pts["xy"])
        v0, p0 = synth.voronoi_polygons(60, seed=92)
        dh.setPolygons(v0, p0)
        h.setDataHandler(dh)
        h.upload()
        sets = [h.polyset(*synth.voronoi_polygons(60, seed=93 + k)) for k in range(4)]
        qs = [make_query(10.0) for _ in range(4)]         # 4000 x 4000 label maps: 32 MB each
        alone = [single(h, s, q) for s, q in zip(sets, qs)]
        res, status, stats = h.execute_batch(qs, sets, raise_on_error=False)
        assert (status == 0).all(), status
        for (c, sm), r in zip(alone, res):
            np.testing.assert_array_equal(r.count, c)
        for s in sets:
            s.close()
    finally:
        h.close()
