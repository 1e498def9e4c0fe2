"""GPU parity: every join type through the C ABI against the CPU oracle.

Counts must be bit-exact; sums (avg) within 1e-6 relative of the oracle's
double-precision accumulation; error bounds bit-exact.
"""
import numpy as np
import pytest

import oracle
import rasterjoin as rj
from rasterjoin import synth

pytestmark = pytest.mark.gpu

SUM_RTOL = 1e-6


@pytest.fixture(scope="module")
def c1():
    """Benchmark configuration 1: 1M points, 260 Voronoi cells, 40 km box."""
    pts = synth.points(1_000_000, seed=20261203, columns=True)
    verts, pidx = synth.voronoi_polygons(260, seed=20261203)
    return pts, verts, pidx


@pytest.fixture(scope="module")
def stars():
    pts = synth.points(300_001, seed=5, columns=True)
    verts, pidx = synth.star_polygons(150, seed=5, vmin=8, vmax=300, rmin=300, rmax=4000)
    return pts, verts, pidx


def make_dh(pts, verts, pidx):
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, pts["xy"])
    if "t" in pts:
        dh.add_column(2, rj.Uint, pts["t"])
        dh.add_column(3, rj.Float, pts["a"])
        dh.add_column(4, rj.Int, pts["f1"])
        dh.add_column(5, rj.Int, pts["f2"])
    dh.setPolygons(verts, pidx)
    return dh


def ocols(pts):
    return oracle.Columns({2: (oracle.Uint, pts["t"]), 3: (oracle.Float, pts["a"]),
                           4: (oracle.Int, pts["f1"]), 5: (oracle.Int, pts["f2"])})


def check_sums(got, want):
    np.testing.assert_allclose(got, want, rtol=SUM_RTOL, atol=1e-9 * max(1.0, float(np.abs(want).max())))


def test_kat_two_squares(handler):
    """RasterJoin/test/baseline.hpp:139-217: counts 2 and 3 for every join."""
    xy, (verts, pidx), expect = synth.kat_two_squares()
    dh = rj.DataHandler()
    dh.add_column(0, rj.Location, xy)
    dh.setPolygons(verts, pidx)
    handler.setDataHandler(dh)
    handler.setCellSize(0.001)
    handler.setPolyIndexResolution(256)
    for fn in (rj.RasterJoinFn, rj.IndexJoinFn, rj.HybridJoinFn, rj.RasterJoinBoundFn):
        np.testing.assert_array_equal(handler.execute(fn).count, expect)
    agg = handler.executeFunction(rj.IndexJoinFn)
    assert list(agg[:2]) == [2, 3]


@pytest.mark.parametrize("cell", [10.0, 10.0 / np.sqrt(2.0)])
def test_c1_raster_count(handler, c1, cell):
    pts, verts, pidx = c1
    handler.setDataHandler(make_dh(pts, verts, pidx))
    handler.setCellSize(cell)
    got = handler.execute(rj.RasterJoinFn)
    want, _, _ = oracle.raster_join(pts["xy"], verts, pidx, cell)
    np.testing.assert_array_equal(got.count, want)


def test_c1_raster_epsilon_semantics(handler, c1):
    """accuracy 10 m -> cell 10/sqrt(2) (GLFunction::setMaxCellSize)."""
    pts, verts, pidx = c1
    handler.setDataHandler(make_dh(pts, verts, pidx))
    handler.setAccuracyDistance(10.0)
    got = handler.execute(rj.RasterJoinFn)
    want, _, _ = oracle.raster_join(pts["xy"], verts, pidx, oracle.raster_cell(accuracy_m=10.0))
    np.testing.assert_array_equal(got.count, want)


@pytest.mark.parametrize("res", [256, 1024])
def test_c1_index_matches_cpujoin(handler, c1, res):
    pts, verts, pidx = c1
    handler.setDataHandler(make_dh(pts, verts, pidx))
    handler.setPolyIndexResolution(res)
    got = handler.execute(rj.IndexJoinFn)
    want, _ = oracle.index_join(pts["xy"], verts, pidx, res)
    np.testing.assert_array_equal(got.count, want)
    cpu, _, _, _ = oracle.cpujoin(pts["xy"], verts, pidx, 1024)
    np.testing.assert_array_equal(got.count, cpu)


def test_c1_hybrid_exact(handler, c1):
    pts, verts, pidx = c1
    handler.setDataHandler(make_dh(pts, verts, pidx))
    handler.setPolyIndexResolution(256)
    got = handler.execute(rj.HybridJoinFn)
    want, _ = oracle.hybrid_join(pts["xy"], verts, pidx, 256)
    np.testing.assert_array_equal(got.count, want)
    cpu, _, _, _ = oracle.cpujoin(pts["xy"], verts, pidx, 1024)
    np.testing.assert_array_equal(got.count, cpu)


def test_c1_error_bounds(handler, c1):
    pts, verts, pidx = c1
    handler.setDataHandler(make_dh(pts, verts, pidx))
    handler.setCellSize(10.0)
    got = handler.execute(rj.RasterJoinBoundFn)
    c, _, b = oracle.raster_join(pts["xy"], verts, pidx, 10.0, bounds=True)
    np.testing.assert_array_equal(got.count, c)
    np.testing.assert_array_equal(got.bounds.astype(np.int64), b)
    # every exact count lies inside its hard range [agg - fp1, agg + fn1]
    exact, _ = oracle.index_join(pts["xy"], verts, pidx, 256)
    P = len(pidx) - 1
    agg = got.count.astype(np.int64)
    lo, hi = agg - b[3 * P:], agg + b[2 * P:3 * P]
    assert np.all((exact.astype(np.int64) >= lo) & (exact.astype(np.int64) <= hi))


@pytest.mark.parametrize("which", ["c1", "stars"])
def test_error_bounds_reference_line_filter(handler, c1, stars, which):
    """RJ_FLAG_LINE_FILTER: the reference's outline pass keeps an edge's
    fragment only when the pixel centre is within 0.5 px of the edge
    (line-bound.frag:221); bounds bit-exact against the oracle's restatement,
    and never wider than the default (every intersected pixel) bounds."""
    pts, verts, pidx = c1 if which == "c1" else stars
    cell = 10.0 if which == "c1" else 25.0
    handler.setDataHandler(make_dh(pts, verts, pidx))
    handler.setCellSize(cell)
    handler.flags = rj.FLAG_LINE_FILTER
    try:
        got = handler.execute(rj.RasterJoinBoundFn)
    finally:
        handler.flags = 0
    c, _, b = oracle.raster_join(pts["xy"], verts, pidx, cell, bounds=True, line_filter=True)
    np.testing.assert_array_equal(got.count, c)
    np.testing.assert_array_equal(got.bounds.astype(np.int64), b)
    full = handler.execute(rj.RasterJoinBoundFn)
    assert np.all(got.bounds.astype(np.int64) <= full.bounds.astype(np.int64))
    assert got.bounds.astype(np.int64).sum() < full.bounds.astype(np.int64).sum()


def c2_query(dh):
    dh.setQueryConstraints([(4, rj.GT, 2), (5, rj.LT, 8), (3, rj.LT, 50.0)])
    dh.setTimeRange(2, synth.T0, synth.T0 + synth.YEAR // 2)
    dh.setAggregation(rj.Avg, 3)


def c2_filter(pts):
    return ocols(pts).filt([(4, oracle.GT, 2), (5, oracle.LT, 8), (3, oracle.LT, 50.0)], aggr_attrib=3,
                           time_range=(2, synth.T0, synth.T0 + synth.YEAR // 2))


@pytest.mark.parametrize("fn", [rj.IndexJoinFn, rj.HybridJoinFn, rj.RasterJoinFn])
def test_c2_filters_avg(handler, c1, fn):
    pts, verts, pidx = c1
    dh = make_dh(pts, verts, pidx)
    c2_query(dh)
    handler.setDataHandler(dh)
    handler.setAccuracyDistance(100.0)
    handler.setPolyIndexResolution(256)
    got = handler.execute(fn)
    f = c2_filter(pts)
    if fn == rj.IndexJoinFn:
        want = oracle.index_join(pts["xy"], verts, pidx, 256, f=f)
    elif fn == rj.HybridJoinFn:
        want = oracle.hybrid_join(pts["xy"], verts, pidx, 256, f=f)
    else:
        want = oracle.raster_join(pts["xy"], verts, pidx, oracle.raster_cell(accuracy_m=100.0), f=f)[:2]
    np.testing.assert_array_equal(got.count, want[0])
    check_sums(got.sum, want[1])
    if fn != rj.RasterJoinFn:
        # avg against the FP64 oracle (double-precision point-in-polygon)
        c64, s64 = oracle.bruteforce_f64(pts["xy"], verts, pidx, f=f)
        agree = got.count == c64
        assert agree.mean() > 0.99
        ok = agree & (c64 > 0)
        np.testing.assert_allclose(got.avg[ok], (s64 / np.maximum(c64, 1))[ok], rtol=SUM_RTOL)


def test_compat3_decodes_to_avg(handler, c1):
    pts, verts, pidx = c1
    dh = make_dh(pts, verts, pidx)
    dh.setAggregation(rj.Avg, 3)
    handler.setDataHandler(dh)
    r = handler.execute(rj.IndexJoinFn)
    dec = rj.decode_avg(r.compat3)
    np.testing.assert_allclose(dec, r.avg, rtol=1e-3)


def test_multi_tile_canvas(handler, c1):
    """Canvas larger than the tile size splits into tiles (RasterJoin.cpp:59-63)."""
    pts, verts, pidx = c1
    dh = make_dh(pts, verts, pidx)
    dh.setAggregation(rj.Sum, 3)
    handler.setDataHandler(dh)
    handler.setCellSize(10.0)
    handler.max_fbo_size = 1500
    try:
        for fn in (rj.RasterJoinFn, rj.RasterJoinBoundFn):
            got = handler.execute(fn)
            f = ocols(pts).filt([], aggr_attrib=None if fn == rj.RasterJoinBoundFn else 3)
            c, s, b = oracle.raster_join(pts["xy"], verts, pidx, 10.0, f=f, max_res=1500,
                                         bounds=fn == rj.RasterJoinBoundFn)
            np.testing.assert_array_equal(got.count, c)
            if fn == rj.RasterJoinBoundFn:
                np.testing.assert_array_equal(got.bounds.astype(np.int64), b)
            else:
                check_sums(got.sum, s)
    finally:
        handler.max_fbo_size = 8192


def test_force_canvas_equals_label(handler, c1):
    pts, verts, pidx = c1
    dh = make_dh(pts, verts, pidx)
    dh.setAggregation(rj.Avg, 3)
    handler.setDataHandler(dh)
    handler.setCellSize(10.0)
    handler.setPolyIndexResolution(256)
    for fn in (rj.RasterJoinFn, rj.HybridJoinFn):
        handler.flags = 0
        a = handler.execute(fn)
        handler.flags = rj.FLAG_FORCE_CANVAS
        b = handler.execute(fn)
        handler.flags = 0
        np.testing.assert_array_equal(a.count, b.count)
        check_sums(a.sum, b.sum)


def test_overlapping_stars(handler, stars):
    """Overlapping polygons: every covering polygon counts (canvas path)."""
    pts, verts, pidx = stars
    dh = make_dh(pts, verts, pidx)
    dh.setAggregation(rj.Avg, 3)
    handler.setDataHandler(dh)
    handler.setCellSize(25.0)
    handler.setPolyIndexResolution(128)
    f = ocols(pts).filt([], aggr_attrib=3)
    want = oracle.index_join(pts["xy"], verts, pidx, 128, f=f)
    for fn in (rj.IndexJoinFn, rj.HybridJoinFn):
        got = handler.execute(fn)
        np.testing.assert_array_equal(got.count, want[0])
        check_sums(got.sum, want[1])
    got = handler.execute(rj.RasterJoinFn)
    c, s, _ = oracle.raster_join(pts["xy"], verts, pidx, 25.0, f=f)
    np.testing.assert_array_equal(got.count, c)
    check_sums(got.sum, s)
    dh.setAggregation(rj.Count, -1)
    got = handler.execute(rj.RasterJoinBoundFn)
    c, _, b = oracle.raster_join(pts["xy"], verts, pidx, 25.0, bounds=True)
    np.testing.assert_array_equal(got.count, c)
    np.testing.assert_array_equal(got.bounds.astype(np.int64), b)


def test_compat_index_clamp(handler, c1):
    pts, verts, pidx = c1
    handler.setDataHandler(make_dh(pts, verts, pidx))
    handler.setPolyIndexResolution(64)
    handler.flags = rj.FLAG_COMPAT_INDEX_CLAMP
    try:
        got = handler.execute(rj.IndexJoinFn)
    finally:
        handler.flags = 0
    want, _ = oracle.index_join(pts["xy"], verts, pidx, 64, compat_clamp=True)
    np.testing.assert_array_equal(got.count, want)
    exact, _ = oracle.index_join(pts["xy"], verts, pidx, 64)
    assert want.sum() < exact.sum()   # the clamp drops the last grid row/column


@pytest.mark.parametrize("compat", [False, True])
def test_lte_gte_equality(handler, c1, compat):
    pts, verts, pidx = c1
    dh = make_dh(pts, verts, pidx)
    cons = [(4, rj.LTE, 5), (5, rj.GTE, 3), (3, rj.GTE, 12.5)]
    dh.setQueryConstraints(cons)
    handler.setDataHandler(dh)
    handler.flags = rj.FLAG_COMPAT_FLOAT_EQ if compat else 0
    try:
        got = handler.execute(rj.IndexJoinFn)
    finally:
        handler.flags = 0
    f = ocols(pts).filt([(4, oracle.LTE, 5), (5, oracle.GTE, 3), (3, oracle.GTE, 12.5)], compat_float_eq=compat)
    want, _ = oracle.index_join(pts["xy"], verts, pidx, handler.presx, f=f)
    np.testing.assert_array_equal(got.count, want)


@pytest.mark.parametrize("n", [0, 1, 3, 5, 4099])
def test_small_and_ragged_tables(handler, c1, n):
    pts, verts, pidx = c1
    sub = {k: v[:n] for k, v in pts.items()}
    dh = make_dh(sub, verts, pidx)
    dh.setAggregation(rj.Avg, 3)
    handler.setDataHandler(dh)
    handler.setCellSize(10.0)
    f = ocols(sub).filt([], aggr_attrib=3)
    for fn in (rj.RasterJoinFn, rj.IndexJoinFn, rj.HybridJoinFn):
        got = handler.execute(fn)
        if fn == rj.RasterJoinFn:
            want = oracle.raster_join(sub["xy"], verts, pidx, 10.0, f=f)[:2]
        else:
            want = oracle.index_join(sub["xy"], verts, pidx, handler.presx, f=f)
        np.testing.assert_array_equal(got.count, want[0])
        check_sums(got.sum, want[1])


def test_points_outside_bounds(handler):
    rng = np.random.default_rng(3)
    xy = rng.uniform(-20000, 60000, size=(100_000, 2)).astype(np.float32)
    verts, pidx = synth.voronoi_polygons(40, seed=3)
    pts = {"xy": xy}
    handler.setDataHandler(make_dh(pts, verts, pidx))
    handler.setCellSize(20.0)
    handler.setPolyIndexResolution(128)
    got = handler.execute(rj.IndexJoinFn)
    np.testing.assert_array_equal(got.count, oracle.index_join(xy, verts, pidx, 128)[0])
    got = handler.execute(rj.HybridJoinFn)
    np.testing.assert_array_equal(got.count, oracle.hybrid_join(xy, verts, pidx, 128)[0])
    got = handler.execute(rj.RasterJoinFn)
    np.testing.assert_array_equal(got.count, oracle.raster_join(xy, verts, pidx, 20.0)[0])


def test_hybrid_canvas_size_invariance(handler, c1):
    """The hybrid join is exact whatever canvas it uses (ε is ignored)."""
    pts, verts, pidx = c1
    handler.setDataHandler(make_dh(pts, verts, pidx))
    handler.setPolyIndexResolution(256)
    ref = None
    try:
        for canvas in (1024, 4096, 8192):
            handler.hybrid_canvas = canvas
            got = handler.execute(rj.HybridJoinFn).count
            if ref is None:
                ref = got
            np.testing.assert_array_equal(got, ref)
    finally:
        handler.hybrid_canvas = 0


def near_edge_points(verts, pidx, seed=1):
    """Points on vertices, on edges and within 1e-4..1 m of them."""
    rng = np.random.default_rng(seed)
    out = [verts.astype(np.float32)]
    for p in range(len(pidx) - 1):
        v = verts[pidx[p]:pidx[p + 1]].astype(np.float64)
        w = np.roll(v, -1, axis=0)
        t = rng.random((len(v), 3))
        for k in range(3):
            q = v + (w - v) * t[:, k:k + 1]
            d = w - v
            nrm = np.c_[-d[:, 1], d[:, 0]] / np.maximum(np.hypot(d[:, 0], d[:, 1]), 1e-9)[:, None]
            for off in (0.0, 1e-4, -1e-4, 1e-2, -1e-2, 0.5, -0.5):
                out.append((q + off * nrm).astype(np.float32))
    xy = np.concatenate(out)
    return xy[(xy[:, 0] >= 0) & (xy[:, 1] >= 0)]


@pytest.mark.parametrize("polys", ["voronoi", "stars"])
def test_points_on_and_near_edges(handler, polys):
    if polys == "voronoi":
        verts, pidx = synth.voronoi_polygons(80, seed=21)
    else:
        verts, pidx = synth.star_polygons(60, seed=21, vmin=5, vmax=200, rmin=300, rmax=5000)
    xy = near_edge_points(verts, pidx)
    handler.setDataHandler(make_dh({"xy": xy}, verts, pidx))
    for res in (64, 256):
        handler.setPolyIndexResolution(res)
        want, _ = oracle.index_join(xy, verts, pidx, res)
        np.testing.assert_array_equal(handler.execute(rj.IndexJoinFn).count, want)
        np.testing.assert_array_equal(handler.execute(rj.HybridJoinFn).count,
                                      oracle.hybrid_join(xy, verts, pidx, res)[0])
        handler.flags = rj.FLAG_NO_CELL_CLASSIFY
        try:
            np.testing.assert_array_equal(handler.execute(rj.IndexJoinFn).count, want)
        finally:
            handler.flags = 0


def _edge_values(typ, n, rng):
    if typ == "f":
        special = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, -np.nan, 1e-45, -1e-45, 1e-38,
                            3.4e38, -3.4e38, 12.5, 50.0], np.float32)
        vals = rng.choice(special, n).astype(np.float32)
        return vals.view(np.uint32), special
    if typ == "i":
        special = np.array([0, 1, -1, 2, -2, 2**31 - 1, -2**31, 7, 8, 9], np.int64).astype(np.int32)
        return rng.choice(special, n).astype(np.int32).view(np.uint32), special
    special = np.array([0, 1, 2, 2**32 - 1, 2**31, 2**31 - 1, 7, 8], np.uint64).astype(np.uint32)
    return rng.choice(special, n).astype(np.uint32), special


@pytest.mark.parametrize("typ", ["f", "i", "u"])
def test_predicates_on_edge_values(handler, typ):
    """Every operator against +-0, +-inf, NaN, denormals and integer extremes."""
    rng = np.random.default_rng(7)
    verts, pidx = synth.voronoi_polygons(16, seed=7)
    n = 400_000
    xy = synth.points(n, seed=7)["xy"]
    col, special = _edge_values(typ, n, rng)
    at = {"f": rj.Float, "i": rj.Int, "u": rj.Uint}[typ]
    ot = {"f": oracle.Float, "i": oracle.Int, "u": oracle.Uint}[typ]
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, xy)
    dh.add_column(9, at, col.view({"f": np.float32, "i": np.int32, "u": np.uint32}[typ]))
    dh.setPolygons(verts, pidx)
    handler.setDataHandler(dh)
    handler.setPolyIndexResolution(64)
    cols = oracle.Columns({9: (ot, col.view({"f": np.float32, "i": np.int32, "u": np.uint32}[typ]))})
    for v in special[:8]:
        for op in (rj.EQ, rj.LT, rj.LTE, rj.GT, rj.GTE):
            cons = [(9, op, v)]
            dh.setQueryConstraints(cons)
            got = handler.execute(rj.IndexJoinFn).count
            want, _ = oracle.index_join(xy, verts, pidx, 64, f=cols.filt(cons))
            np.testing.assert_array_equal(got, want, err_msg="op %d value %r" % (op, v))
    # two predicates on one column intersect; an empty intersection selects nothing
    for cons, nonempty in (([(9, rj.GTE, special[1]), (9, rj.LTE, special[2])], True),
                           ([(9, rj.GT, special[2]), (9, rj.LT, special[2])], False)):
        dh.setQueryConstraints(cons)
        got = handler.execute(rj.IndexJoinFn).count
        want, _ = oracle.index_join(xy, verts, pidx, 64, f=cols.filt(cons))
        np.testing.assert_array_equal(got, want)
        if not nonempty:
            assert got.sum() == 0


def test_errors_are_status_codes(handler, c1):
    pts, verts, pidx = c1
    dh = make_dh(pts, verts, pidx)
    dh.setQueryConstraints([(4, rj.GT, 0)] * 11)
    handler.setDataHandler(dh)
    with pytest.raises(rj.RJError) as e:
        handler.execute(rj.IndexJoinFn)
    assert e.value.code == -3
    dh.setQueryConstraints([(99, rj.GT, 0)])
    with pytest.raises(rj.RJError) as e:
        handler.execute(rj.IndexJoinFn)
    assert e.value.code == -1
    dh.setQueryConstraints([])
    q = handler.make_query(7)
    with pytest.raises(rj.RJError) as e:
        handler.execute(7, query=q)
    assert e.value.code == -7
    # the context stays usable after errors
    got = handler.execute(rj.IndexJoinFn)
    assert got.count.sum() > 0


def test_timing_line(handler, c1):
    pts, verts, pidx = c1
    handler.setDataHandler(make_dh(pts, verts, pidx))
    handler.flags = rj.FLAG_PHASE_TIMING
    try:
        handler.execute(rj.RasterJoinFn)
    finally:
        handler.flags = 0
    line = handler.printTimeStats()
    fields = line.split()
    assert len(fields) == 15 and int(fields[0]) == len(pts["xy"]) and int(fields[2]) == 0
    t = handler.timings()
    assert t["pt_render_ms"] > 0


def test_overlap_status_is_per_canvas(handler):
    """Two squares sharing a 0.1-wide strip: no pixel centre of a 10-unit
    canvas falls in the strip (label map), every 0.05-unit canvas has some
    (the canvas path must take over after the coarse query)."""
    rng = np.random.default_rng(3)
    xy = np.c_[rng.uniform(0, 200, 200_000), rng.uniform(0, 100, 200_000)].astype(np.float32)
    xy[:20_000, 0] = rng.uniform(99.9, 100.0, 20_000).astype(np.float32)
    verts = np.array([[0, 0], [100, 0], [100, 100], [0, 100],
                      [99.9, 0], [200, 0], [200, 100], [99.9, 100]], np.float32)
    pidx = np.array([0, 4, 8], np.int32)
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, xy)
    dh.setPolygons(verts, pidx)
    handler.setDataHandler(dh)
    for cell in (10.0, 0.05, 10.0):
        handler.setCellSize(cell)
        got = handler.execute(rj.RasterJoinFn)
        want, _, _ = oracle.raster_join(xy, verts, pidx, cell)
        np.testing.assert_array_equal(got.count, want)


@pytest.mark.parametrize("cell", [800.0, 450.0, 120.0])
def test_canvas_splat_small_and_large_canvases(handler, c1, cell):
    """Canvas path (forced): shared-memory private canvases (<= 8192 pixels)
    and warp-merged global splats give the oracle's counts and sums."""
    pts, verts, pidx = c1
    dh = make_dh(pts, verts, pidx)
    dh.setAggregation(rj.Avg, 3)
    handler.setDataHandler(dh)
    handler.setCellSize(cell)
    handler.flags = rj.FLAG_FORCE_CANVAS
    try:
        got = handler.execute(rj.RasterJoinFn)
    finally:
        handler.flags = 0
    cols = ocols(pts)
    want = oracle.raster_join(pts["xy"], verts, pidx, cell, f=cols.filt(aggr_attrib=3))
    np.testing.assert_array_equal(got.count, want[0])
    check_sums(got.sum, want[1])


@pytest.mark.parametrize("fn", [rj.RasterJoinFn, rj.IndexJoinFn, rj.HybridJoinFn, rj.RasterJoinBoundFn])
def test_streamed_host_table_matches_resident(c1, fn, built):
    """A host-resident table streamed in chunks gives the resident table's
    results; the timing line counts the passes."""
    pts, verts, pidx = c1
    res = {}
    for mode in ("resident", "streamed"):
        h = rj.GLHandler()
        try:
            if mode == "resident":
                dh = make_dh(pts, verts, pidx)
            else:
                dh = rj.DataHandler()
                dh.setPolygons(verts, pidx)
                for aid, typ in ((2, rj.Uint), (3, rj.Float), (4, rj.Int), (5, rj.Int)):
                    dh.declare(aid, typ)
                h.attachHost([(1, rj.Location, pts["xy"]), (2, rj.Uint, pts["t"]), (3, rj.Float, pts["a"]),
                              (4, rj.Int, pts["f1"]), (5, rj.Int, pts["f2"])], len(pts["t"]), 1, 100_000)
            c2_query(dh)
            h.setDataHandler(dh)
            h.setCellSize(40.0)
            h.setPolyIndexResolution(256)
            r = h.execute(fn)
            res[mode] = (r.count.copy(), r.sum.copy(), None if r.bounds is None else r.bounds.copy())
            if mode == "streamed":
                assert h.timings()["no_pt_passes"] == (len(pts["t"]) + 99_999) // 100_000
        finally:
            h.close()
    for a, b in zip(res["resident"], res["streamed"]):
        if a is not None:
            np.testing.assert_array_equal(a, b)


def _raster(handler, cell, flags=0, max_fbo=8192):
    handler.setCellSize(cell)
    handler.flags = flags
    handler.max_fbo_size = max_fbo
    try:
        r = handler.execute(rj.RasterJoinFn)
        return r.count.copy(), r.sum.copy()
    finally:
        handler.flags = 0
        handler.max_fbo_size = 8192


def test_tiered_label_canvas_matches_flat_and_oracle(handler, c1):
    """64M-pixel canvas (cell 5 m): 16 x 16 block tiers in the label form give
    the flat canvas's and the oracle's results."""
    pts, verts, pidx = c1
    dh = make_dh(pts, verts, pidx)
    c2_query(dh)
    handler.setDataHandler(dh)
    tier = _raster(handler, 5.0)
    flat = _raster(handler, 5.0, rj.FLAG_FLAT_CANVAS)
    np.testing.assert_array_equal(tier[0], flat[0])
    np.testing.assert_array_equal(tier[1], flat[1])
    want = oracle.raster_join(pts["xy"], verts, pidx, 5.0, f=c2_filter(pts))
    np.testing.assert_array_equal(tier[0], want[0])
    check_sums(tier[1], want[1])


def test_tiered_canvas_form_overlapping_stars(handler, stars):
    """Overlapping polygons on a 100M-pixel canvas: block sums for full blocks,
    pixel canvases for mixed ones; identical to the flat canvas."""
    pts, verts, pidx = stars
    dh = make_dh(pts, verts, pidx)
    dh.setAggregation(rj.Avg, 3)
    handler.setDataHandler(dh)
    tier = _raster(handler, 4.0)
    flat = _raster(handler, 4.0, rj.FLAG_FLAT_CANVAS)
    np.testing.assert_array_equal(tier[0], flat[0])
    np.testing.assert_array_equal(tier[1], flat[1])
    assert tier[0].sum() > 0


def test_tiered_multi_tile_matches_flat(handler, c1):
    """3 x 3 tiles of 5334^2 pixels, label form, against the flat canvas."""
    pts, verts, pidx = c1
    handler.setDataHandler(make_dh(pts, verts, pidx))
    tier = _raster(handler, 2.5, max_fbo=6000)
    flat = _raster(handler, 2.5, rj.FLAG_FLAT_CANVAS, max_fbo=6000)
    np.testing.assert_array_equal(tier[0], flat[0])


@pytest.mark.parametrize("fn", [rj.IndexJoinFn, rj.HybridJoinFn])
def test_edge_test_counter(handler, c1, fn):
    """RJ_FLAG_COUNT_EDGE_TESTS counts the exact tests without changing the
    result; without the flag the count stays 0."""
    pts, verts, pidx = c1
    handler.setDataHandler(make_dh(pts, verts, pidx))
    handler.setPolyIndexResolution(256)
    base = handler.execute(fn)
    assert handler.timings()["edge_tests"] == 0
    handler.flags = rj.FLAG_COUNT_EDGE_TESTS
    try:
        got = handler.execute(fn)
        n = handler.timings()["edge_tests"]
    finally:
        handler.flags = 0
    np.testing.assert_array_equal(got.count, base.count)
    assert 0 < n < 1000 * len(pts["xy"])
