"""Lean raster pass onto a point canvas (one canvas tile): polygon sets whose
coverage overlaps on the canvas, forced canvases and the error-bounds join.
Every shape -- canvas copies in shared memory, or atomics into the canvas in
global memory -- gives the oracle's counts bit for bit, sums within 1e-6 and
error bounds exactly, on tables with odd sizes and with points outside the
canvas (NaN, infinities, far away, on the canvas edges)."""
import numpy as np
import pytest

import oracle
import rasterjoin as rj
from rasterjoin import synth

pytestmark = pytest.mark.gpu

SUM_RTOL = 1e-6


def _with_specials(xy, seed):
    xy = xy.copy()
    rng = np.random.default_rng(seed)
    bad = rng.choice(len(xy), size=min(len(xy), 64), replace=False)
    specials = np.array([[np.nan, 10.0], [10.0, np.nan], [np.inf, 5.0], [-np.inf, 5.0], [1e30, 1e30],
                         [-1e30, 3.0], [0.0, 0.0], [40000.0, 40000.0], [0.0, 39999.996], [39999.996, 0.0],
                         [-0.004, 20000.0], [20000.0, -0.004]], np.float32)
    for k, i in enumerate(bad):
        xy[i] = specials[k % len(specials)]
    return xy


@pytest.fixture(scope="module")
def table():
    pts = synth.points(600_001, seed=41, columns=True)
    pts["xy"] = _with_specials(pts["xy"], 41)
    return pts


@pytest.fixture(scope="module")
def stars():
    return synth.star_polygons(40, seed=43, vmin=8, vmax=60, rmin=1000, rmax=6000)


def _dh(pts, verts, pidx, filters):
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, pts["xy"])
    dh.add_column(2, rj.Uint, pts["t"])
    dh.add_column(3, rj.Float, pts["a"])
    dh.add_column(4, rj.Int, pts["f1"])
    dh.setPolygons(verts, pidx)
    if filters:
        dh.setQueryConstraints([(4, rj.GT, 2)])
        dh.setTimeRange(2, synth.T0, synth.T0 + synth.YEAR // 2)
        dh.setAggregation(rj.Avg, 3)
    return dh


def _want(pts, verts, pidx, cell, filters, bounds=False):
    cols = oracle.Columns({2: (oracle.Uint, pts["t"]), 3: (oracle.Float, pts["a"]), 4: (oracle.Int, pts["f1"])})
    f = cols.filt([(4, oracle.GT, 2)], aggr_attrib=3, time_range=(2, synth.T0, synth.T0 + synth.YEAR // 2)) \
        if filters else None
    return oracle.raster_join(pts["xy"], verts, pidx, cell, f=f, bounds=bounds)


def _check_sums(got, want):
    np.testing.assert_allclose(got, want, rtol=SUM_RTOL, atol=1e-9 * max(1.0, float(np.abs(want).max())))


# 400 m: a 100 x 100 canvas, whose copies fit in shared memory (count and
# sum); 10 m: 4000 x 4000, atomics into the global canvas only
@pytest.mark.parametrize("cell", [400.0, 10.0])
@pytest.mark.parametrize("filters", [False, True])
def test_every_splat_shape_matches_oracle(handler, table, stars, cell, filters):
    verts, pidx = stars
    handler.setDataHandler(_dh(table, verts, pidx, filters))
    handler.setCellSize(cell)
    want = _want(table, verts, pidx, cell, filters)
    nshapes = handler.getTuning(rj.TUNE_SPLAT_SHAPES)
    assert nshapes >= 2
    taken = set()
    handler.flags = rj.FLAG_FORCE_CANVAS
    try:
        for sh in range(nshapes):
            handler.setTuning(rj.TUNE_COUNT_SHAPE, sh)
            got = handler.execute(rj.RasterJoinFn)
            np.testing.assert_array_equal(got.count, want[0], err_msg="shape %d" % sh)
            if filters:
                _check_sums(got.sum, want[1])
            ran = handler.getTuning(rj.TUNE_COUNT_SHAPE)
            assert ran in (sh, -1)
            if ran == sh:
                taken.add(sh)
        # the global-atomic shapes always apply; the shared-memory ones when
        # the canvas fits
        assert len(taken) >= (nshapes if cell == 400.0 else nshapes // 2)
        handler.setTuning(rj.TUNE_COUNT_SHAPE, -1)
        got = handler.execute(rj.RasterJoinFn)         # autotuned
        np.testing.assert_array_equal(got.count, want[0])
        assert handler.getTuning(rj.TUNE_COUNT_SHAPE) >= 0
    finally:
        handler.setTuning(rj.TUNE_COUNT_SHAPE, -1)
        handler.flags = 0


@pytest.mark.parametrize("cell", [400.0, 10.0])
def test_error_bounds_through_the_lean_splat(handler, table, stars, cell):
    verts, pidx = stars
    handler.setDataHandler(_dh(table, verts, pidx, False))
    handler.setCellSize(cell)
    want = _want(table, verts, pidx, cell, False, bounds=True)
    got = handler.execute(rj.RasterJoinBoundFn)
    assert handler.getTuning(rj.TUNE_COUNT_SHAPE) >= 0   # the lean splat ran
    np.testing.assert_array_equal(got.count, want[0])
    np.testing.assert_array_equal(got.bounds, want[2])


def test_forced_canvas_on_a_partition(handler, table):
    """Polygons that do not overlap, forced onto the canvas path."""
    verts, pidx = synth.voronoi_polygons(260, seed=20261203)
    handler.setDataHandler(_dh(table, verts, pidx, True))
    handler.setCellSize(10.0)
    handler.flags = rj.FLAG_FORCE_CANVAS
    try:
        got = handler.execute(rj.RasterJoinFn)
        assert handler.getTuning(rj.TUNE_COUNT_SHAPE) >= 0
    finally:
        handler.flags = 0
    want = _want(table, verts, pidx, 10.0, True)
    np.testing.assert_array_equal(got.count, want[0])
    _check_sums(got.sum, want[1])


@pytest.mark.parametrize("n", [0, 1, 2, 3, 5, 4097, 65539])
def test_small_and_ragged_tables(handler, table, stars, n):
    verts, pidx = stars
    pts = {k: v[:n] for k, v in table.items()}
    handler.setDataHandler(_dh(pts, verts, pidx, True))
    handler.setCellSize(400.0)
    got = handler.execute(rj.RasterJoinFn)
    if n == 0:
        assert got.count.sum() == 0
        return
    want = _want(pts, verts, pidx, 400.0, True)
    np.testing.assert_array_equal(got.count, want[0])
    _check_sums(got.sum, want[1])
