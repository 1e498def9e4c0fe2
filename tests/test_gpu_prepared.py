"""Prepared queries (rj_prepare / rj_execute_prepared): the device work of one
query captured as a CUDA graph and replayed gives rj_execute's results bit for
bit; in-place table reloads keep the plan valid, other changes invalidate it;
queries that read values back to the host mid-way are refused."""
import numpy as np
import pytest

import oracle
import rasterjoin as rj
from rasterjoin import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def data():
    pts = synth.points(400_001, seed=51, columns=True)
    verts, pidx = synth.voronoi_polygons(260, seed=20261203)
    return pts, verts, pidx


def _dh(pts, verts, pidx, xy=None, a=None):
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, pts["xy"] if xy is None else xy)
    dh.add_column(2, rj.Uint, pts["t"])
    dh.add_column(3, rj.Float, pts["a"] if a is None else a)
    dh.add_column(4, rj.Int, pts["f1"])
    dh.setPolygons(verts, pidx)
    return dh


def _same(a, b):
    np.testing.assert_array_equal(a.count, b.count)
    assert a.sum.tobytes() == b.sum.tobytes()


@pytest.mark.parametrize("fn,flags,filters", [
    (rj.RasterJoinFn, rj.FLAG_NO_CACHE, False),      # the headline's step: label map rebuilt every replay
    (rj.RasterJoinFn, 0, True),                      # filters + avg through the lean pass
    (rj.RasterJoinBoundFn, 0, False),                # canvas + polygon pass + error bounds
    (rj.HybridJoinFn, 0, True),                      # cached classified grid, lean hybrid pass
    (rj.IndexJoinFn, 0, True),
])
def test_replay_equals_execute(handler, data, fn, flags, filters):
    pts, verts, pidx = data
    dh = _dh(pts, verts, pidx)
    if filters:
        dh.setQueryConstraints([(4, rj.GT, 2)])
        dh.setTimeRange(2, synth.T0, synth.T0 + synth.YEAR // 2)
        dh.setAggregation(rj.Avg, 3)
    handler.setDataHandler(dh)
    handler.setCellSize(10.0)
    handler.setPolyIndexResolution(256)
    handler.flags = flags
    try:
        want = handler.execute(fn)
        plan = handler.prepare(fn)
        try:
            for _ in range(3):
                got = plan.execute()
                _same(got, want)
                if fn == rj.RasterJoinBoundFn:
                    np.testing.assert_array_equal(got.bounds, want.bounds)
        finally:
            plan.close()
    finally:
        handler.flags = 0
    if fn == rj.RasterJoinFn and not filters:
        np.testing.assert_array_equal(want.count, oracle.raster_join(pts["xy"], verts, pidx, 10.0)[0])


def test_in_place_reload_keeps_the_plan(handler, data):
    """rj_load_points with the same columns and size copies into the plan's
    buffers: a replay joins the new rows (equal to a fresh rj_execute)."""
    pts, verts, pidx = data
    dh = _dh(pts, verts, pidx)
    handler.setDataHandler(dh)
    handler.setCellSize(10.0)
    handler.flags = rj.FLAG_NO_CACHE
    try:
        plan = handler.prepare(rj.RasterJoinFn)
        try:
            other = synth.points(len(pts["xy"]), seed=52)["xy"]
            dh.add_column(1, rj.Location, other)          # the same polygons stay on the device
            handler.upload()                              # same layout: copied in place
            got = plan.execute()
            want = handler.execute(rj.RasterJoinFn)
            np.testing.assert_array_equal(got.count, want.count)
            np.testing.assert_array_equal(got.count, oracle.raster_join(other, verts, pidx, 10.0)[0])
            # a table of another size reallocates: the plan refuses
            handler.setDataHandler(_dh({k: v[:1000] for k, v in pts.items()}, verts, pidx))
            handler.upload()
            with pytest.raises(rj.RJError) as ei:
                plan.execute()
            assert ei.value.code == -1
        finally:
            plan.close()
    finally:
        handler.flags = 0


def test_queries_needing_readbacks_are_refused(handler, data):
    pts, verts, pidx = data
    handler.setDataHandler(_dh(pts, verts, pidx))
    handler.setPolyIndexResolution(256)
    handler.flags = rj.FLAG_NO_CACHE                  # the hybrid rebuilds its grid every call
    try:
        with pytest.raises(rj.RJError) as ei:
            handler.prepare(rj.HybridJoinFn)
        assert ei.value.code == -7
        handler.flags = 0
        handler.setCellSize(1.0)                      # 40000 px: tiered canvas, slot count read back
        with pytest.raises(rj.RJError) as ei:
            handler.prepare(rj.RasterJoinFn)
        assert ei.value.code == -7
        got = handler.execute(rj.RasterJoinFn)        # the context still joins
        assert got.count.sum() > 0
    finally:
        handler.flags = 0
        handler.setCellSize(10.0)


def test_reload_refuses_plans_narrowed_by_the_time_index(handler, data):
    """A reload in place drops the time index: a plan whose rows it narrowed
    is refused, a plan over every row stays valid."""
    pts, verts, pidx = data
    dh = _dh(pts, verts, pidx)
    handler.setDataHandler(dh)
    handler.upload(force=True)
    handler.buildTimeIndex(2)
    handler.setCellSize(10.0)
    try:
        plan_all = handler.prepare(rj.RasterJoinFn)
        dh.setTimeRange(2, synth.T0, synth.T0 + synth.YEAR // 4)
        plan_t = handler.prepare(rj.RasterJoinFn)
        try:
            other = synth.points(len(pts["xy"]), seed=53)["xy"]
            dh.add_column(1, rj.Location, other)
            handler.upload()                              # same layout: copied in place
            got = plan_all.execute()
            np.testing.assert_array_equal(got.count, oracle.raster_join(other, verts, pidx, 10.0)[0])
            with pytest.raises(rj.RJError) as ei:
                plan_t.execute()
            assert ei.value.code == -1
        finally:
            plan_t.close()
            plan_all.close()
    finally:
        handler.setDataHandler(_dh(pts, verts, pidx))
        handler.upload(force=True)
