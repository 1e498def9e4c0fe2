"""Failure handling through the C ABI: every failure comes back as a status
code with a message, nothing exits the process, and the context stays usable
afterwards.  The reference exit(0)s or returns an empty vector on these
(GLData.cpp:18-23, GLFunction.cpp:251-252, GLHandler.cpp:190-203).

The faults are made on the host (a memory budget too small, malformed
polygons, bad arguments) or with a bounded device wait that nothing can
satisfy (rj_selftest_bounded_wait); none of them faults the GPU."""
import ctypes as C

import numpy as np
import pytest

import oracle
import rasterjoin as rj
from rasterjoin import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small():
    pts = synth.points(200_001, seed=41)
    verts, pidx = synth.voronoi_polygons(40, seed=41)
    return pts["xy"], verts, pidx


def _join(h, xy, verts, pidx):
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, xy)
    dh.setPolygons(verts, pidx)
    h.setDataHandler(dh)
    h.setCellSize(50.0)
    return h.execute(rj.RasterJoinFn)


def _expect(code, fn, *args):
    with pytest.raises(rj.RJError) as ei:
        fn(*args)
    assert ei.value.code == code, ei.value
    return str(ei.value)


def test_memory_budget_exceeded_then_usable(small):
    """gpu_mem_mb (GLHandler::getInstance's budget, GLHandler.cpp:43-54): a table
    larger than the budget is refused with RJ_E_OOM, a smaller one then works."""
    xy, verts, pidx = small
    h = rj.GLHandler(gpu_mem_mb=8)
    try:
        big = np.tile(xy, (8, 1))                       # 12.8 MB of locations > 8 MB
        msg = _expect(-2, _join, h, big, verts, pidx)
        assert "budget" in msg
        got = _join(h, xy[:50_000], verts, pidx)          # 400 KB + a 1.3 MB label map fit
        np.testing.assert_array_equal(got.count, oracle.raster_join(xy[:50_000], verts, pidx, 50.0)[0])
    finally:
        h.close()


@pytest.mark.parametrize("case", ["non_monotone", "nan_vertex", "inf_vertex", "first_not_zero", "no_polygons",
                                  "empty_bounds"])
def test_malformed_polygons_refused(handler, small, case):
    xy, verts, pidx = small
    v, p = verts.copy(), pidx.copy()
    if case == "non_monotone":
        p[5], p[6] = p[6], p[5]
    elif case == "nan_vertex":
        v[17, 0] = np.nan
    elif case == "inf_vertex":
        v[3, 1] = np.inf
    elif case == "first_not_zero":
        p = p + 1
    elif case == "no_polygons":
        p = np.zeros(1, np.int32)
    elif case == "empty_bounds":
        v = np.ones_like(v)
    _expect(-1, _join, handler, xy, v, p)
    # the context still joins a valid set
    got = _join(handler, xy, verts, pidx)
    np.testing.assert_array_equal(got.count, oracle.raster_join(xy, verts, pidx, 50.0)[0])


def test_bad_arguments_refused(handler, small):
    xy, verts, pidx = small
    _join(handler, xy, verts, pidx)
    lib = handler.lib
    P = len(pidx) - 1
    # result buffers sized for another polygon set
    q = handler.make_query(rj.RasterJoinFn)
    res = rj.Result()
    res.npolys = P + 1
    assert lib.rj_execute(handler.ctx, C.byref(q), C.byref(res)) == -1
    # unknown join type (GLHandler.cpp:201)
    q.function_type = 9
    res.npolys = 0
    assert lib.rj_execute(handler.ctx, C.byref(q), C.byref(res)) == -7
    # device columns must be 16-byte aligned
    cols = (rj.Column * 1)()
    cols[0].attrib_id, cols[0].type, cols[0].data = 1, rj.Location, C.c_void_p(0x1008)
    assert lib.rj_attach_points_device(handler.ctx, cols, 1, 10, 1) == -1
    # unknown tuning knob / value out of range
    assert lib.rj_set_tuning(handler.ctx, 99, 0) == -1
    assert lib.rj_set_tuning(handler.ctx, rj.TUNE_COUNT_BLOCK_SHIFT, 2) == -1
    assert b"block shift" in lib.rj_last_error(handler.ctx)
    # canvas tiles above the reference's 8192-pixel framebuffer (GLFunction.hpp:14)
    q = handler.make_query(rj.RasterJoinFn)
    q.max_fbo_size = 16384
    res = rj.Result()
    assert lib.rj_execute(handler.ctx, C.byref(q), C.byref(res)) == -1
    assert b"tile side" in lib.rj_last_error(handler.ctx)
    handler._loaded_points = None
    got = _join(handler, xy, verts, pidx)
    np.testing.assert_array_equal(got.count, oracle.raster_join(xy, verts, pidx, 50.0)[0])


def test_bounded_device_wait_times_out_and_context_survives(handler, small):
    """A bounded device wait that nothing completes returns RJ_E_TIMEOUT (the
    kernel returns once its wall-time limit has passed); joins on the context
    still work."""
    xy, verts, pidx = small
    lib = handler.lib
    for limit_us in (1, 1000, 100_000):
        rc = lib.rj_selftest_bounded_wait(handler.ctx, limit_us)
        assert rc == -4, rc
        assert b"ran out" in lib.rj_last_error(handler.ctx)
    assert lib.rj_selftest_bounded_wait(handler.ctx, 0) == -1
    got = _join(handler, xy, verts, pidx)
    np.testing.assert_array_equal(got.count, oracle.raster_join(xy, verts, pidx, 50.0)[0])


def test_pipeline_with_its_wait_limit_knob(handler, small):
    """The bulk-copy pipeline (RJ_TUNE_POINT_SHAPE 2) under the default and an
    explicit wait limit gives the oracle's result; the knob reads back."""
    xy, verts, pidx = small
    big = np.tile(xy, (20, 1))                          # 4M points: enough tiles for the pipeline
    want = oracle.raster_join(big, verts, pidx, 50.0)[0]
    try:
        handler.setTuning(rj.TUNE_POINT_SHAPE, 2)
        dh = rj.DataHandler()
        dh.add_column(1, rj.Location, big)
        dh.add_column(4, rj.Int, np.zeros(len(big), np.int32))
        dh.setPolygons(verts, pidx)
        dh.setQueryConstraints([(4, rj.EQ, 0)])
        handler.setDataHandler(dh)
        handler.setCellSize(50.0)
        handler.flags = rj.FLAG_COMPAT_FLOAT_EQ         # general predicate form: the generic point pass
        for limit_us in (1_000_000, 200_000):
            handler.setTuning(rj.TUNE_WAIT_LIMIT, limit_us)
            assert handler.getTuning(rj.TUNE_WAIT_LIMIT) == limit_us
            got = handler.execute(rj.RasterJoinFn)
            np.testing.assert_array_equal(got.count, want)
    finally:
        handler.flags = 0
        handler.setTuning(rj.TUNE_POINT_SHAPE, -1)
        handler.setTuning(rj.TUNE_WAIT_LIMIT, 1_000_000)
