"""The GPU against the committed golden fixtures (tests/golden/, inputs and
expected outputs stored together, generated by make_golden.py from the CPU
oracle): index joins with and without the reference's grid clamp, the hybrid
join, the index join against CPUJoin's counts, filters with avg, the raster
and error-bounds joins, and a multi-tile canvas.  Counts and bounds bit for
bit, sums within 1e-6 relative."""
import os

import numpy as np
import pytest

import rasterjoin as rj
from rasterjoin import synth

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _dh(g, filters):
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, g["xy"])
    dh.add_column(2, rj.Uint, g["t"])
    dh.add_column(3, rj.Float, g["a"])
    dh.add_column(4, rj.Int, g["f1"])
    dh.add_column(5, rj.Int, g["f2"])
    dh.setPolygons(g["verts"], g["pindex"])
    if filters:
        dh.setQueryConstraints([(4, rj.GT, 2), (5, rj.LT, 8), (3, rj.LT, 50.0)])
        dh.setTimeRange(2, synth.T0, synth.T0 + synth.YEAR // 2)
        dh.setAggregation(rj.Avg, 3)
    return dh


@pytest.mark.parametrize("name", ["voronoi", "stars"])
def test_golden_fixture(handler, name):
    g = dict(np.load(os.path.join(HERE, "golden_%s.npz" % name)))

    def run(fn, filters=False, grid=64, cell=50.0, fbo=8192, flags=0):
        handler.setDataHandler(_dh(g, filters))
        handler.setPolyIndexResolution(grid)
        handler.setCellSize(cell)
        handler.max_fbo_size = fbo
        handler.flags = flags
        try:
            return handler.execute(fn)
        finally:
            handler.flags = 0
            handler.max_fbo_size = 8192

    np.testing.assert_array_equal(run(rj.IndexJoinFn).count, g["index64_count"])
    np.testing.assert_array_equal(run(rj.IndexJoinFn, flags=rj.FLAG_COMPAT_INDEX_CLAMP).count,
                                  g["index64_clamp_count"])
    np.testing.assert_array_equal(run(rj.HybridJoinFn).count, g["hybrid64_count"])
    np.testing.assert_array_equal(run(rj.IndexJoinFn, grid=256).count, g["cpujoin256_count"])
    r = run(rj.IndexJoinFn, filters=True)
    np.testing.assert_array_equal(r.count, g["index64_filt_count"])
    np.testing.assert_allclose(r.sum, g["index64_filt_sum"], rtol=1e-6, atol=1e-9)
    np.testing.assert_array_equal(run(rj.RasterJoinFn).count, g["raster50_count"])
    r = run(rj.RasterJoinBoundFn)
    np.testing.assert_array_equal(r.count, g["raster50_count"])
    np.testing.assert_array_equal(r.bounds, g["raster50_bounds"])
    r = run(rj.RasterJoinFn, filters=True)
    np.testing.assert_array_equal(r.count, g["raster50_filt_count"])
    np.testing.assert_allclose(r.sum, g["raster50_filt_sum"], rtol=1e-6, atol=1e-9)
    np.testing.assert_array_equal(run(rj.RasterJoinFn, cell=20.0, fbo=700).count, g["raster20_tiles_count"])
