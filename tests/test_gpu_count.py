"""Lean raster count pass (one canvas tile, polygon label map, no filter,
count only): every kernel shape and every block-code size gives the oracle's
counts bit for bit, on tables with odd sizes and with points outside the
canvas (NaN, infinities, far away, on the canvas edges)."""
import numpy as np
import pytest

import oracle
import rasterjoin as rj
from rasterjoin import synth

pytestmark = pytest.mark.gpu


def _table(n, seed):
    xy = synth.points(n, seed=seed)["xy"].copy()
    rng = np.random.default_rng(seed)
    bad = rng.choice(n, size=min(n, 64), replace=False)
    specials = np.array([[np.nan, 10.0], [10.0, np.nan], [np.inf, 5.0], [-np.inf, 5.0], [1e30, 1e30],
                         [-1e30, 3.0], [0.0, 0.0], [40000.0, 40000.0], [0.0, 39999.996], [39999.996, 0.0],
                         [-0.004, 20000.0], [20000.0, -0.004]], np.float32)
    for k, i in enumerate(bad):
        xy[i] = specials[k % len(specials)]
    return xy


def _handler_for(handler, xy, verts, pidx):
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, xy)
    dh.setPolygons(verts, pidx)
    handler.setDataHandler(dh)
    handler.setCellSize(10.0)


@pytest.fixture(scope="module")
def voronoi():
    return synth.voronoi_polygons(260, seed=20261203)


def test_every_shape_and_block_size_matches_oracle(handler, voronoi):
    verts, pidx = voronoi
    xy = _table(1_000_003, 31)
    _handler_for(handler, xy, verts, pidx)
    want, _, _ = oracle.raster_join(xy, verts, pidx, 10.0)
    nshapes = handler.getTuning(rj.TUNE_COUNT_SHAPES)
    assert nshapes >= 2
    taken = 0
    try:
        for bs in (4, 5, 6):
            handler.setTuning(rj.TUNE_COUNT_BLOCK_SHIFT, bs)
            for sh in range(nshapes):
                handler.setTuning(rj.TUNE_COUNT_SHAPE, sh)
                got = handler.execute(rj.RasterJoinFn)
                np.testing.assert_array_equal(got.count, want, err_msg="shape %d, block shift %d" % (sh, bs))
                ran = handler.getTuning(rj.TUNE_COUNT_SHAPE)
                assert ran in (sh, -1)
                if ran == sh:
                    assert handler.getTuning(rj.TUNE_COUNT_BLOCK_SHIFT) == bs
                    taken += 1
    finally:
        handler.setTuning(rj.TUNE_COUNT_SHAPE, -1)
        handler.setTuning(rj.TUNE_COUNT_BLOCK_SHIFT, -1)
    assert taken >= 2 * nshapes          # every shape fits at the coarser block sizes
    # autotuned: the tuner times the candidates into scratch, then runs one
    got = handler.execute(rj.RasterJoinFn)
    np.testing.assert_array_equal(got.count, want)
    assert handler.getTuning(rj.TUNE_COUNT_SHAPE) >= 0
    got = handler.execute(rj.RasterJoinFn)           # the kept choice
    np.testing.assert_array_equal(got.count, want)


@pytest.mark.parametrize("n", [0, 1, 2, 3, 5, 4097, 65539])
def test_small_and_ragged_tables(handler, voronoi, n):
    verts, pidx = voronoi
    xy = _table(max(n, 1), 7 + n)[:n] if n else np.zeros((0, 2), np.float32)
    _handler_for(handler, xy, verts, pidx)
    want = oracle.raster_join(xy, verts, pidx, 10.0)[0] if n else np.zeros(len(pidx) - 1, np.uint64)
    got = handler.execute(rj.RasterJoinFn)
    np.testing.assert_array_equal(got.count, want)


def test_lean_pass_is_taken_only_where_it_applies(handler, voronoi):
    """Filters, avg and multi-tile canvases keep the generic pass (and its results)."""
    verts, pidx = voronoi
    pts = synth.points(200_001, seed=3, columns=True)
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, pts["xy"])
    dh.add_column(4, rj.Int, pts["f1"])
    dh.setPolygons(verts, pidx)
    handler.setDataHandler(dh)
    handler.setCellSize(10.0)
    handler.execute(rj.RasterJoinFn)
    assert handler.getTuning(rj.TUNE_COUNT_SHAPE) >= 0
    dh.setQueryConstraints([(4, rj.GT, 2)])
    got = handler.execute(rj.RasterJoinFn)
    assert handler.getTuning(rj.TUNE_COUNT_SHAPE) == -1
    f = oracle.Columns({4: (oracle.Int, pts["f1"])}).filt([(4, rj.GT, 2)])
    np.testing.assert_array_equal(got.count, oracle.raster_join(pts["xy"], verts, pidx, 10.0, f=f)[0])
    dh.setQueryConstraints([])
    handler.max_fbo_size = 2048         # 4000 px across: 2 x 2 tiles of 2000 px
    try:
        got = handler.execute(rj.RasterJoinFn)
        assert handler.getTuning(rj.TUNE_COUNT_SHAPE) == -1
    finally:
        handler.max_fbo_size = 8192
    np.testing.assert_array_equal(got.count, oracle.raster_join(pts["xy"], verts, pidx, 10.0, max_res=2048)[0])
