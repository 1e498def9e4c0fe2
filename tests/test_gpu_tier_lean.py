"""Lean point pass over tiered canvases (16 x 16-pixel blocks), label and
canvas forms, one tile and several: every shape gives the oracle's results
bit for bit (sums within 1e-6), including points on and around the tile seams
(which the reference counts in every tile whose window holds them) and points
off the canvas."""
import numpy as np
import pytest

import oracle
import rasterjoin as rj
from rasterjoin import synth

pytestmark = pytest.mark.gpu

BOX = 6000.0          # metres: about 6000 x 6000 pixels at 1 m (tiered from 2^24 pixels)


def _table(n, seed, seam_x, seam_y):
    pts = synth.points(n, seed=seed, box=BOX, columns=True)
    xy = pts["xy"].copy()
    rng = np.random.default_rng(seed)
    # points on, just left and just right of every seam line, and off the canvas
    k = 0
    offs = np.array([0.0, 1e-3, -1e-3, 0.25, -0.25, 0.5, -0.5, 0.75, -0.75, 1.0, -1.0], np.float32)
    for sx in seam_x:
        for o in offs:
            xy[k] = (sx + o, rng.uniform(0, BOX)); k += 1
    for sy in seam_y:
        for o in offs:
            xy[k] = (rng.uniform(0, BOX), sy + o); k += 1
    for sx in seam_x:
        for sy in seam_y:
            for o in offs[:5]:
                xy[k] = (sx + o, sy - o); k += 1
    specials = np.array([[np.nan, 10.0], [10.0, np.nan], [np.inf, 5.0], [-1e30, 3.0], [-0.004, 200.0],
                         [BOX + 0.004, 300.0], [9000.0, 9000.0]], np.float32)
    xy[k:k + len(specials)] = specials
    pts["xy"] = xy
    return pts


@pytest.fixture(scope="module")
def sets():
    vor = synth.voronoi_polygons(40, seed=77, box=BOX, verts_per_poly=40, jitter=5.0)
    stars = synth.star_polygons(25, seed=78, box=BOX, vmin=6, vmax=60, rmin=100, rmax=900)
    return {"voronoi": vor, "stars": stars}


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


# one tile (fbo 8192) and 3 x 3 tiles of 2100 pixels
@pytest.mark.parametrize("fbo", [8192, 2100])
@pytest.mark.parametrize("name", ["voronoi", "stars"])
@pytest.mark.parametrize("filters", [False, True])
def test_every_tier_shape_matches_oracle(handler, sets, fbo, name, filters):
    verts, pidx = sets[name]
    bb = (verts[:, 0].min(), verts[:, 1].min())
    seams_x = [float(bb[0]) + k * fbo * 1.0 for k in (1, 2)] if fbo < 8192 else []
    seams_y = [float(bb[1]) + k * fbo * 1.0 for k in (1, 2)] if fbo < 8192 else []
    pts = _table(200_003, 79, seams_x, seams_y)
    handler.setDataHandler(_dh(pts, verts, pidx, filters))
    handler.setCellSize(1.0)
    handler.max_fbo_size = fbo
    cols = oracle.Columns({2: (oracle.Uint, pts["t"]), 3: (oracle.Float, pts["a"]), 4: (oracle.Int, pts["f1"])})
    f = cols.filt([(4, oracle.GT, 2)], aggr_attrib=3, time_range=(2, synth.T0, synth.T0 + synth.YEAR // 2)) \
        if filters else None
    want = oracle.raster_join(pts["xy"], verts, pidx, 1.0, f=f, max_res=fbo)
    handler.flags = rj.FLAG_TIERED_CANVAS
    taken = 0
    try:
        for sh in range(3):
            handler.setTuning(rj.TUNE_COUNT_SHAPE, sh)
            got = handler.execute(rj.RasterJoinFn)
            np.testing.assert_array_equal(got.count, want[0], err_msg="shape %d" % sh)
            if filters:
                np.testing.assert_allclose(got.sum, want[1], rtol=1e-6, atol=1e-9 * max(1.0, float(np.abs(want[1]).max())))
            taken += handler.getTuning(rj.TUNE_COUNT_SHAPE) == sh
        handler.setTuning(rj.TUNE_COUNT_SHAPE, -1)
        got = handler.execute(rj.RasterJoinFn)                       # autotuned
        np.testing.assert_array_equal(got.count, want[0])
    finally:
        handler.setTuning(rj.TUNE_COUNT_SHAPE, -1)
        handler.flags = 0
        handler.max_fbo_size = 8192
    assert taken == 3
    assert want[0].sum() > 0


@pytest.mark.parametrize("fbo", [8192, 2100])
@pytest.mark.parametrize("name", ["voronoi", "stars"])
@pytest.mark.parametrize("line_filter", [False, True])
def test_tiered_error_bounds_match_oracle(handler, sets, fbo, name, line_filter):
    """The error-bounds join on a tiered canvas: the blocks within two pixels
    of an edge keep per-pixel counts, so the outline pass reads the same
    counts as on a flat canvas; counts and bounds equal the oracle's, with and
    without the reference's 0.5 px fragment filter, on one tile and 3 x 3."""
    verts, pidx = sets[name]
    bb = (verts[:, 0].min(), verts[:, 1].min())
    seams_x = [float(bb[0]) + k * fbo * 1.0 for k in (1, 2)] if fbo < 8192 else []
    seams_y = [float(bb[1]) + k * fbo * 1.0 for k in (1, 2)] if fbo < 8192 else []
    pts = _table(200_003, 83, seams_x, seams_y)
    handler.setDataHandler(_dh(pts, verts, pidx, False))
    handler.setCellSize(1.0)
    handler.max_fbo_size = fbo
    want = oracle.raster_join(pts["xy"], verts, pidx, 1.0, max_res=fbo, bounds=True, line_filter=line_filter)
    handler.flags = rj.FLAG_TIERED_CANVAS | (rj.FLAG_LINE_FILTER if line_filter else 0)
    try:
        got = handler.execute(rj.RasterJoinBoundFn)
        flat_flags = rj.FLAG_FLAT_CANVAS | (rj.FLAG_LINE_FILTER if line_filter else 0)
        handler.flags = flat_flags
        flat = handler.execute(rj.RasterJoinBoundFn)
    finally:
        handler.flags = 0
        handler.max_fbo_size = 8192
    np.testing.assert_array_equal(got.count, want[0])
    np.testing.assert_array_equal(got.bounds, want[2])
    np.testing.assert_array_equal(flat.bounds, want[2])


def _crowded_sets():
    """Polygons that crowd one band of 16 rows: a sawtooth 4000 px long whose
    teeth (8 px wide, 8 px high) put a crossing inside every block of its band
    (250 listed blocks: four rounds of 64), and a star of 1,200 vertices 120 px
    across (more than 256 edges in a band: the edges are read from global
    memory).  Two small triangles stretch the canvas past 2^24 pixels.  Set
    "apart" has no overlaps (label form); "frame" adds a square over most of
    the canvas (canvas form)."""
    k = np.arange(501)
    teeth = np.c_[1000.0 + 8.0 * k, 3000.0 + np.where(k % 2 == 1, 4.0, -4.0) + 0.37]
    saw = np.r_[teeth, [[5000.0, 2900.25], [1000.0, 2900.25]]]
    n = 1200
    ang = 2 * np.pi * np.arange(n) / n
    rad = np.where(np.arange(n) % 2 == 0, 60.0, 20.0)
    star = np.c_[3000.3 + rad * np.cos(ang), 4500.6 + rad * np.sin(ang)]
    t1 = np.array([[5900.0, 100.0], [5990.0, 100.0], [5950.0, 150.0]])
    t2 = np.array([[100.0, 5900.0], [150.0, 5950.0], [100.0, 5950.0]])
    frame = np.array([[500.0, 500.0], [5500.0, 500.0], [5500.0, 5500.0], [500.0, 5500.0]])

    def pack(polys):
        v = np.concatenate(polys).astype(np.float32)
        pidx = np.r_[0, np.cumsum([len(q) for q in polys])].astype(np.int32)
        return v, pidx
    return {"apart": pack([saw, star, t1, t2]), "frame": pack([saw, star, t1, t2, frame])}


@pytest.mark.parametrize("fbo", [8192, 2100])
@pytest.mark.parametrize("name", ["apart", "frame"])
def test_crowded_bands_match_oracle(handler, fbo, name):
    verts, pidx = _crowded_sets()[name]
    rng = np.random.default_rng(91)
    xy = np.r_[rng.uniform(0, BOX, (300_000, 2)),
               np.c_[rng.uniform(990, 5010, 200_000), rng.uniform(2890, 3012, 200_000)],
               np.c_[rng.normal(3000.3, 40, 100_000), rng.normal(4500.6, 40, 100_000)]].astype(np.float32)
    pts = synth.points(len(xy), seed=92, box=BOX, columns=True)
    pts["xy"] = xy
    handler.setDataHandler(_dh(pts, verts, pidx, False))
    handler.setCellSize(1.0)
    handler.max_fbo_size = fbo
    want = oracle.raster_join(xy, verts, pidx, 1.0, max_res=fbo, bounds=True)
    try:
        handler.flags = rj.FLAG_TIERED_CANVAS
        got = handler.execute(rj.RasterJoinFn)
        bnd = handler.execute(rj.RasterJoinBoundFn)
        handler.flags = rj.FLAG_FLAT_CANVAS
        flat = handler.execute(rj.RasterJoinFn)
    finally:
        handler.flags = 0
        handler.max_fbo_size = 8192
    np.testing.assert_array_equal(got.count, want[0])
    np.testing.assert_array_equal(flat.count, want[0])
    np.testing.assert_array_equal(bnd.count, want[0])
    np.testing.assert_array_equal(bnd.bounds, want[2])
    assert want[0][:2].min() > 0
