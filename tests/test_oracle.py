"""CPU oracle: pinned against the reference's own known-answer fixture, the
committed golden fixtures, and cross-consistency between the restated joins."""
import os

import numpy as np
import pytest

import oracle
from rasterjoin import synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = [os.path.join(HERE, "golden", "golden_%s.npz" % n) for n in ("voronoi", "stars")]


def test_reference_kat_all_joins():
    """RasterJoin/test/baseline.hpp:139-217: squares [5.1,5.2]^2 and [4.9,5.1]^2,
    two points at (5.15,5.15) and three at (5,5): counts 2 and 3."""
    xy, (verts, pidx), expect = synth.kat_two_squares()
    np.testing.assert_array_equal(oracle.bruteforce(xy, verts, pidx)[0], expect)
    np.testing.assert_array_equal(oracle.bruteforce_f64(xy, verts, pidx)[0], expect)
    for res in (1, 16, 256):
        np.testing.assert_array_equal(oracle.index_join(xy, verts, pidx, res)[0], expect)
        np.testing.assert_array_equal(oracle.hybrid_join(xy, verts, pidx, res)[0], expect)
    np.testing.assert_array_equal(oracle.cpujoin(xy, verts, pidx, 1024)[0], expect)
    for cell in (0.01, 0.001):
        np.testing.assert_array_equal(oracle.raster_join(xy, verts, pidx, cell)[0], expect)


@pytest.mark.parametrize("path", GOLDEN)
def test_golden_fixtures_reproduce(path):
    d = np.load(path)
    xy, verts, pidx = d["xy"], d["verts"], d["pindex"]
    cols = oracle.Columns({2: (oracle.Uint, d["t"]), 3: (oracle.Float, d["a"]), 4: (oracle.Int, d["f1"]),
                           5: (oracle.Int, d["f2"])})
    f = cols.filt([(4, oracle.GT, 2), (5, oracle.LT, 8), (3, oracle.LT, 50.0)], aggr_attrib=3,
                  time_range=(2, synth.T0, synth.T0 + synth.YEAR // 2))
    np.testing.assert_array_equal(oracle.index_join(xy, verts, pidx, 64)[0], d["index64_count"])
    np.testing.assert_array_equal(oracle.index_join(xy, verts, pidx, 64, compat_clamp=True)[0],
                                  d["index64_clamp_count"])
    np.testing.assert_array_equal(oracle.hybrid_join(xy, verts, pidx, 64)[0], d["hybrid64_count"])
    np.testing.assert_array_equal(oracle.cpujoin(xy, verts, pidx, 256)[0], d["cpujoin256_count"])
    c, s = oracle.index_join(xy, verts, pidx, 64, f=f)
    np.testing.assert_array_equal(c, d["index64_filt_count"])
    np.testing.assert_allclose(s, d["index64_filt_sum"], rtol=1e-12)
    c, _, b = oracle.raster_join(xy, verts, pidx, 50.0, bounds=True)
    np.testing.assert_array_equal(c, d["raster50_count"])
    np.testing.assert_array_equal(b, d["raster50_bounds"])
    c, s, _ = oracle.raster_join(xy, verts, pidx, 50.0, f=f)
    np.testing.assert_array_equal(c, d["raster50_filt_count"])
    np.testing.assert_allclose(s, d["raster50_filt_sum"], rtol=1e-12)
    np.testing.assert_array_equal(oracle.raster_join(xy, verts, pidx, 20.0, max_res=700)[0],
                                  d["raster20_tiles_count"])


@pytest.fixture(scope="module")
def lite():
    pts = synth.points(200_000, seed=3, columns=True)
    verts, pidx = synth.voronoi_polygons(120, seed=3)
    return pts, verts, pidx


def test_exact_joins_agree(lite):
    pts, verts, pidx = lite
    xy = pts["xy"]
    brute, _ = oracle.bruteforce(xy, verts, pidx)
    assert brute.sum() == len(xy)      # the Voronoi cells tile the box: every point in exactly one
    np.testing.assert_array_equal(oracle.index_join(xy, verts, pidx, 256)[0], brute)
    np.testing.assert_array_equal(oracle.hybrid_join(xy, verts, pidx, 256)[0], brute)
    np.testing.assert_array_equal(oracle.cpujoin(xy, verts, pidx, 1024)[0], brute)
    c64, _ = oracle.bruteforce_f64(xy, verts, pidx)
    assert np.abs(c64.astype(np.int64) - brute.astype(np.int64)).sum() <= 4


def test_raster_converges_and_bounds_contain_exact(lite):
    pts, verts, pidx = lite
    xy = pts["xy"]
    exact, _ = oracle.index_join(xy, verts, pidx, 256)
    P = len(pidx) - 1
    errs = []
    for cell in (200.0, 50.0, 10.0):
        c, _, b = oracle.raster_join(xy, verts, pidx, cell, bounds=True)
        agg = c.astype(np.int64)
        lo, hi = agg - b[3 * P:], agg + b[2 * P:3 * P]
        ex = exact.astype(np.int64)
        assert np.all((ex >= lo) & (ex <= hi)), cell
        errs.append(np.abs(agg - ex).sum())
    assert errs[0] > errs[1] > errs[2]


def test_line_filter_keeps_fewer_pixels(lite):
    pts, verts, pidx = lite
    _, _, b_all = oracle.raster_join(pts["xy"], verts, pidx, 50.0, bounds=True)
    _, _, b_f = oracle.raster_join(pts["xy"], verts, pidx, 50.0, bounds=True, line_filter=True)
    assert np.all(b_f <= b_all) and b_f.sum() < b_all.sum()


def test_filters_and_time_range(lite):
    pts, verts, pidx = lite
    cols = oracle.Columns({2: (oracle.Uint, pts["t"]), 3: (oracle.Float, pts["a"]), 4: (oracle.Int, pts["f1"]),
                           5: (oracle.Int, pts["f2"])})
    lo, hi = synth.T0, synth.T0 + synth.YEAR // 2
    f = cols.filt([(4, oracle.GT, 2), (5, oracle.LTE, 7), (3, oracle.LT, 50.0)], aggr_attrib=3,
                  time_range=(2, lo, hi))
    c, s = oracle.bruteforce(pts["xy"], verts, pidx, f=f)
    m = (pts["f1"] > 2) & (pts["f2"] <= 7) & (pts["a"] < np.float32(50)) & (pts["t"] >= lo) & (pts["t"] <= hi)
    assert c.sum() == m.sum()
    np.testing.assert_allclose(s.sum(), pts["a"][m].astype(np.float64).sum(), rtol=1e-9)


@pytest.mark.parametrize("cell,expect", [
    (10.0, (1, 1, 4000, 4000)),                       # eps = 10 m as the pixel side: a 4000^2 canvas
    (10.0 / np.sqrt(2.0), (1, 1, 5657, 5657)),        # accuracy 10 m, GLFunction.cpp:26-30
    (1.0, (5, 5, 8000, 8000)),
    (1.0 / np.sqrt(2.0), (7, 7, 8082, 8082)),         # accuracy 1 m: 7x7 tiles of 8082^2 (RasterJoin.cpp:59-63)
])
def test_canvas_geometry(cell, expect):
    assert oracle.raster_geometry(np.array([0, 0, 40000.0, 40000.0]), cell) == expect


def test_compat_float_equality_semantics():
    """LTE/GTE equality as float compare of raw bits (points.vert:99,107) vs typed."""
    xy = np.array([[5.0, 5.0]] * 4, np.float32)
    verts, pidx = synth.kat_two_squares()[1]
    vals = np.array([1, 2, 3, -1], np.int32)
    cols = oracle.Columns({7: (oracle.Int, vals)})
    typed = oracle.bruteforce(xy, verts, pidx, f=cols.filt([(7, oracle.GTE, 2)]))[0]
    compat = oracle.bruteforce(xy, verts, pidx, f=cols.filt([(7, oracle.GTE, 2)], compat_float_eq=True))[0]
    assert typed.sum() == 2 and compat.sum() == 2     # same for small ints (distinct denormal patterns)
    # 0 and 0x80000000 (-0.0 as float) compare equal as floats but not as ints
    vals2 = np.array([0, -2147483648, 5, 6], np.int32)
    cols2 = oracle.Columns({7: (oracle.Int, vals2)})
    typed = oracle.bruteforce(xy, verts, pidx, f=cols2.filt([(7, oracle.GTE, 0)]))[0]
    compat = oracle.bruteforce(xy, verts, pidx, f=cols2.filt([(7, oracle.GTE, 0)], compat_float_eq=True))[0]
    assert typed.sum() == 3 and compat.sum() == 4


def _near_edges(verts, pidx, seed):
    """Points on the vertices, on the edges and 1e-4..0.5 m to either side."""
    rng = np.random.default_rng(seed)
    out = [verts.astype(np.float32)]
    for p in range(len(pidx) - 1):
        v = verts[pidx[p]:pidx[p + 1]].astype(np.float64)
        w = np.roll(v, -1, axis=0)
        d = w - v
        nrm = np.c_[-d[:, 1], d[:, 0]] / np.maximum(np.hypot(d[:, 0], d[:, 1]), 1e-9)[:, None]
        for t in rng.random(2):
            q = v + d * t
            for off in (0.0, 1e-4, -1e-4, 0.5, -0.5):
                out.append((q + off * nrm).astype(np.float32))
    return np.concatenate(out)


@pytest.mark.parametrize("seed", [11, 12])
def test_exact_joins_agree_on_overlapping_stars_near_edges(seed):
    """Concave, overlapping star polygons (each polygon counts on its own) and
    points placed on and next to every edge: the index, hybrid and CPUJoin
    restatements give the brute-force fp32 crossing-number counts exactly."""
    from rasterjoin import workloads
    rng = np.random.default_rng(seed)
    verts, pidx = workloads.star_set(rng, 40, 6, 60, 300.0, 4000.0)
    xy = np.concatenate([_near_edges(verts, pidx, seed),
                         rng.uniform(0, synth.BOX, (20_000, 2)).astype(np.float32)])
    brute, _ = oracle.bruteforce(xy, verts, pidx)
    assert brute.sum() > 0
    np.testing.assert_array_equal(oracle.index_join(xy, verts, pidx, 256)[0], brute)
    np.testing.assert_array_equal(oracle.hybrid_join(xy, verts, pidx, 256)[0], brute)
    np.testing.assert_array_equal(oracle.cpujoin(xy, verts, pidx, 1024)[0], brute)
