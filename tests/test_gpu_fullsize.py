"""Full-size parity: benchmark configuration 2's table (100M points with the
time range, three predicates and avg) through the hybrid and index joins,
against the CPUJoin restatement (CPUJoin.cpp:62-122, GridIndexF.cpp:60-549;
filters and sums are the oracle's labelled extension of it).  Counts
bit-exact, sums within 1e-6 relative."""
import numpy as np
import pytest

import oracle
import rasterjoin as rj
from rasterjoin import synth

pytestmark = pytest.mark.gpu

N = 100_000_000


@pytest.fixture(scope="module")
def c2():
    pts = synth.points(N, seed=20261203, columns=True)
    verts, pidx = synth.voronoi_polygons(260, seed=20261203)
    return pts, verts, pidx


def test_config2_hybrid_and_index_match_cpujoin(handler, c2):
    pts, verts, pidx = c2
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, pts["xy"])
    dh.add_column(2, rj.Uint, pts["t"])
    dh.add_column(3, rj.Float, pts["a"])
    dh.add_column(4, rj.Int, pts["f1"])
    dh.add_column(5, rj.Int, pts["f2"])
    dh.setPolygons(verts, pidx)
    cons = [(4, rj.GT, 2), (5, rj.LT, 8), (3, rj.LT, 50.0)]
    trange = (2, synth.T0, synth.T0 + synth.YEAR // 2)
    dh.setQueryConstraints(cons)
    dh.setTimeRange(*trange)
    dh.setAggregation(rj.Avg, 3)
    handler.setDataHandler(dh)
    handler.setPolyIndexResolution(256)
    cols = oracle.Columns({2: (oracle.Uint, pts["t"]), 3: (oracle.Float, pts["a"]),
                           4: (oracle.Int, pts["f1"]), 5: (oracle.Int, pts["f2"])})
    f = cols.filt(cons, aggr_attrib=3, time_range=trange)
    want_c, want_s, _, _ = oracle.cpujoin(pts["xy"], verts, pidx, 256, f=f)
    assert want_c.sum() > N // 10          # the filters keep a sizeable share of the table
    for fn in (rj.HybridJoinFn, rj.IndexJoinFn):
        got = handler.execute(fn)
        np.testing.assert_array_equal(got.count, want_c, err_msg="function type %d" % fn)
        np.testing.assert_allclose(got.sum, want_s, rtol=1e-6, atol=1e-9 * float(np.abs(want_s).max()))
