"""Host-resident tables read in place (rj_attach_points_mapped): page-locked
host columns that the point passes read over the host link every query give
the resident table's results, for every join type, with filters and avg;
memory the device cannot address is refused."""
import numpy as np
import pytest

import oracle
import rasterjoin as rj
from rasterjoin import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


class _Pinned:
    """A page-locked host copy of an array (the tensor keeps the memory)."""

    def __init__(self, a):
        self.t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        self.a = self.t.numpy().view(a.dtype).reshape(a.shape)
        self.a[...] = a

    def numpy(self):
        return self.a


def _pinned(a):
    return _Pinned(np.ascontiguousarray(a))


@pytest.fixture(scope="module")
def data():
    pts = synth.points(500_001, seed=61, columns=True)
    verts, pidx = synth.voronoi_polygons(260, seed=20261203)
    return pts, verts, pidx


@pytest.mark.parametrize("fn", [rj.RasterJoinFn, rj.RasterJoinBoundFn, rj.HybridJoinFn, rj.IndexJoinFn])
def test_mapped_equals_resident(data, fn, built):
    pts, verts, pidx = data
    cons, trange = [(4, rj.GT, 2)], (2, synth.T0, synth.T0 + synth.YEAR // 2)
    res = {}
    keep = []
    for mode in ("resident", "mapped"):
        h = rj.GLHandler()
        try:
            dh = rj.DataHandler()
            if mode == "resident":
                dh.add_column(1, rj.Location, pts["xy"])
                dh.add_column(2, rj.Uint, pts["t"])
                dh.add_column(3, rj.Float, pts["a"])
                dh.add_column(4, rj.Int, pts["f1"])
            else:
                cols = [_pinned(pts["xy"]), _pinned(pts["t"]), _pinned(pts["a"]), _pinned(pts["f1"])]
                keep.append(cols)
                h.attachMapped([(1, rj.Location, cols[0].numpy()), (2, rj.Uint, cols[1].numpy()),
                                (3, rj.Float, cols[2].numpy()), (4, rj.Int, cols[3].numpy())], len(pts["t"]), 1)
                for aid, typ in ((2, rj.Uint), (3, rj.Float), (4, rj.Int)):
                    dh.declare(aid, typ)
            dh.setPolygons(verts, pidx)
            if fn != rj.RasterJoinBoundFn:
                dh.setQueryConstraints(cons)
                dh.setTimeRange(*trange)
                dh.setAggregation(rj.Avg, 3)
            h.setDataHandler(dh)
            h.setCellSize(10.0)
            h.setPolyIndexResolution(256)
            r = h.execute(fn)
            res[mode] = (r.count.copy(), r.sum.copy(), None if r.bounds is None else r.bounds.copy())
        finally:
            h.close()
    np.testing.assert_array_equal(res["mapped"][0], res["resident"][0])
    assert res["mapped"][1].tobytes() == res["resident"][1].tobytes()
    if fn == rj.RasterJoinBoundFn:
        np.testing.assert_array_equal(res["mapped"][2], res["resident"][2])
        np.testing.assert_array_equal(res["mapped"][0], oracle.raster_join(pts["xy"], verts, pidx, 10.0)[0])


def test_pageable_memory_is_refused(data, built):
    pts, verts, pidx = data
    h = rj.GLHandler()
    try:
        with pytest.raises(rj.RJError) as ei:
            h.attachMapped([(1, rj.Location, np.ascontiguousarray(pts["xy"]))], len(pts["xy"]), 1)
        assert ei.value.code == -1
    finally:
        h.close()
