"""The allocation-free raster count (rj_raster_count_noalloc) through the C ABI.

Callers that may not allocate device memory -- hosts that budget every byte
of GPU memory, loops that must not stall on an allocation, processes already
at the memory limit -- use this entry point with their own device buffers.
Its counts must equal the regular raster join's (rj_execute) exactly, on two
calls in a row that reuse the library's fixed scratch array.  This file runs
last in the suite so that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

import rasterjoin as rj
from rasterjoin import synth

pytestmark = pytest.mark.gpu


def _entry(lib):
    fn = lib.rj_raster_count_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                   C.POINTER(C.c_double), C.c_double, C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
    return fn


def _reference_counts(xy, verts, pidx, cell):
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, xy)
    dh.setPolygons(verts, pidx)
    h = rj.GLHandler()
    try:
        h.setDataHandler(dh)
        h.setCellSize(cell)
        return h.execute(rj.RasterJoinFn).count.copy()
    finally:
        h.close()


def test_noalloc_raster_count_matches_execute(built):
    torch = pytest.importorskip("torch")
    lib = rj.load_library()
    fn = _entry(lib)
    verts, pidx = synth.voronoi_polygons(120, seed=31)
    bbox = (C.c_double * 4)(float(verts[:, 0].min()), float(verts[:, 1].min()),
                            float(verts[:, 0].max()), float(verts[:, 1].max()))
    cell = 25.0           # 1600 x 1600 canvas: within the 2048 x 2048 limit
    d_verts = torch.from_numpy(np.ascontiguousarray(verts)).cuda()
    d_pidx = torch.from_numpy(np.ascontiguousarray(pidx)).cuda()
    P, V = len(pidx) - 1, len(verts)
    stream = torch.cuda.current_stream()
    err = C.create_string_buffer(256)
    for call, seed in enumerate((41, 43)):          # two calls in a row share the scratch array
        xy = synth.points(700_001 + call * 99_999, seed=seed)["xy"]
        d_xy = torch.from_numpy(xy).cuda()
        d_count = torch.full((P,), -1, dtype=torch.int64, device="cuda")
        rc = fn(d_xy.data_ptr(), len(xy), d_verts.data_ptr(), d_pidx.data_ptr(), P, V, bbox, cell,
                d_count.data_ptr(), C.c_void_p(stream.cuda_stream), err, len(err))
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        got = d_count.cpu().numpy().astype(np.uint64)
        want = _reference_counts(xy, verts, pidx, cell)
        np.testing.assert_array_equal(got, want)
        assert got.sum() > 0
    # a canvas above the limit is refused with a message, nothing is launched
    rc = fn(d_xy.data_ptr(), len(xy), d_verts.data_ptr(), d_pidx.data_ptr(), P, V, bbox, 1.0,
            d_count.data_ptr(), C.c_void_p(stream.cuda_stream), err, len(err))
    assert rc == -1 and b"2048" in err.value
