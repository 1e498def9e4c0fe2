"""ctypes wrapper of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline arm of bench.py, never by the library.  Each function mirrors one
reference algorithm (see oracle.c's header for the file:line citations).

Parity anchors: the oracle is checked against the reference's own known-answer
fixture (RasterJoin/test/baseline.hpp:139-217: two squares, five points,
counts 2 and 3) and against the reference's clip2tri triangulation compiled
from its sources (oracle/ref_tri) for the pixel-centre fill rule.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MAXF = 12

Location, Uint, Int, Float = 0, 1, 2, 3
EQ, LT, LTE, GT, GTE = 0, 1, 2, 3, 4


class OrcFilter(C.Structure):
    _fields_ = [("n", C.c_int), ("col", C.c_void_p * MAXF), ("op", C.c_int * MAXF), ("typ", C.c_int * MAXF),
                ("val", C.c_uint32 * MAXF), ("compat_mask", C.c_uint32), ("aggr", C.c_int),
                ("aggr_typ", C.c_int), ("aggr_col", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build()
        L = C.CDLL(path)
        P = C.POINTER
        fp, ip, dp, u64p, i64p = P(C.c_float), P(C.c_int), P(C.c_double), P(C.c_uint64), P(C.c_int64)
        L.orc_bruteforce.argtypes = [fp, C.c_uint64, P(OrcFilter), fp, ip, C.c_int, dp, C.c_int, u64p, dp]
        L.orc_bruteforce.restype = None
        L.orc_bruteforce_f64.argtypes = [fp, C.c_uint64, P(OrcFilter), fp, ip, C.c_int, C.c_int, u64p, dp]
        L.orc_bruteforce_f64.restype = None
        L.orc_index_join.argtypes = [fp, C.c_uint64, P(OrcFilter), fp, ip, C.c_int, dp, C.c_int, C.c_int, C.c_int,
                                     u64p, dp]
        L.orc_index_join.restype = None
        L.orc_hybrid_join.argtypes = [fp, C.c_uint64, P(OrcFilter), fp, ip, C.c_int, dp, C.c_int, C.c_int, u64p, dp]
        L.orc_hybrid_join.restype = None
        L.orc_cpujoin.argtypes = [fp, C.c_uint64, P(OrcFilter), fp, ip, C.c_int, dp, C.c_int, C.c_int, u64p, dp, dp]
        L.orc_cpujoin.restype = C.c_double
        L.orc_raster_join.argtypes = [fp, C.c_uint64, P(OrcFilter), fp, ip, C.c_int, dp, C.c_double, C.c_int,
                                      C.c_int, C.c_int, u64p, dp, i64p]
        L.orc_raster_join.restype = C.c_int
        L.orc_raster_geometry.argtypes = [dp, C.c_double, C.c_int, ip]
        L.orc_raster_geometry.restype = None
        L.orc_cover_maps.argtypes = [fp, ip, C.c_int, dp, ip, C.c_int, dp, C.c_double, P(C.c_int32), P(C.c_int32), ip]
        L.orc_cover_maps.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Columns:
    """Keeps column arrays alive and builds OrcFilter structs."""

    def __init__(self, columns):
        # columns: attrib id -> (type, ndarray)
        self.columns = {k: (t, np.ascontiguousarray(a)) for k, (t, a) in columns.items()}

    def filt(self, constraints=(), aggr_attrib=None, time_range=None, compat_float_eq=False):
        f = OrcFilter()
        k = 0
        for aid, op, val in constraints:
            typ, arr = self.columns[aid]
            f.col[k] = arr.ctypes.data
            f.op[k] = op
            f.typ[k] = typ
            f.val[k] = _bits(val, typ)
            if compat_float_eq:
                f.compat_mask |= 1 << k
            k += 1
        if time_range is not None:
            aid, lo, hi = time_range
            typ, arr = self.columns[aid]
            for op, v in ((GTE, lo), (LTE, hi)):
                f.col[k] = arr.ctypes.data
                f.op[k] = op
                f.typ[k] = typ
                f.val[k] = _bits(v, typ)
                k += 1
        f.n = k
        if aggr_attrib is not None and aggr_attrib >= 0:
            typ, arr = self.columns[aggr_attrib]
            f.aggr = 1
            f.aggr_typ = typ
            f.aggr_col = arr.ctypes.data
        return f


def _bits(val, typ):
    if typ == Float:
        return int(np.array([val], np.float32).view(np.uint32)[0])
    if typ == Int:
        return int(np.array([val], np.int32).view(np.uint32)[0])
    return int(val) & 0xFFFFFFFF


def _prep(xy, verts, pindex, bbox):
    xy = np.ascontiguousarray(xy, np.float32).reshape(-1, 2)
    verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 2)
    pindex = np.ascontiguousarray(pindex, np.int32)
    if bbox is None:
        bbox = np.array([verts[:, 0].min(), verts[:, 1].min(), verts[:, 0].max(), verts[:, 1].max()], np.float64)
    bbox = np.ascontiguousarray(bbox, np.float64)
    return xy, verts, pindex, bbox


def _empty_filter():
    return OrcFilter()


def bruteforce(xy, verts, pindex, f=None, bbox=None, nthreads=0):
    xy, verts, pindex, bbox = _prep(xy, verts, pindex, bbox)
    P = len(pindex) - 1
    cnt, s = np.zeros(P, np.uint64), np.zeros(P, np.float64)
    f = f or _empty_filter()
    lib().orc_bruteforce(_ptr(xy, C.c_float), len(xy), C.byref(f), _ptr(verts, C.c_float), _ptr(pindex, C.c_int), P,
                         _ptr(bbox, C.c_double), nthreads, _ptr(cnt, C.c_uint64), _ptr(s, C.c_double))
    return cnt, s


def bruteforce_f64(xy, verts, pindex, f=None, nthreads=0):
    xy, verts, pindex, _ = _prep(xy, verts, pindex, None)
    P = len(pindex) - 1
    cnt, s = np.zeros(P, np.uint64), np.zeros(P, np.float64)
    f = f or _empty_filter()
    lib().orc_bruteforce_f64(_ptr(xy, C.c_float), len(xy), C.byref(f), _ptr(verts, C.c_float),
                             _ptr(pindex, C.c_int), P, nthreads, _ptr(cnt, C.c_uint64), _ptr(s, C.c_double))
    return cnt, s


def index_join(xy, verts, pindex, res, f=None, bbox=None, compat_clamp=False, nthreads=0):
    xy, verts, pindex, bbox = _prep(xy, verts, pindex, bbox)
    P = len(pindex) - 1
    cnt, s = np.zeros(P, np.uint64), np.zeros(P, np.float64)
    f = f or _empty_filter()
    lib().orc_index_join(_ptr(xy, C.c_float), len(xy), C.byref(f), _ptr(verts, C.c_float), _ptr(pindex, C.c_int),
                         P, _ptr(bbox, C.c_double), res, 1 if compat_clamp else 0, nthreads, _ptr(cnt, C.c_uint64),
                         _ptr(s, C.c_double))
    return cnt, s


def hybrid_join(xy, verts, pindex, res, f=None, bbox=None, nthreads=0):
    xy, verts, pindex, bbox = _prep(xy, verts, pindex, bbox)
    P = len(pindex) - 1
    cnt, s = np.zeros(P, np.uint64), np.zeros(P, np.float64)
    f = f or _empty_filter()
    lib().orc_hybrid_join(_ptr(xy, C.c_float), len(xy), C.byref(f), _ptr(verts, C.c_float), _ptr(pindex, C.c_int),
                          P, _ptr(bbox, C.c_double), res, nthreads, _ptr(cnt, C.c_uint64), _ptr(s, C.c_double))
    return cnt, s


def cpujoin(xy, verts, pindex, res=1024, f=None, bbox=None, nthreads=0):
    """CPUJoin restatement; returns (count, sum, join_seconds, build_seconds)."""
    xy, verts, pindex, bbox = _prep(xy, verts, pindex, bbox)
    P = len(pindex) - 1
    cnt, s = np.zeros(P, np.uint64), np.zeros(P, np.float64)
    bt = C.c_double(0.0)
    fp = C.byref(f) if f is not None else None
    t = lib().orc_cpujoin(_ptr(xy, C.c_float), len(xy), fp, _ptr(verts, C.c_float), _ptr(pindex, C.c_int), P,
                          _ptr(bbox, C.c_double), res, nthreads, _ptr(cnt, C.c_uint64), _ptr(s, C.c_double),
                          C.byref(bt))
    return cnt, s, t, bt.value


def raster_cell(accuracy_m=None, cell_size=None, ground_resolution=1.0):
    """GLFunction::setMaxCellSize (GLFunction.cpp:26-30): the pixel diagonal is epsilon."""
    if cell_size:
        return float(cell_size)
    return (accuracy_m / np.sqrt(2.0)) / ground_resolution


def raster_join(xy, verts, pindex, cell, f=None, bbox=None, max_res=8192, bounds=False, line_filter=False,
                nthreads=0):
    xy, verts, pindex, bbox = _prep(xy, verts, pindex, bbox)
    P = len(pindex) - 1
    cnt, s = np.zeros(P, np.uint64), np.zeros(P, np.float64)
    b = np.zeros(4 * P, np.int64) if bounds else None
    f = f or _empty_filter()
    rc = lib().orc_raster_join(_ptr(xy, C.c_float), len(xy), C.byref(f), _ptr(verts, C.c_float),
                               _ptr(pindex, C.c_int), P, _ptr(bbox, C.c_double), float(cell), max_res,
                               1 if line_filter else 0, nthreads, _ptr(cnt, C.c_uint64), _ptr(s, C.c_double),
                               _ptr(b, C.c_int64) if bounds else None)
    if rc != 0:
        raise MemoryError("oracle raster canvas allocation failed")
    return cnt, s, b


def cover_maps(verts, pindex, tris, tri_poly, bbox, cell):
    """Per-pixel coverage of a single-tile canvas by the polygon crossing rule
    and by GL's triangle rule (fill-rule cross-check); returns two int32 maps
    (polygon id, -1 none, -2 several)."""
    verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 2)
    pindex = np.ascontiguousarray(pindex, np.int32)
    tris = np.ascontiguousarray(tris, np.float64).reshape(-1, 6)
    tri_poly = np.ascontiguousarray(tri_poly, np.int32)
    bbox = np.ascontiguousarray(bbox, np.float64)
    geo = raster_geometry(bbox, cell, 1 << 30)
    rx, ry = geo[2], geo[3]
    a = np.empty(rx * ry, np.int32)
    b = np.empty(rx * ry, np.int32)
    dims = np.zeros(2, np.int32)
    lib().orc_cover_maps(_ptr(verts, C.c_float), _ptr(pindex, C.c_int), len(pindex) - 1, _ptr(tris, C.c_double),
                         _ptr(tri_poly, C.c_int), len(tri_poly), _ptr(bbox, C.c_double), float(cell),
                         _ptr(a, C.c_int32), _ptr(b, C.c_int32), _ptr(dims, C.c_int))
    return a.reshape(ry, rx), b.reshape(ry, rx)


def raster_geometry(bbox, cell, max_res=8192):
    out = np.zeros(4, np.int32)
    lib().orc_raster_geometry(_ptr(np.ascontiguousarray(bbox, np.float64), C.c_double), float(cell), max_res,
                              _ptr(out, C.c_int))
    return tuple(int(v) for v in out)
