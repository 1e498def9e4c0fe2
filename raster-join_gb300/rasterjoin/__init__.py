"""Python binding of librj.so (the C ABI in include/rj.h), via ctypes.

The class :class:`GLHandler` mirrors the reference's join dispatcher
(RasterJoin/join/GLHandler.hpp:20-78) and :class:`DataHandler` its query/data
holder (RasterJoin/db/DataHandler.hpp:14-41): same method names, same argument
meaning, results returned as the reference's flat int32 vector
``[count | sum/100 | decimal*10]`` (GLFunction.cpp:42) plus exact numpy views.

The binding never computes a join itself: when librj.so is missing or no CUDA
device is present, constructing a handler raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.dirname(_HERE)
LIB_PATH = os.path.join(_PKG, "lib", "librj.so")

# ---- enums (values identical to the reference) ------------------------------
# GLHandler::FunctionType, GLHandler.hpp:23-29
RasterJoinFn, IndexJoinFn, HybridJoinFn, RasterJoinBoundFn = 0, 1, 2, 3
# Aggregation, Common.h:34
Count, Avg, Sum = 0, 1, 2
# ConstraintType, Common.h:30
EQ, LT, LTE, GT, GTE = 0, 1, 2, 3, 4
# AttributeType, Common.h:28
Location, Uint, Int, Float = 0, 1, 2, 3

RJ_OK = 0
STATUS = {0: "RJ_OK", -1: "RJ_E_INVALID", -2: "RJ_E_OOM", -3: "RJ_E_TOO_MANY_CONSTRAINTS",
          -4: "RJ_E_TIMEOUT", -5: "RJ_E_CUDA", -6: "RJ_E_NO_DATA", -7: "RJ_E_UNSUPPORTED",
          -8: "RJ_E_BUSY", 1: "RJ_PENDING"}
RJ_PENDING = 1
SUM_SHIFT_AUTO = -2147483648
# rj_set_tuning knobs (include/rj.h)
TUNE_POINT_SHAPE, TUNE_COUNT_SHAPE, TUNE_COUNT_BLOCK_SHIFT, TUNE_HYBRID_EXACT_SCALE = 0, 1, 2, 3
TUNE_COUNT_SHAPES, TUNE_LEAN_SHAPES, TUNE_WAIT_LIMIT, TUNE_SPLAT_SHAPES, TUNE_HYBRID_SHAPES = 4, 5, 6, 7, 8
BATCH_AUTOTUNE = 0x1
BATCH_NO_FUSE = 0x2
BATCH_FUSE_ALL = 0x4
BATCH_FUSE = 0x8
MAX_CONSTRAINTS = 10

FLAG_COMPAT_INDEX_CLAMP = 0x1
FLAG_COMPAT_FLOAT_EQ = 0x2
FLAG_LINE_FILTER = 0x4
FLAG_FORCE_CANVAS = 0x8
FLAG_PHASE_TIMING = 0x10
FLAG_NO_CELL_CLASSIFY = 0x20
FLAG_NO_CACHE = 0x40
FLAG_FLAT_CANVAS = 0x80
FLAG_TIERED_CANVAS = 0x100
FLAG_COUNT_EDGE_TESTS = 0x200


class RJError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (STATUS.get(code, "?"), code, msg))
        self.code = code


# ---- C structs ---------------------------------------------------------------
class Value(C.Union):
    _fields_ = [("ival", C.c_int32), ("fval", C.c_float), ("uval", C.c_uint32)]


class QueryConstraint(C.Structure):
    """QueryConstraint, Common.h:42-47 (16 bytes)."""
    _fields_ = [("attribId", C.c_int32), ("type", C.c_int32), ("val", Value), ("dummy", C.c_int32)]


class Query(C.Structure):
    _fields_ = [("function_type", C.c_int32), ("aggregation", C.c_int32), ("aggr_attrib", C.c_int32),
                ("n_constraints", C.c_int32), ("constraints", QueryConstraint * MAX_CONSTRAINTS),
                ("accuracy_m", C.c_double), ("cell_size", C.c_double), ("ground_resolution", C.c_double),
                ("grid_res", C.c_int32), ("max_fbo_size", C.c_int32), ("time_attrib", C.c_int32),
                ("t_start", C.c_uint32), ("t_end", C.c_uint32), ("hybrid_canvas", C.c_int32),
                ("flags", C.c_uint32)]


class Result(C.Structure):
    _fields_ = [("npolys", C.c_int32), ("count", C.POINTER(C.c_uint64)), ("sum", C.POINTER(C.c_double)),
                ("compat3", C.POINTER(C.c_int32)), ("bounds", C.POINTER(C.c_int32))]


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("gpu_mem_mb", C.c_int64), ("stream", C.c_void_p)]


class Column(C.Structure):
    _fields_ = [("attrib_id", C.c_int32), ("type", C.c_int32), ("data", C.c_void_p)]


class Timings(C.Structure):
    _fields_ = [("pts_size", C.c_uint64), ("poly_size", C.c_int32), ("function", C.c_int32),
                ("no_pt_passes", C.c_int32), ("no_constraints", C.c_int32), ("execute_ms", C.c_double),
                ("pt_mem_ms", C.c_double), ("pt_render_ms", C.c_double), ("poly_mem_ms", C.c_double),
                ("poly_render_ms", C.c_double), ("setup_ms", C.c_double), ("triangulation_ms", C.c_double),
                ("poly_index_ms", C.c_double), ("backend_query_ms", C.c_double), ("accuracy", C.c_int32),
                ("kernel_launches", C.c_int32), ("edge_tests", C.c_uint64)]


class BatchStats(C.Structure):
    _fields_ = [("nqueries", C.c_int32), ("fused", C.c_int32), ("fallback", C.c_int32), ("segments", C.c_int32),
                ("items", C.c_uint64), ("rows_read", C.c_uint64), ("point_queries", C.c_uint64),
                ("total_ms", C.c_double), ("setup_ms", C.c_double), ("poly_ms", C.c_double),
                ("point_ms", C.c_double), ("reduce_ms", C.c_double), ("threads", C.c_int32),
                ("rows_per_item", C.c_int32), ("direct", C.c_int32), ("tuned", C.c_int32),
                ("kernel_launches", C.c_int32)]


class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_int32), ("canvas_mb", C.c_int64), ("max_batch", C.c_int32),
                ("max_wait_ms", C.c_double), ("batch_flags", C.c_uint32)]


class RequestInfo(C.Structure):
    _fields_ = [("submit_ms", C.c_double), ("start_ms", C.c_double), ("done_ms", C.c_double),
                ("batch_id", C.c_int32), ("batch_size", C.c_int32), ("status", C.c_int32)]


_lib = None


def load_library(path=LIB_PATH):
    """Load librj.so and declare every entry point of include/rj.h."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("librj.so not built (%s); run __graft_entry__.build()" % path)
    lib = C.CDLL(path)
    P = C.POINTER
    sig = {
        "rj_abi_version": (C.c_int, []),
        "rj_query_init": (None, [P(Query)]),
        "rj_create": (C.c_int, [P(Config), P(C.c_void_p)]),
        "rj_destroy": (None, [C.c_void_p]),
        "rj_last_error": (C.c_char_p, [C.c_void_p]),
        "rj_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
        "rj_load_points": (C.c_int, [C.c_void_p, P(Column), C.c_int32, C.c_uint64, C.c_int32]),
        "rj_attach_points_device": (C.c_int, [C.c_void_p, P(Column), C.c_int32, C.c_uint64, C.c_int32]),
        "rj_free_points": (C.c_int, [C.c_void_p]),
        "rj_attach_points_host": (C.c_int, [C.c_void_p, P(Column), C.c_int32, C.c_uint64, C.c_int32, C.c_uint64]),
        "rj_attach_points_mapped": (C.c_int, [C.c_void_p, P(Column), C.c_int32, C.c_uint64, C.c_int32]),
        "rj_set_polygons": (C.c_int, [C.c_void_p, P(C.c_float), P(C.c_int32), C.c_int32, P(C.c_double)]),
        "rj_execute": (C.c_int, [C.c_void_p, P(Query), P(Result)]),
        "rj_get_timings": (C.c_int, [C.c_void_p, P(Timings)]),
        "rj_format_time_stats": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
        "rj_polyset_create": (C.c_int, [C.c_void_p, P(C.c_float), P(C.c_int32), C.c_int32, P(C.c_double),
                                        P(C.c_void_p)]),
        "rj_polyset_destroy": (None, [C.c_void_p]),
        "rj_use_polyset": (C.c_int, [C.c_void_p, C.c_void_p]),
        "rj_build_time_index": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
        "rj_cluster_points": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
        "rj_execute_batch": (C.c_int, [C.c_void_p, C.c_int32, P(Query), P(C.c_void_p), P(Result), P(C.c_int32),
                                       C.c_uint32, P(BatchStats)]),
        "rj_server_create": (C.c_int, [C.c_void_p, P(ServerConfig), P(C.c_void_p)]),
        "rj_submit": (C.c_int, [C.c_void_p, P(Query), C.c_void_p, P(Result), P(C.c_uint64)]),
        "rj_poll": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int32, P(RequestInfo)]),
        "rj_server_destroy": (None, [C.c_void_p]),
        "rj_set_tuning": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
        "rj_selftest_bounded_wait": (C.c_int, [C.c_void_p, C.c_uint32]),
        "rj_prepare": (C.c_int, [C.c_void_p, P(Query), P(C.c_void_p)]),
        "rj_execute_prepared": (C.c_int, [C.c_void_p, P(Result)]),
        "rj_plan_destroy": (None, [C.c_void_p]),
        "rj_get_sum_partials": (C.c_int, [C.c_void_p, P(C.c_int64), P(C.c_double), P(C.c_int32)]),
        "rj_set_sum_shift": (C.c_int, [C.c_void_p, C.c_int32]),
        "rj_sum_shift_for": (C.c_int32, [C.c_double, C.c_uint64]),
        "rj_column_absmax": (C.c_int, [C.c_void_p, C.c_int32, P(C.c_double)]),
        "rj_get_tuning": (C.c_int, [C.c_void_p, C.c_int32, P(C.c_int32)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def default_query():
    q = Query()
    load_library().rj_query_init(C.byref(q))
    return q


def constraint(attrib_id, ctype, value, attr_type):
    """QueryConstraint with the value stored by the column's type (Value union)."""
    c = QueryConstraint()
    c.attribId = attrib_id
    c.type = ctype
    if attr_type == Float:
        c.val.fval = float(value)
    elif attr_type == Int:
        c.val.ival = int(value)
    else:
        c.val.uval = int(value) & 0xFFFFFFFF
    c.dummy = 0
    return c


class JoinResult:
    """Per-polygon results of one execute call."""

    def __init__(self, count, sum_, compat3, bounds):
        self.count = count
        self.sum = sum_
        self.compat3 = compat3
        self.bounds = bounds

    @property
    def avg(self):
        with np.errstate(invalid="ignore", divide="ignore"):
            return np.where(self.count > 0, self.sum / np.maximum(self.count, 1), 0.0)


class _ResultBuffers:
    """Host result arrays of one query and the rj_result pointing at them."""

    def __init__(self, P, bounds=False):
        self.count = np.zeros(P, np.uint64)
        self.sum = np.zeros(P, np.float64)
        self.compat3 = np.zeros(3 * P, np.int32)
        self.bounds = np.zeros(4 * P, np.int32) if bounds else None
        self.r = Result(P, self.count.ctypes.data_as(C.POINTER(C.c_uint64)),
                        self.sum.ctypes.data_as(C.POINTER(C.c_double)),
                        self.compat3.ctypes.data_as(C.POINTER(C.c_int32)),
                        self.bounds.ctypes.data_as(C.POINTER(C.c_int32)) if bounds else None)

    def result(self):
        return JoinResult(self.count, self.sum, self.compat3, self.bounds)


class PolySet:
    """A polygon collection resident on the device (rj_polyset)."""

    def __init__(self, handler, xy, pindex, bbox=None):
        self.handler = handler
        self.xy = np.ascontiguousarray(xy, dtype=np.float32).reshape(-1, 2)
        self.pindex = np.ascontiguousarray(pindex, dtype=np.int32)
        self.P = len(self.pindex) - 1
        h = C.c_void_p()
        bb = None if bbox is None else (C.c_double * 4)(*bbox)
        handler._check(handler.lib.rj_polyset_create(handler.ctx, self.xy.ctypes.data_as(C.POINTER(C.c_float)),
                                                     self.pindex.ctypes.data_as(C.POINTER(C.c_int32)), self.P,
                                                     bb, C.byref(h)))
        self.ptr = h

    def close(self):
        if getattr(self, "ptr", None) and getattr(self.handler, "ctx", None):
            self.handler.lib.rj_polyset_destroy(self.ptr)
        self.ptr = None


class Plan:
    """A prepared query (rj_prepare): replays its captured CUDA graph."""

    def __init__(self, handler, fn, query, P):
        self.h = handler
        self.fn = fn
        self.P = P
        self.ptr = C.c_void_p()
        handler._check(handler.lib.rj_prepare(handler.ctx, C.byref(query), C.byref(self.ptr)))

    def execute(self):
        P = self.P
        count = np.zeros(P, np.uint64)
        sum_ = np.zeros(P, np.float64)
        compat3 = np.zeros(3 * P, np.int32)
        bounds = np.zeros(4 * P, np.int32)
        r = Result(P, count.ctypes.data_as(C.POINTER(C.c_uint64)), sum_.ctypes.data_as(C.POINTER(C.c_double)),
                   compat3.ctypes.data_as(C.POINTER(C.c_int32)), bounds.ctypes.data_as(C.POINTER(C.c_int32)))
        self.h._check(self.h.lib.rj_execute_prepared(self.ptr, C.byref(r)))
        return JoinResult(count, sum_, compat3, bounds if self.fn == RasterJoinBoundFn else None)

    def close(self):
        if self.ptr:
            self.h.lib.rj_plan_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request loop over the handler's resident table (rj_server_*).

    submit(query, polyset) -> ticket; poll(ticket, timeout_ms) -> (JoinResult,
    info dict) or None while pending."""

    def __init__(self, handler, slots=0, canvas_mb=0, max_batch=0, max_wait_ms=0.0, batch_flags=0):
        self.handler = handler
        self.lib = handler.lib
        cfg = ServerConfig(slots, canvas_mb, max_batch, max_wait_ms, batch_flags)
        h = C.c_void_p()
        handler._check(self.lib.rj_server_create(handler.ctx, C.byref(cfg), C.byref(h)))
        self.ptr = h
        self._pending = {}

    def submit(self, query, polyset=None):
        P = polyset.P if polyset is not None else len(self.handler.dataHandler.polys[1]) - 1
        buf = _ResultBuffers(P)
        t = C.c_uint64()
        q = Query()
        C.pointer(q)[0] = query
        rc = self.lib.rj_submit(self.ptr, C.byref(q), polyset.ptr if polyset is not None else None,
                                C.byref(buf.r), C.byref(t))
        if rc != RJ_OK:
            raise RJError(rc, "rj_submit failed")
        self._pending[t.value] = (buf, q)
        return t.value

    def poll(self, ticket, timeout_ms=-1):
        info = RequestInfo()
        rc = self.lib.rj_poll(self.ptr, ticket, timeout_ms, C.byref(info))
        if rc == RJ_PENDING:
            return None
        buf, _ = self._pending.pop(ticket)
        if rc != RJ_OK:
            raise RJError(rc, "request %d failed" % ticket)
        return buf.result(), {f: getattr(info, f) for f, _ in RequestInfo._fields_}

    def close(self):
        if getattr(self, "ptr", None):
            self.lib.rj_server_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DataHandler:
    """Point columns, polygons, constraints and aggregation of a query
    (DataHandler.hpp:14-41)."""

    def __init__(self):
        self.columns = {}          # attrib id -> (type, ndarray)
        self.location_attribute = None
        self.polys = None          # (xy float32 [V,2], pindex int32 [P+1])
        self.bbox = None
        self.constraints = []
        self.aggr = Count
        self.aggr_attrib = -1
        self.time_range = None     # (attrib, start, end)
        self.types = {}            # attribute types of a table loaded elsewhere (device / host attach)

    def add_column(self, attrib_id, attr_type, data):
        if attr_type == Location:
            data = np.ascontiguousarray(data, dtype=np.float32).reshape(-1, 2)
            self.location_attribute = attrib_id
        elif attr_type == Float:
            data = np.ascontiguousarray(data, dtype=np.float32)
        elif attr_type == Int:
            data = np.ascontiguousarray(data, dtype=np.int32)
        else:
            data = np.ascontiguousarray(data, dtype=np.uint32)
        self.columns[attrib_id] = (attr_type, data)

    def setPolygons(self, xy, pindex, bbox=None):
        self.polys = (np.ascontiguousarray(xy, dtype=np.float32).reshape(-1, 2),
                      np.ascontiguousarray(pindex, dtype=np.int32))
        self.bbox = None if bbox is None else np.asarray(bbox, dtype=np.float64)

    def setQueryConstraints(self, constraints):
        """constraints: list of (attrib_id, ConstraintType, value)."""
        self.constraints = list(constraints)

    def setAggregation(self, aggr=Count, attrib_id=-1):
        self.aggr = aggr
        self.aggr_attrib = attrib_id

    def setTimeRange(self, attrib_id, start, end):
        self.time_range = None if attrib_id is None else (attrib_id, start, end)

    def declare(self, attrib_id, attr_type):
        """Type of a column held outside this DataHandler (attachDevice / attachHost)."""
        self.types[attrib_id] = attr_type

    def attr_type(self, attrib_id):
        if attrib_id in self.columns:
            return self.columns[attrib_id][0]
        return self.types.get(attrib_id, Uint)


class GLHandler:
    """Join dispatcher over one CUDA device (GLHandler.hpp:20-78).

    getInstance(gpuMemMB) -> handler; setDataHandler; setAccuracyDistance;
    setPolyIndexResolution; executeFunction(FunctionType) -> int32[3P];
    getErrorBounds(FunctionType) -> int32[4P]; printTimeStats.
    """

    def __init__(self, gpu_mem_mb=0, device=0, stream=None):
        self.lib = load_library()
        cfg = Config(device, gpu_mem_mb, stream)
        h = C.c_void_p()
        rc = self.lib.rj_create(C.byref(cfg), C.byref(h))
        if rc != RJ_OK:
            raise RJError(rc, "rj_create failed (no CUDA device?)")
        self.ctx = h
        self.dataHandler = None
        self.accuracy = 100.0
        self.cell_size = 0.0
        self.ground_resolution = 1.0
        self.presx = 256
        self.max_fbo_size = 8192
        self.hybrid_canvas = 0          # 0: library default
        self.flags = 0
        self._loaded_points = None
        self._loaded_polys = None
        self.bounds = None
        self.last = None
        self._bound = None               # PolySet bound by usePolySet

    @classmethod
    def getInstance(cls, gpuMemMB=2048, inMemory=True):
        return cls(gpu_mem_mb=gpuMemMB)

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.rj_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != RJ_OK:
            raise RJError(rc, self.lib.rj_last_error(self.ctx).decode())

    # ---- configuration (GLHandler.cpp:250-262) ----
    def setDataHandler(self, dh):
        self.dataHandler = dh

    def setAccuracyDistance(self, metres):
        self.accuracy = float(metres)
        self.cell_size = 0.0

    def setCellSize(self, cell):
        self.cell_size = float(cell)

    def setPolyIndexResolution(self, resx, resy=None):
        self.presx = int(resx)   # only x is used (GLFunction.cpp:76)

    def setStream(self, stream_ptr):
        self._check(self.lib.rj_set_stream(self.ctx, C.c_void_p(stream_ptr)))

    # ---- exact partial sums (rj_get_sum_partials / rj_set_sum_shift) ----
    def sumPartials(self):
        """(fixed int64[P], nonfinite float64[P], shift) of the last execute."""
        P = len(self.last.count) if self.last is not None else 0
        fixed = np.zeros(P, np.int64)
        nf = np.zeros(P, np.float64)
        sh = C.c_int32(0)
        self._check(self.lib.rj_get_sum_partials(self.ctx, fixed.ctypes.data_as(C.POINTER(C.c_int64)),
                                                 nf.ctypes.data_as(C.POINTER(C.c_double)), C.byref(sh)))
        return fixed, nf, sh.value

    def setSumShift(self, shift=None):
        self._check(self.lib.rj_set_sum_shift(self.ctx, SUM_SHIFT_AUTO if shift is None else int(shift)))

    def columnAbsMax(self, attrib_id):
        self.upload()
        v = C.c_double(0.0)
        self._check(self.lib.rj_column_absmax(self.ctx, int(attrib_id), C.byref(v)))
        return v.value

    # ---- kernel tuning (rj_set_tuning / rj_get_tuning; results never change) ----
    def setTuning(self, knob, value):
        self._check(self.lib.rj_set_tuning(self.ctx, int(knob), int(value)))

    def getTuning(self, knob):
        v = C.c_int32(0)
        self._check(self.lib.rj_get_tuning(self.ctx, int(knob), C.byref(v)))
        return v.value

    # ---- data upload ----
    def upload(self, force=False):
        dh = self.dataHandler
        if dh is None:
            raise RJError(-6, "DataHandler not set")
        key = tuple((k, id(v[1])) for k, v in sorted(dh.columns.items()))
        if dh.columns and (force or key != self._loaded_points):
            cols = (Column * len(dh.columns))()
            n = None
            for i, (aid, (typ, arr)) in enumerate(sorted(dh.columns.items())):
                cols[i].attrib_id = aid
                cols[i].type = typ
                cols[i].data = arr.ctypes.data
                m = arr.shape[0]
                n = m if n is None else n
                if m != n:
                    raise RJError(-1, "columns have different lengths")
            self._check(self.lib.rj_load_points(self.ctx, cols, len(dh.columns), n or 0,
                                                dh.location_attribute))
            self._loaded_points = key
        pkey = (id(dh.polys[0]), id(dh.polys[1]), None if dh.bbox is None else tuple(dh.bbox))
        if force or pkey != self._loaded_polys:
            xy, pidx = dh.polys
            bb = None
            if dh.bbox is not None:
                bb = (C.c_double * 4)(*dh.bbox)
            self._check(self.lib.rj_set_polygons(self.ctx, xy.ctypes.data_as(C.POINTER(C.c_float)),
                                                 pidx.ctypes.data_as(C.POINTER(C.c_int32)), len(pidx) - 1,
                                                 bb))
            self._loaded_polys = pkey
            self._bound = None

    def make_query(self, fn):
        dh = self.dataHandler
        q = default_query()
        q.function_type = fn
        q.aggregation = dh.aggr
        q.aggr_attrib = dh.aggr_attrib
        if len(dh.constraints) > MAX_CONSTRAINTS:
            q.n_constraints = len(dh.constraints)
        else:
            q.n_constraints = len(dh.constraints)
            for i, (aid, ct, val) in enumerate(dh.constraints):
                q.constraints[i] = constraint(aid, ct, val, dh.attr_type(aid))
        q.accuracy_m = self.accuracy
        q.cell_size = self.cell_size
        q.ground_resolution = self.ground_resolution
        q.grid_res = self.presx
        q.max_fbo_size = self.max_fbo_size
        q.hybrid_canvas = self.hybrid_canvas
        if dh.time_range is not None:
            q.time_attrib, q.t_start, q.t_end = dh.time_range
        q.flags = self.flags
        return q

    def execute(self, fn, query=None):
        """Run one join; returns JoinResult with exact arrays."""
        if self.dataHandler is not None:
            self.upload()
        q = query if query is not None else self.make_query(fn)
        P = self._bound.P if self._bound is not None else len(self.dataHandler.polys[1]) - 1
        count = np.zeros(P, np.uint64)
        sum_ = np.zeros(P, np.float64)
        compat3 = np.zeros(3 * P, np.int32)
        bounds = np.zeros(4 * P, np.int32)
        r = Result(P, count.ctypes.data_as(C.POINTER(C.c_uint64)), sum_.ctypes.data_as(C.POINTER(C.c_double)),
                   compat3.ctypes.data_as(C.POINTER(C.c_int32)), bounds.ctypes.data_as(C.POINTER(C.c_int32)))
        self._check(self.lib.rj_execute(self.ctx, C.byref(q), C.byref(r)))
        self.last = JoinResult(count, sum_, compat3, bounds if fn == RasterJoinBoundFn else None)
        self.bounds = bounds if fn == RasterJoinBoundFn else None
        return self.last

    def prepare(self, fn, query=None):
        """rj_prepare: a Plan whose execute() replays the query's captured graph."""
        if self.dataHandler is not None:
            self.upload()
        q = query if query is not None else self.make_query(fn)
        P = self._bound.P if self._bound is not None else len(self.dataHandler.polys[1]) - 1
        return Plan(self, fn, q, P)

    def executeFunction(self, fn):
        """GLHandler::executeFunction (GLHandler.cpp:188-204): int32[3P]."""
        return self.execute(fn).compat3

    def getErrorBounds(self, fn):
        """GLHandler::getErrorBounds (GLHandler.cpp:206-212): int32[4P] or empty."""
        if fn == RasterJoinBoundFn and self.bounds is not None:
            return self.bounds
        return np.zeros(0, np.int32)

    def attachDevice(self, columns, npoints, loc_attrib):
        """Use device-resident columns as the point table without a copy.
        columns: [(attrib_id, type, device_pointer)], 16-byte aligned, kept
        alive by the caller."""
        cols = (Column * len(columns))()
        for i, (aid, typ, ptr) in enumerate(columns):
            cols[i].attrib_id = aid
            cols[i].type = typ
            cols[i].data = ptr
        self._check(self.lib.rj_attach_points_device(self.ctx, cols, len(columns), npoints, loc_attrib))
        self._loaded_points = ("device", tuple(columns), npoints)

    def attachHost(self, columns, npoints, loc_attrib, chunk_points=0):
        """Out-of-core table: host arrays (kept alive by the caller) streamed
        through the device in chunks of chunk_points rows by every query."""
        cols = (Column * len(columns))()
        keep = []
        for i, (aid, typ, arr) in enumerate(columns):
            arr = np.ascontiguousarray(arr)
            keep.append(arr)
            cols[i].attrib_id = aid
            cols[i].type = typ
            cols[i].data = arr.ctypes.data
        self._check(self.lib.rj_attach_points_host(self.ctx, cols, len(columns), npoints, loc_attrib, chunk_points))
        self._host_table = keep
        self._loaded_points = ("host", tuple(id(a) for a in keep), npoints)

    def attachMapped(self, columns, npoints, loc_attrib):
        """Host table read in place over the host link: columns are
        (attrib_id, type, array or address) in page-locked host memory (e.g. a
        pinned torch tensor's numpy view), kept alive by the caller."""
        cols = (Column * len(columns))()
        keep = []
        for i, (aid, typ, arr) in enumerate(columns):
            cols[i].attrib_id = aid
            cols[i].type = typ
            if isinstance(arr, int):
                cols[i].data = arr
            else:
                keep.append(arr)
                cols[i].data = arr.ctypes.data
        self._check(self.lib.rj_attach_points_mapped(self.ctx, cols, len(columns), npoints, loc_attrib))
        self._host_table = keep
        self._loaded_points = ("device",)

    # ---- polygon sets, time index, batches ----
    def polyset(self, xy, pindex, bbox=None):
        return PolySet(self, xy, pindex, bbox)

    def usePolySet(self, ps):
        if self.dataHandler is not None:
            self.upload()
        self._check(self.lib.rj_use_polyset(self.ctx, ps.ptr if ps is not None else None))
        self._bound = ps

    def buildTimeIndex(self, attrib_id, nbuckets=0):
        if self.dataHandler is not None and not (isinstance(self._loaded_points, tuple)
                                                 and self._loaded_points[:1] == ("device",)):
            self.upload()
        self._check(self.lib.rj_build_time_index(self.ctx, attrib_id, nbuckets))

    def clusterPoints(self, time_attrib=-1, nbuckets=0, cell_bits=8):
        """Reorder the resident table by (time bucket, Z-order cell); with a
        time attribute this also builds the time index."""
        if self.dataHandler is not None and not (isinstance(self._loaded_points, tuple)
                                                 and self._loaded_points[:1] == ("device",)):
            self.upload()
        self._check(self.lib.rj_cluster_points(self.ctx, time_attrib, nbuckets, cell_bits))

    def execute_batch(self, queries, polysets, flags=0, raise_on_error=True):
        """Run queries[i] on polysets[i] (None: the handler's polygons) in one
        batch; returns (list of JoinResult, status array, stats dict)."""
        n = len(queries)
        qa = (Query * max(n, 1))()
        for i, q in enumerate(queries):
            qa[i] = q
        sa = (C.c_void_p * max(n, 1))()
        bufs = []
        for i, ps in enumerate(polysets):
            sa[i] = ps.ptr if ps is not None else None
            P = ps.P if ps is not None else len(self.dataHandler.polys[1]) - 1
            bufs.append(_ResultBuffers(P, bounds=queries[i].function_type == RasterJoinBoundFn))
        ra = (Result * max(n, 1))()
        for i, b in enumerate(bufs):
            ra[i] = b.r
        st = (C.c_int32 * max(n, 1))()
        stats = BatchStats()
        rc = self.lib.rj_execute_batch(self.ctx, n, qa, sa, ra, st, flags, C.byref(stats))
        if rc != RJ_OK and raise_on_error:
            self._check(rc)
        return ([b.result() for b in bufs], np.array(st[:n], np.int32),
                {f: getattr(stats, f) for f, _ in BatchStats._fields_})

    def server(self, **kw):
        return Server(self, **kw)

    def timings(self):
        t = Timings()
        self._check(self.lib.rj_get_timings(self.ctx, C.byref(t)))
        return {f: getattr(t, f) for f, _ in Timings._fields_}

    def printTimeStats(self, fn=None):
        buf = C.create_string_buffer(512)
        self._check(self.lib.rj_format_time_stats(self.ctx, buf, 512))
        return buf.value.decode()


def sum_shift_for(max_abs, rows):
    """Fixed-point shift the library picks for |values| <= max_abs over `rows` rows."""
    return int(load_library().rj_sum_shift_for(float(max_abs), int(rows)))


def decode_sums(fixed, nonfinite, shift):
    """Per-polygon sums from exact partials, as rj_execute decodes them."""
    return np.ldexp(np.asarray(fixed, np.int64).astype(np.float64), -int(shift)) + np.asarray(nonfinite, np.float64)


def decode_avg(agg):
    """printResults avg decode (RasterJoin/main.cpp:206-208) of an int32[3P] vector."""
    agg = np.asarray(agg, dtype=np.int64)
    P = len(agg) // 3
    num = agg[P:2 * P].astype(np.float32) * np.float32(100) + agg[2 * P:].astype(np.float32) / np.float32(10)
    den = agg[:P].astype(np.float32)
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(agg[:P] == 0, 0.0, num / np.where(den == 0, 1, den))
