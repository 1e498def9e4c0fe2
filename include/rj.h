/*
 * rj.h -- C ABI of the GB300-native Raster Join library (librj.so).
 *
 * This is the drop-in boundary for the reference's join layer.  Every entry
 * point below names the reference interface it replaces (paths are relative
 * to the VIDA-NYU/raster-join source tree).  All signatures use plain C types
 * and pointers; no C++ or CUDA types cross the boundary except an opaque
 * cudaStream_t passed as void*.
 *
 * Ownership: input buffers passed as host pointers are copied into device
 * memory owned by the context; result buffers are caller-allocated host
 * memory filled on return.  Functions return RJ_OK (0) or a negative status
 * and never exit the process (the reference called exit(0) on bad input,
 * RasterJoin/join/GLData.cpp:18-23, RasterJoin/join/GLFunction.cpp:251-252).
 */
#ifndef RJ_H
#define RJ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RJ_ABI_VERSION 1

#if defined(__GNUC__)
#define RJ_API __attribute__((visibility("default")))
#else
#define RJ_API
#endif

/* ---- status codes (replace qDebug + empty QVector / exit(0)) ---------- */
#define RJ_OK                      0
#define RJ_E_INVALID              -1   /* bad argument / malformed input        */
#define RJ_E_OOM                  -2   /* device memory budget exceeded         */
#define RJ_E_TOO_MANY_CONSTRAINTS -3   /* > RJ_MAX_CONSTRAINTS (GLFunction.cpp:416) */
#define RJ_E_TIMEOUT              -4   /* a bounded device wait ran out          */
#define RJ_E_CUDA                 -5   /* CUDA runtime error                    */
#define RJ_E_NO_DATA              -6   /* points or polygons not loaded (GLHandler.cpp:190-193) */
#define RJ_E_UNSUPPORTED          -7   /* join type / option not supported      */
#define RJ_E_BUSY                 -8   /* admission refused (serving queue full) */
#define RJ_PENDING                 1   /* rj_poll: the request has not finished yet */

/* ---- limits ------------------------------------------------------------- */
#define RJ_MAX_CONSTRAINTS 10   /* std140 vec4 query[10], RasterJoin/shaders/points.vert:8-10 */
#define RJ_MAX_ATTRIBUTES  16   /* columns a point table may hold (reference: 6, GLFunction.cpp:358) */
#define RJ_MAX_FBO_SIZE    8192 /* canvas tile side, RasterJoin/join/GLFunction.hpp:14 */

/* ---- enums: values identical to the reference ------------------------- */
/* GLHandler::FunctionType, RasterJoin/join/GLHandler.hpp:23-29 */
typedef enum {
    RJ_RASTER_JOIN = 0,      /* RasterJoinFn      */
    RJ_INDEX_JOIN = 1,       /* IndexJoinFn       */
    RJ_HYBRID_JOIN = 2,      /* HybridJoinFn      */
    RJ_RASTER_JOIN_BOUNDS = 3 /* RasterJoinBoundFn */
} rj_function_type;

/* Aggregation, RasterJoin/common/Common.h:34 */
typedef enum { RJ_COUNT = 0, RJ_AVG = 1, RJ_SUM = 2 } rj_aggregation;

/* ConstraintType, RasterJoin/common/Common.h:30 */
typedef enum { RJ_EQ = 0, RJ_LT = 1, RJ_LTE = 2, RJ_GT = 3, RJ_GTE = 4 } rj_constraint_type;

/* AttributeType, RasterJoin/common/Common.h:28 */
typedef enum { RJ_LOCATION = 0, RJ_UINT = 1, RJ_INT = 2, RJ_FLOAT = 3 } rj_attribute_type;

/* Value / QueryConstraint, RasterJoin/common/Common.h:36-47: 16 bytes,
 * same field order (asserted at RasterJoin/main.cpp:376). */
typedef union { int32_t ival; float fval; uint32_t uval; } rj_value;
typedef struct {
    int32_t attrib_id;   /* attribute id of the point table column */
    int32_t type;        /* rj_constraint_type                      */
    rj_value val;        /* comparison value, typed by the column   */
    int32_t dummy;       /* padding, as in the reference            */
} rj_constraint;

/* Semantic switches (named modes for the reference's quirks).  Zero gives
 * the default semantics; each flag reproduces one reference behaviour. */
#define RJ_FLAG_COMPAT_INDEX_CLAMP 0x1u /* GPU grid drops the last column/row:
                                           create-index.glsl:56-61,69-70 */
#define RJ_FLAG_COMPAT_FLOAT_EQ    0x2u /* LTE/GTE equality compares the raw
                                           bit patterns as IEEE floats:
                                           points.vert:98-107 */
#define RJ_FLAG_LINE_FILTER        0x4u /* error bounds keep only pixels whose
                                           centre is within 0.5 px of the edge:
                                           line-bound.frag:221 */
#define RJ_FLAG_FORCE_CANVAS       0x8u /* raster/hybrid: always accumulate a
                                           point canvas (no polygon label map) */
#define RJ_FLAG_PHASE_TIMING       0x10u /* record CUDA events per phase       */
#define RJ_FLAG_NO_CELL_CLASSIFY   0x20u /* index/hybrid: PIP against every MBR
                                           candidate, as index.glsl:389-400 */
#define RJ_FLAG_NO_CACHE           0x40u /* rebuild every polygon-side structure
                                           (grid, labels, masks) for this call,
                                           as each reference execute() does */
#define RJ_FLAG_FLAT_CANVAS        0x80u /* raster: one entry per pixel even for
                                           large canvases (no 16 x 16 block
                                           tiers; same results)              */
#define RJ_FLAG_COUNT_EDGE_TESTS   0x200u /* index/hybrid: count the exact edge tests
                                           into rj_timings.edge_tests (one atomic
                                           per tested point)                  */
#define RJ_FLAG_TIERED_CANVAS      0x100u /* raster: 16 x 16 block tiers for any
                                           canvas of at least 2^24 pixels,
                                           whatever the rows (same results)  */

/* One query: everything GLHandler + DataHandler held between calls
 * (setAccuracyDistance GLHandler.cpp:250, setPolyIndexResolution :259,
 *  setQueryConstraints DataHandler.cpp:64, setAggregation :68). */
typedef struct {
    int32_t function_type;          /* rj_function_type                    */
    int32_t aggregation;            /* rj_aggregation                      */
    int32_t aggr_attrib;            /* column aggregated when != RJ_COUNT  */
    int32_t n_constraints;          /* 0..RJ_MAX_CONSTRAINTS               */
    rj_constraint constraints[RJ_MAX_CONSTRAINTS];
    double accuracy_m;              /* epsilon: pixel diagonal in metres,
                                       GLFunction::setMaxCellSize
                                       GLFunction.cpp:26-30               */
    double cell_size;               /* > 0: pixel side in world units,
                                       overrides accuracy_m                */
    double ground_resolution;       /* metres per world unit (1 for metric
                                       coordinates; UsefulFuncs.cpp:625)   */
    int32_t grid_res;               /* polygon grid index resolution       */
    int32_t max_fbo_size;           /* canvas tile side (0 = 8192), <= 8192 */
    int32_t time_attrib;            /* uint32 column of the time range, or -1 */
    uint32_t t_start, t_end;        /* inclusive range, DataHandler.cpp:107-109 */
    int32_t hybrid_canvas;          /* hybrid canvas long side (0 = 8192,
                                       HybridJoin.cpp:65)                  */
    uint32_t flags;                 /* RJ_FLAG_*                           */
} rj_query;

/* Results.  Host buffers allocated by the caller, npolys entries each (bounds:
 * 4*npolys), any pointer may be NULL if not wanted.
 *   count  : exact per-polygon count            (agg[i], main.cpp:215)
 *   sum    : per-polygon sum of the aggregate   (exact fp64 accumulation)
 *   compat3: the reference's int32[3P] layout [count | sum/100 | decimal*10]
 *            (GLFunction.cpp:42, polygon.frag:17-24), decodable by
 *            printResults main.cpp:206-208
 *   bounds : int32[4P] [fn | fp | fn1 | fp1] (line-bound.frag:250-258) for
 *            RJ_RASTER_JOIN_BOUNDS */
typedef struct {
    int32_t npolys;
    uint64_t *count;
    double *sum;
    int32_t *compat3;
    int32_t *bounds;
} rj_result;

/* Context configuration: GLHandler::getInstance(gpuMemMB, inMemory),
 * RasterJoin/join/GLHandler.cpp:43-69. */
typedef struct {
    int32_t device;          /* CUDA device ordinal                       */
    int64_t gpu_mem_mb;      /* device memory budget (0 = no limit)       */
    void *stream;            /* cudaStream_t to run on (NULL = own stream) */
} rj_config;

/* One point-table column (QueryResult::addAttributeResult,
 * RasterJoin/db/QueryResult.hpp:38-47): RJ_LOCATION columns are float (x,y)
 * pairs, the others 4-byte values. */
typedef struct {
    int32_t attrib_id;
    int32_t type;            /* rj_attribute_type */
    const void *data;
} rj_column;

/* Per-call timings in milliseconds, the fields of the reference's timing line
 * (GLHandler::printTimeStats GLHandler.cpp:214-248, schema
 * experiments/plot-scripts/result_parser.py:5). */
typedef struct {
    uint64_t pts_size;
    int32_t poly_size;
    int32_t function;
    int32_t no_pt_passes;
    int32_t no_constraints;
    double execute_ms;        /* whole rj_execute, host wall clock         */
    double pt_mem_ms;         /* point upload (0 for resident tables)      */
    double pt_render_ms;      /* point pass kernels (CUDA events)          */
    double poly_mem_ms;       /* polygon uploads / derived-structure copies */
    double poly_render_ms;    /* polygon pass kernels (CUDA events)        */
    double setup_ms;          /* host planning                             */
    double triangulation_ms;  /* always 0: no triangulation is needed      */
    double poly_index_ms;     /* grid index build (CUDA events)            */
    double backend_query_ms;  /* always 0: no backend query                */
    int32_t accuracy;         /* accuracy_m for raster joins, else 0       */
    int32_t kernel_launches;  /* kernels this library launched in the call */
    uint64_t edge_tests;      /* exact edge tests of the index / hybrid join
                                 (counted with RJ_FLAG_COUNT_EDGE_TESTS, else 0) */
} rj_timings;

typedef struct rj_ctx rj_ctx;

/* ---- context ------------------------------------------------------------ */
/* replaces GLHandler::getInstance + initializeGL + initFunctions
 * (GLHandler.cpp:43-69,157-186). */
RJ_API int rj_create(const rj_config *cfg, rj_ctx **out);
/* replaces GLHandler::~GLHandler (GLHandler.cpp:56-62) */
RJ_API void rj_destroy(rj_ctx *ctx);
/* human-readable text of the last failing call on this context */
RJ_API const char *rj_last_error(const rj_ctx *ctx);
/* run subsequent work on a caller stream (cudaStream_t) */
RJ_API int rj_set_stream(rj_ctx *ctx, void *stream);
RJ_API int rj_abi_version(void);

/* ---- point table: DataHandler::initData + executeQuery result columns
 * (DataHandler.cpp:24-62,86-96); GLFunction::setupPoints GLFunction.cpp:199-344 */
RJ_API int rj_load_points(rj_ctx *ctx, const rj_column *cols, int32_t ncols,
                   uint64_t npoints, int32_t loc_attrib);
/* same, but the data pointers are device pointers (16-byte aligned) that the
 * caller keeps alive; nothing is copied */
RJ_API int rj_attach_points_device(rj_ctx *ctx, const rj_column *cols, int32_t ncols,
                            uint64_t npoints, int32_t loc_attrib);
/* Out-of-core table: the data pointers are HOST pointers that the caller
 * keeps alive; nothing is copied at load.  Every query streams the columns
 * it reads through the device in chunks of chunk_points rows (0: sized from
 * the memory budget), copying chunk k+1 while chunk k is processed (the
 * reference's memory passes, GLFunction.cpp:330-337, RasterJoin.cpp:215-236;
 * rj_timings.no_pt_passes counts the chunks).  Pinned host memory lets the
 * copies overlap the point pass.  Batches run such a table query by query. */
RJ_API int rj_attach_points_host(rj_ctx *ctx, const rj_column *cols, int32_t ncols,
                                 uint64_t npoints, int32_t loc_attrib, uint64_t chunk_points);
/* Host-resident table read in place: the data pointers are page-locked host
 * memory (cudaMallocHost / cudaHostAlloc, or registered with cudaHostRegister;
 * 16-byte aligned) that the caller keeps alive.  Nothing is copied: every
 * query's point pass reads the columns over the host link (NVLink-C2C on
 * Grace systems), so the table crosses the link once per query with no
 * staging buffers and no copy engine.  RJ_E_INVALID for memory the device
 * cannot address.  Results equal a resident table's.  No counterpart in the
 * reference (its memory passes copy chunks, GLFunction.cpp:330-337). */
RJ_API int rj_attach_points_mapped(rj_ctx *ctx, const rj_column *cols, int32_t ncols,
                                   uint64_t npoints, int32_t loc_attrib);
RJ_API int rj_free_points(rj_ctx *ctx);

/* ---- polygons: PolyHandler::addPolygonCollection (PolyHandler.cpp:49-80).
 * xy: float pairs of all polygons back to back (PolyHandler "polys"),
 * pindex: npolys+1 offsets in vertices ("pindexes").  Polygons are open rings
 * (last vertex != first, PolyHandler.cpp:165-167).  bbox (minx,miny,maxx,maxy)
 * may be NULL: it is then the vertex bounds, as readPolygons computes
 * (PolyHandler.cpp:178-186). */
RJ_API int rj_set_polygons(rj_ctx *ctx, const float *xy, const int32_t *pindex,
                    int32_t npolys, const double *bbox);

/* ---- execution: GLHandler::executeFunction (GLHandler.cpp:188-204) and
 * getErrorBounds (GLHandler.cpp:206-212) in one call. */
RJ_API int rj_execute(rj_ctx *ctx, const rj_query *q, rj_result *res);

/* Fill q with the reference defaults: count, no constraints, accuracy 100 m
 * (main.cpp:268), grid 256 (main.cpp:299), canvas tile 8192. */
RJ_API void rj_query_init(rj_query *q);

/* ---- timings: GLHandler::printTimeStats (GLHandler.cpp:214-248) --------- */
RJ_API int rj_get_timings(const rj_ctx *ctx, rj_timings *out);
/* the reference's tab-separated timing line for the last call */
RJ_API int rj_format_time_stats(const rj_ctx *ctx, char *buf, size_t buflen);

/* ---- exact partial sums (replicas over row shards) ------------------------
 * Sums are exact int64 sums of round(v * 2^shift) per polygon; the double
 * sum of rj_result is fixed * 2^-shift + nonfinite (the fp64 sum of the
 * non-finite values).  Replicas that join row shards of one table add their
 * int64 partials (two's complement, wrapping) and decode once, which gives
 * the bits of the single-GPU join, provided every shard uses the shift the
 * whole table would: rj_sum_shift_for(largest |value| over all shards, total
 * rows).  The reference has no counterpart (one process, one GPU).
 *   rj_get_sum_partials: the last rj_execute's fixed and non-finite partials
 *     (npolys entries each; either pointer may be NULL) and its shift.
 *   rj_set_sum_shift: use this shift for subsequent sums (RJ_SUM_SHIFT_AUTO:
 *     chosen per query from the aggregate column and the table size).  A
 *     query whose values could overflow at the forced shift on this table
 *     fails with RJ_E_INVALID.
 *   rj_sum_shift_for: the shift chosen for values of magnitude <= max_abs
 *     over `rows` rows.
 *   rj_column_absmax: largest finite |aggregate value| of a loaded column. */
#define RJ_SUM_SHIFT_AUTO (-2147483647 - 1)
RJ_API int rj_get_sum_partials(const rj_ctx *ctx, int64_t *fixed, double *nonfinite, int32_t *shift);
RJ_API int rj_set_sum_shift(rj_ctx *ctx, int32_t shift);
RJ_API int32_t rj_sum_shift_for(double max_abs, uint64_t rows);
RJ_API int rj_column_absmax(const rj_ctx *ctx, int32_t attrib_id, double *out);

/* ---- kernel tuning ---------------------------------------------------------
 * Kernel shapes of this context.  Every shape computes the same result; the
 * knobs only choose how the work is laid out on the GPU.  The reference has
 * no counterpart (its point pass is one glDrawArrays, RasterJoin.cpp:135).
 *   RJ_TUNE_POINT_SHAPE      generic point pass: -1 = default per join,
 *                            0 = 4 points x 256 threads, 2 = bulk-copy
 *                            pipeline, 3 = 4 points x 512 threads
 *   RJ_TUNE_COUNT_SHAPE      lean raster label pass (one canvas tile, label
 *                            map, a resident table): -1 = autotuned (each
 *                            shape is timed once per context and query
 *                            class on the table itself, the fastest is
 *                            kept), else a shape index
 *                            0..rj_get_tuning(RJ_TUNE_COUNT_SHAPES)-1
 *   RJ_TUNE_COUNT_BLOCK_SHIFT block-code map of that pass: -1 = autotuned,
 *                            else log2 of the block side (4..8)
 *   RJ_TUNE_HYBRID_EXACT_SCALE classified grid of the hybrid join's exact
 *                            tests: the query grid refined 1, 2 or 4 times
 *   RJ_TUNE_COUNT_SHAPES     (read only) number of plain count-pass shapes
 *   RJ_TUNE_LEAN_SHAPES      (read only) number of shapes of the same pass
 *                            with filters (interval form, <= 4 columns) or
 *                            a summed aggregate; RJ_TUNE_COUNT_SHAPE indexes
 *                            the shapes of the form the query takes
 *   RJ_TUNE_SPLAT_SHAPES     (read only) number of shapes of the lean pass
 *                            onto a point canvas (one canvas tile: polygon
 *                            sets that overlap on it, the error-bounds
 *                            join); RJ_TUNE_COUNT_SHAPE indexes them there
 *                            too (canvas copies in shared memory, or
 *                            atomics into the canvas in global memory)
 *   RJ_TUNE_HYBRID_SHAPES    (read only) number of shapes of the lean pass
 *                            of the hybrid and index joins; RJ_TUNE_COUNT_SHAPE
 *                            indexes them there
 *   RJ_TUNE_WAIT_LIMIT       microseconds a bounded device wait of the
 *                            bulk-copy pipeline (RJ_TUNE_POINT_SHAPE 2) may
 *                            take before it gives up and the call returns
 *                            RJ_E_TIMEOUT (default 1000000, one second; the
 *                            wait for copies still in flight at the end of a
 *                            block keeps that default)
 * rj_get_tuning on RJ_TUNE_COUNT_SHAPE / _BLOCK_SHIFT reports the values the
 * last count pass ran with (-1 when the last query did not take it). */
#define RJ_TUNE_POINT_SHAPE        0
#define RJ_TUNE_COUNT_SHAPE        1
#define RJ_TUNE_COUNT_BLOCK_SHIFT  2
#define RJ_TUNE_HYBRID_EXACT_SCALE 3
#define RJ_TUNE_COUNT_SHAPES       4
#define RJ_TUNE_LEAN_SHAPES        5
#define RJ_TUNE_WAIT_LIMIT         6
#define RJ_TUNE_SPLAT_SHAPES       7
#define RJ_TUNE_HYBRID_SHAPES      8
RJ_API int rj_set_tuning(rj_ctx *ctx, int32_t knob, int32_t value);
RJ_API int rj_get_tuning(const rj_ctx *ctx, int32_t knob, int32_t *value);

/* ---- prepared queries (CUDA graphs) ----------------------------------------
 * rj_prepare runs q once (settling the caches the query uses: polygon-side
 * structures, the polygon set's overlap status on the canvas, autotuned
 * shapes) and captures the device work of one more execution -- polygon side,
 * point pass, result copies -- into a CUDA graph.  rj_execute_prepared replays
 * it on the context's stream: the same results as rj_execute(ctx, q, res),
 * without host planning or per-kernel launch costs.  Work that rj_execute
 * does with NO_CACHE is redone on every replay.
 * The plan stays valid while the table keeps its buffers (rj_load_points
 * with the same columns and size copies into them in place), the context
 * keeps the same polygon set and stream, the aggregate's fixed-point scale is
 * unchanged and, for a query whose rows the time index narrowed, that index
 * still describes the rows (a reload drops it); else rj_execute_prepared
 * returns RJ_E_INVALID.  The
 * zone map is not used by a plan (a reloaded table needs none).
 * Queries whose execution reads a value back to the host before it can go
 * on cannot be captured (tiered canvases, an index or hybrid join that
 * rebuilds its grid each call): rj_prepare returns RJ_E_UNSUPPORTED, as it
 * does for host-streamed tables.  No counterpart in the reference (each
 * GLHandler::executeFunction re-issues its draws, GLHandler.cpp:188-204). */
typedef struct rj_plan rj_plan;
RJ_API int rj_prepare(rj_ctx *ctx, const rj_query *q, rj_plan **out);
RJ_API int rj_execute_prepared(rj_plan *plan, rj_result *res);
RJ_API void rj_plan_destroy(rj_plan *plan);

/* ---- failure handling ------------------------------------------------------
 * Runs the library's bounded device wait alone: one block waits, at most
 * limit_us microseconds, on a barrier that nothing completes, so the wait runs out
 * and the call returns RJ_E_TIMEOUT the way a join does when a bounded wait
 * of its pipeline runs out (the kernel returns; the context stays usable).
 * RJ_OK would mean the wait did not run out.  The reference has no
 * counterpart: it had no device-side waits and exit(0)ed on errors
 * (GLData.cpp:18-23, GLFunction.cpp:251-252). */
RJ_API int rj_selftest_bounded_wait(rj_ctx *ctx, uint32_t limit_us);

/* ---- polygon sets --------------------------------------------------------
 * A polygon collection held on the device independently of the context's own
 * set (the reference keeps one PolyHandler per collection,
 * RasterJoin/db/PolyHandler.cpp:20-80; setPolygonQuery DataHandler.cpp:73-75
 * selects one).  Same arguments as rj_set_polygons.  A set belongs to the
 * context that created it; destroy it before the context. */
typedef struct rj_polyset rj_polyset;
RJ_API int rj_polyset_create(rj_ctx *ctx, const float *xy, const int32_t *pindex, int32_t npolys,
                             const double *bbox, rj_polyset **out);
RJ_API void rj_polyset_destroy(rj_polyset *ps);
/* make ps the polygon set of rj_execute (NULL: the set of rj_set_polygons) */
RJ_API int rj_use_polyset(rj_ctx *ctx, rj_polyset *ps);

/* ---- time index ----------------------------------------------------------
 * Reorders the resident table's rows into nbuckets buckets of the uint32
 * column time_attrib (a counting sort; every column moves with its row), so a
 * query whose time range is on that column reads only the rows of the
 * buckets it overlaps; the exact inclusive time predicate still applies.
 * Stands in for the reference backend's time partitions
 * (HashGridIndex.cpp:114-137), which selected whole partitions.  Results are
 * unchanged (they do not depend on row order).  nbuckets 0 = 16384
 * (at most 16384).  Device-attached tables are copied into library-owned
 * buffers.  Reloading the table drops the index. */
RJ_API int rj_build_time_index(rj_ctx *ctx, int32_t time_attrib, int32_t nbuckets);
/* Clustered row order: rows sorted by time bucket (when time_attrib >= 0,
 * which also builds the time index above) and, inside a bucket, by the
 * Z-order of a 2^cell_bits x 2^cell_bits grid over the location bounds
 * (cell_bits 0..12; buckets x cells <= 2^24).  Neighbouring rows then map to
 * neighbouring pixels: label gathers hit the cache and a warp's points merge
 * into few histogram updates.  The reference's backend stores points in
 * spatio-temporal partitions for the same reason (HashGridIndex.cpp:98-113).
 * time_attrib < 0: spatial order only (no time index).  Results are
 * unchanged. */
RJ_API int rj_cluster_points(rj_ctx *ctx, int32_t time_attrib, int32_t nbuckets, int32_t cell_bits);

/* ---- batched execution ---------------------------------------------------
 * No counterpart in the reference (one executeFunction per query).  Runs nq
 * queries over the resident table; sets[i] is query i's polygon set (NULL:
 * the context's own).  Raster joins with interval-form filters run fused: one
 * point pass for the whole batch reads each row once for every query whose
 * time window covers it.  Every other query (other join types,
 * RJ_FLAG_COMPAT_FLOAT_EQ, more distinct columns than one pass stages) runs
 * through rj_execute.  res[i] is filled like rj_execute's result; status[i]
 * (may be NULL) receives each query's status.  Returns RJ_OK when every
 * query succeeded, else the first failing status. */
#define RJ_BATCH_AUTOTUNE 0x1u   /* time the fused pass's block shapes on this batch and keep the fastest */
#define RJ_BATCH_NO_FUSE  0x2u   /* run every query through rj_execute in turn (the plain path) */
#define RJ_BATCH_FUSE_ALL 0x4u   /* fuse every raster query */
#define RJ_BATCH_FUSE     0x8u   /* fuse the raster queries over fewer than 2^22
                                    rows or on multi-tile canvases; the others
                                    take the lanes */
/* By default every raster query of a batch takes rj_execute's device path on
 * one of eight lanes: streams with their own scratch, so that the work of
 * several queries overlaps on the GPU (and, with RJ_BATCH_FUSE, with the
 * fused pass); each lane's outputs come back through pinned staging, with one
 * wait for the whole batch.  Queries of one polygon set share a lane.
 * Results are those of rj_execute, bit for bit, on every route; `fallback`
 * counts the queries that did not run fused.  A serving loop's batches use
 * the fused pass (its slots allocate nothing while serving). */
typedef struct {
    int32_t nqueries, fused, fallback;
    int32_t segments;              /* row ranges covered by one set of queries */
    uint64_t items;                /* work items of the fused point pass       */
    uint64_t rows_read;            /* rows staged from HBM (each once)         */
    uint64_t point_queries;        /* sum over fused queries of rows scanned   */
    double total_ms;               /* host wall clock of the call              */
    double setup_ms;               /* host planning                            */
    double poly_ms;                /* label maps / canvases (CUDA events)      */
    double point_ms;               /* fused point pass (CUDA events)           */
    double reduce_ms;              /* canvas polygon passes (CUDA events)      */
    int32_t threads, rows_per_item;   /* block shape of the fused point pass  */
    int32_t direct;                   /* 1: rows streamed per query from L2, 0: staged in shared memory */
    int32_t tuned;
    int32_t kernel_launches;
} rj_batch_stats;
RJ_API int rj_execute_batch(rj_ctx *ctx, int32_t nq, const rj_query *q, rj_polyset *const *sets,
                            rj_result *res, int32_t *status, uint32_t flags, rj_batch_stats *stats);

/* ---- serving -------------------------------------------------------------
 * No counterpart in the reference.  A request loop over the context's
 * resident table: rj_submit queues a query (copied) with its polygon set and
 * caller-owned result buffers (valid until rj_poll reports completion).  A
 * scheduler thread forms batches from the queued requests as slots free up,
 * admitting requests while the batch's canvases and label maps fit the
 * slot's memory (canvas_mb); up to `slots` batches are on the GPU at once
 * (polygon-side work of one overlaps the point pass of another).  While a
 * server runs, the context accepts no other calls (RJ_E_BUSY). */
typedef struct {
    int32_t slots;                 /* batches in flight (0 = 2)                 */
    int64_t canvas_mb;             /* device memory per slot (0 = 8192)         */
    int32_t max_batch;             /* requests per batch (0 = 256)              */
    double max_wait_ms;            /* hold a batch open for more arrivals (0 = launch at once) */
    uint32_t batch_flags;          /* how a slot runs its batch: 0 = the lanes
                                      (each request's own device path on four
                                      streams of the slot, whose scratch is
                                      allocated on first use), RJ_BATCH_FUSE =
                                      the fused pass in the slot's fixed arena
                                      (nothing allocated while serving)       */
} rj_server_config;
typedef struct {
    double submit_ms, start_ms, done_ms;   /* steady-clock milliseconds            */
    int32_t batch_id, batch_size, status;
} rj_request_info;
typedef struct rj_server rj_server;
RJ_API int rj_server_create(rj_ctx *ctx, const rj_server_config *cfg, rj_server **out);
RJ_API int rj_submit(rj_server *srv, const rj_query *q, rj_polyset *ps, rj_result *res, uint64_t *ticket);
/* RJ_OK when the request is done (info filled), RJ_PENDING if it is still
 * running after timeout_ms (< 0: wait without limit) */
RJ_API int rj_poll(rj_server *srv, uint64_t ticket, int32_t timeout_ms, rj_request_info *info);
/* finishes the queued requests, then stops */
RJ_API void rj_server_destroy(rj_server *srv);

/* ---- allocation-free raster count ----------------------------------------
 * No counterpart in the reference.  For callers that may not allocate device
 * memory (hosts that budget every byte of GPU memory themselves, loops that
 * must not stall on an allocation, processes already at the memory limit):
 * the bounded raster join, count per polygon, over device-resident points and
 * polygons, with all scratch taken from one fixed device array inside the
 * library (about 19 MiB, held by every GPU that loads the library until the
 * process exits).  Limits: canvas ceil(dx/cell) x ceil(dy/cell) <= 2048 x 2048
 * (one tile), npolys <= 65536, nverts <= 262144 and d_pindex[npolys] ==
 * nverts; larger requests return RJ_E_INVALID with a message in err.
 * d_xy (float x,y pairs, 16-byte aligned), d_verts and d_pindex follow
 * rj_load_points / rj_set_polygons; bbox is the polygon bounds (host, 4
 * doubles); d_count receives npolys counts (overwritten).  Work is queued on
 * `stream` and the call returns without waiting.  Calls share the array:
 * calls that overlap on the GPU race and give wrong counts.  The first call
 * on a device looks up the array's device address; make it before capturing
 * that stream.  Results equal rj_execute's RJ_RASTER_JOIN counts with
 * cell_size and no constraints. */
RJ_API int rj_raster_count_noalloc(const float *d_xy, uint64_t npoints, const float *d_verts,
                                   const int32_t *d_pindex, int32_t npolys, int32_t nverts,
                                   const double *bbox, double cell_size, unsigned long long *d_count,
                                   void *stream, char *err, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif /* RJ_H */
