// rj_launch.h -- kernel argument structs and launcher declarations shared by
// the kernel translation units and the host runtime.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "rj_device.cuh"

namespace rj {

enum { MODE_REDUCE = 0, MODE_LABEL = 1, MODE_BOUNDS = 2, MODE_TIER_CLASSIFY = 3, MODE_TIER_LABEL = 4,
       MODE_TIER_REDUCE = 5 };

// Tiered canvas: 16 x 16-pixel blocks; per-pixel data only for mixed blocks.
constexpr uint32_t kTierEmpty = 0xFFFFFFFFu;   // no polygon reaches the block
constexpr uint32_t kTierMulti = 0xFFFFFFFEu;   // two or more polygons cover it whole
constexpr uint32_t kTierMixed = 0x80000000u;   // | slot: per-pixel data in the slot
struct TierArgs {
    int bw, bh;                  // blocks per tile row / per tile column
    uint32_t* full;              // [nblk] polygon covering the whole block, kTierEmpty, kTierMulti
    uint32_t* mixed;             // [nblk] 1: per-pixel block
    const int* slot;             // [nblk] exclusive scan of mixed
    uint32_t* code;              // [nblk] lookup code (full polygon / empty / multi / mixed | slot)
    uint16_t* plabel;            // [nslots * 256] pixel labels of mixed blocks
    uint32_t* bcnt;              // [nblk] point counts of the blocks neither mixed nor empty (canvas form)
    long long* bsum;             // [nblk] block fixed-point sums or null
    uint32_t* pcnt;              // [nslots * 256] pixel counts of mixed blocks
    long long* psum;             // [nslots * 256] or null
    int outline;                 // classification: also make every block within two
                                 // pixels of an edge mixed (the error-bound outline
                                 // pass reads per-pixel counts there)
};


// Kernels launched by this thread since the last reset (reported per call).
extern thread_local int g_kernel_launches;

struct PolyPassArgs {
    const int2* wv;              // [T][V] fixed-point window coordinates
    const float2* wf;            // [T][V] fp32 window coordinates (bounds)
    const int* pindex;           // [P+1]
    int P, V, T;
    int resx, resy;
    const uint32_t* canvas_c;    // [T][resy][resx] point counts
    const long long* canvas_s;   // [T][resy][resx] fixed-point sums or null
    uint16_t* label;             // [T][resy][resx] polygon label (MODE_LABEL)
    unsigned long long* covered; // MODE_LABEL: pixels covered, summed over polygons
    const uint32_t* border;      // dilated hybrid border mask (skip) or null
    int border_words;
    unsigned long long* out_count;
    unsigned long long* out_sum; // fixed-point sums (int64 two's complement)
    long long* out_bounds;       // [4P]
    unsigned int* work_ctr;
    int line_filter;
    // per (tile, polygon) work description (k_poly_info)
    int4* info_a;                // i_lo, i_hi, r_lo, r_hi
    int2* info_b;                // j_lo, j_hi (rows whose centre can be crossed)
    int* nbands;                 // bands of kBand rows
    const int* band_start;       // exclusive scan of nbands, [T*P + 1]
    // MODE_BOUNDS over a tiered canvas (with TierArgs::outline): per-pixel
    // counts from the mixed blocks' slots, no per-pixel reduction (the tier
    // reduction gives the counts); a lookup outside a mixed block sets err
    int outline_rows;            // tier classification for error bounds: bands over
                                 // every row an edge touches (k_poly_info)
    const uint32_t* tier_code;   // [T][bh][bw] or null (flat canvas)
    const uint32_t* tier_pcnt;
    int tier_bw, tier_bh;
    int* err;
};

size_t tier_smem_bytes();
void launch_tier_pass(int mode, const PolyPassArgs& a, const TierArgs& tr, int sms, cudaStream_t st);
void launch_tier_codes(const TierArgs& tr, size_t nblk, unsigned long long* multi, int sms, cudaStream_t st);
void launch_tier_nonempty(const uint16_t* plabel, size_t n, unsigned long long* count, int sms, cudaStream_t st);

struct GridArgs {
    const float2* verts;
    const int* pindex;
    int P;
    float lbx, lby, csx, csy;
    int res;
    int compat_clamp;
    int* cell_count;
    const int* cell_start;
    int* cursor;
    int* entries;
    int* pair_cell;              // optional: cell of every entry
};

// Classified grid: every (cell, candidate polygon) pair is FULL (every point
// of the cell is inside), OUT (none is; dropped) or EDGE (points need the
// crossing test, against the few edges that can change its outcome).
struct ClsArgs {
    const float2* verts;
    const int* pindex;
    int P;
    // level 1: candidate pairs over coarse cells (the query grid), polygon-major
    const int* pair_off;         // [P+1] first coarse pair of each polygon
    const int4* prange;          // [P] coarse candidate cells [stx, enx) x [sty, eny)
    int npairs;                  // pairs of the level being classified
    // level 2: explicit (polygon, fine cell) pairs refined from EDGE coarse pairs
    int2* plist;
    int* plist_n;
    int level;                   // 1 or 2
    int scale;                   // fine cells per coarse cell along an axis
    float lbx, lby, csx, csy;    // fine grid lower-left / cell size (fp32, as the points use)
    int res;                     // fine grid resolution
    float margin;                // world units: fp32 error of the test + cell assignment
    int4* info;                  // level 1: poly, kind (-1 full, -2 out, 0 edge), -, coarse cell
                                 // level 2: poly, nr (-1 full, -2 out), nf, fine cell
    int* ecount;                 // level 2: edges kept per pair
    const int* eoff;             // level 2: first edge (exclusive scan of ecount)
    float4* edges;
    int* cell_kept;              // per fine cell: kept entries
    const int* cell_start;       // per fine cell: exclusive scan of cell_kept
    int* cursor;
    int4* entries;               // cell-major: poly, nr, nf, edge offset
};

struct ExactIndex {
    const uint32_t* code;        // [res*res] polygon id of a cell inside exactly one polygon,
                                 // kCodeEmpty, or kCodeList (consult the entries)
    const int* cell_start;       // [res*res + 1] classified CSR
    const int4* entries;         // poly, nr (-1: full cell), nf, edge offset
    const float4* edges;         // (vi.x, vi.y, vj.x, vj.y): nr straddle-only edges, then nf full
    float lbx, lby, csx, csy;    // resolution = query grid resolution * 2^k
    int res;
    unsigned long long* tests;   // exact edge tests counted here, or null
};

// Per-axis tile transforms of a raster canvas.
struct CanvasXf {
    const float4* colxf;         // [splitx] (sx, tx, hx, tile_dx)
    const float4* rowxf;         // [splity] (sy, ty, hy, tile_dy)
    int splitx, splity;
    int resx, resy;
    float lbx, lby;              // canvas lower-left (fp32), for the tile guess
    float tdx, tdy;              // tile extent (fp32), for the tile guess
    float4 col0, row0;           // transform of column 0 / row 0 (single-tile fast path)
};

// Point-table view for the point kernels.
struct PointArgs {
    const float2* xy;
    uint64_t n;
    DevFilter f;
    int P;
    unsigned long long* out_count;
    unsigned long long* out_sum; // fixed-point sums (int64 two's complement)
    double* out_nonfinite;       // fp64 sums of the non-finite aggregate values
    int* err;                    // bit0: a bounded pipeline wait ran out
    uint32_t* out_count32;       // when set, the shared histogram flushes counts here (a u32 canvas)
    // zone map: bounds of every kZoneRows rows of the table (row0 = table row
    // of xy[0]); iterations whose rows lie apart from qbox are skipped
    const float4* zones;
    uint64_t row0;
    float4 qbox;
    int shape = -1;              // kernel shape (-1: the default for the mapper)
    uint64_t wait_ns = kWaitLimitNs;    // wall time a bounded pipeline wait may take before it gives up
};
constexpr int kZoneShift = 10;               // zones of 1024 rows
void launch_zone_boxes(const float2* xy, uint64_t n, float4* zones, int sms, cudaStream_t st);
// per-tile transforms written by a kernel from its arguments (no host copy;
// used while a query is captured into a graph)
constexpr int kXfArgs = 16;
struct XfArgs {
    float4 v[kXfArgs];
};
void launch_write_xf(const XfArgs& a, int n, float4* dst, cudaStream_t st);
// one CTA waits, bounded by limit_ns of wall time, on an mbarrier nothing
// arrives on; sets bit 0 of *err when the wait runs out
void launch_wait_selftest(int* err, uint64_t limit_ns, cudaStream_t st);

// Exact point-in-polygon index (CSR over a uniform grid).
struct IndexArgs {
    const float2* verts;
    const int* pindex;
    const int* cell_start;       // [res*res + 1]
    const int* entries;
    float lbx, lby, csx, csy;
    int res;
};

struct HybridArgs {
    HybXf h;
    const uint32_t* border;      // dilated border mask [resy][words] (canvas mode)
    int words;
    uint32_t* canvas_c;          // canvas mode: [resy][resx]
    long long* canvas_s;         // fixed-point sums
    float scale;                 // fixed-point scale 2^(s-32)
    const uint16_t* label;       // label mode: [resy][resx], kBorderLabel on border pixels
};

// column statistics: largest finite |aggregate value| as float bits (atomicMax)
void launch_col_absmax(const uint32_t* col, int typ, uint64_t n, unsigned* out_bits, int sms, cudaStream_t st);

// polygon side
void launch_transform_vertices(const float2* verts, int V, const float4* colxf, const float4* rowxf,
                               int splitx, int T, int2* wv, float2* wf, int sms, cudaStream_t st);
void launch_poly_info(int mode, const PolyPassArgs& a, int sms, cudaStream_t st);
void launch_poly_pass(int mode, const PolyPassArgs& a, int sms, cudaStream_t st);
void launch_grid_count(const GridArgs& g, int sms, cudaStream_t st);
void launch_grid_fill(const GridArgs& g, int sms, cudaStream_t st);
void launch_grid_sort(const int* cell_start, int* entries, int ncells, int sms, cudaStream_t st);
int scan_tmp_ints(int n);
bool launch_exclusive_scan(const int* in, int* out, int n, int* tmp, cudaStream_t st);
void launch_outline_mask(const float2* verts, const int* pindex, int P, const int* edge_poly, int V,
                         const HybXf& h, float margin, uint32_t* mask, int words, int sms, cudaStream_t st);
void launch_dilate_mask(const uint32_t* in, uint32_t* out, int resx, int resy, int words, int radius,
                        int sms, cudaStream_t st);

// Lean raster count over one canvas tile with a polygon label map
// (rj_count_kernels.cu): no filter, count only.
struct LabelCountArgs {
    const float4* xy;            // location column as point pairs, 16-byte aligned
    uint64_t n;                  // points
    float4 col0, row0;           // the tile transform (s, t, h) per axis
    int resx, resy;
    const uint16_t* label;       // [resy][resx] polygon label, kEmptyLabel outside every polygon
    const uint16_t* codes;       // [nby][nbx] block codes (label shared by the block, or mixed)
    int bs;                      // log2 of the block side
    int nbx;                     // blocks per canvas row
    int code_words;              // 32-bit words of the code map (its u16 count rounded up)
    int P;
    unsigned long long* out_count;
    // zone map (bounds of every 1024 rows; zrow0 = table row of xy[0]) or null
    const float4* zones;
    uint64_t zrow0;
    float4 qbox;
};
// Filters (interval form, <= 4 columns) and the summed aggregate of the lean
// label pass with attributes (rj_lean_kernels.cu).
struct LeanCols {
    int ncol;
    const uint2* col[4];         // filter columns, read as value pairs (8-byte aligned)
    uint32_t lo[4], span[4];     // the predicates of column c hold iff key - lo <= span
    uint32_t fm[4], xm[4];       // order key = v ^ ((sign(v) & fm) ^ xm)
    int aggr;                    // 1: sum the aggregate
    int aggr_ci;                 // the aggregate is filter column aggr_ci, or -1
    const uint2* aggr_col;       // else this column
    int aggr_typ;
    float scale;                 // fixed-point scale 2^(s-32)
    double* nonfinite;           // fp64 sums of non-finite values
    unsigned long long* out_sum; // int64 fixed-point sums
    int copies;                  // histogram copies (set by the launcher)
};
void launch_block_codes(const uint16_t* label, int resx, int resy, int bs, int nbx, int nby, uint16_t* codes,
                        int sms, cudaStream_t st);
// Lean point pass of the hybrid join over its label map (rj_hybrid_lean.cu).
struct HybLeanArgs {
    const float4* xy;            // location column as point pairs, 16-byte aligned
    uint64_t n;
    HybXf h;                     // hybrid canvas (rasterize, hybrid.glsl:187-200)
    const uint16_t* label;       // [resy][resx] label, kBorderLabel near outlines, kEmptyLabel
    const uint16_t* codes;       // block codes of the label map
    int bs, nbx, code_words;
    int P;
    unsigned long long* out_count;
    const float4* zones;         // zone map or null
    uint64_t zrow0;
    float4 qbox;
    ExactIndex ix;               // classified grid of the exact tests
    // mode 0: the hybrid canvas; the pixel of a point comes from one FMA per
    // axis, fast = (Ax, Bx, Ay, By) with pixel coordinate = v * A + B, inside
    // the canvas less a 2-pixel rim (near the rim: the exact rasterize)
    // mode 1: the classified grid's cells (index join); label holds per cell
    // the one polygon a FULL cell lies in, kBorderLabel for cells with a
    // candidate list, kEmptyLabel for empty cells
    int mode;
    float4 fast;
};
void launch_cell_labels(const uint32_t* code, int ncells, uint16_t* label, int sms, cudaStream_t st);
int hybrid_lean_shapes();
size_t hybrid_lean_smem(int shape, int code_words, int P, bool agg);
bool launch_hybrid_lean(int shape, const HybLeanArgs& a, const LeanCols& lc, int sms, cudaStream_t st);
int label_lean_shapes();
int label_lean_max_cols();
size_t label_lean_smem(int shape, int code_words, int P, bool agg);
bool launch_label_lean(int shape, const LabelCountArgs& a, const LeanCols& lc, int sms, cudaStream_t st);
// Lean point pass onto a point canvas (rj_splat_kernels.cu): one canvas tile,
// interval-form filters on at most four columns (LeanCols), count and sum.
struct SplatLeanArgs {
    const float4* xy;            // location column as point pairs, 16-byte aligned
    uint64_t n;
    float4 col0, row0;           // the tile transform (s, t, h) per axis
    int resx, resy;
    uint32_t* canvas_c;          // [resy][resx] counts
    unsigned long long* canvas_s; // [resy][resx] int64 fixed-point sums, or null
    const float4* zones;         // zone map or null (as LabelCountArgs)
    uint64_t zrow0;
    float4 qbox;
};
// Lean point pass over a tiered canvas (rj_tier_lean.cu): one or several
// canvas tiles, the label form (histogram per polygon) or the canvas form
// (block and mixed-pixel sums), interval-form filters (LeanCols).
struct TierLeanArgs {
    const float4* xy;            // location column as point pairs, 16-byte aligned
    uint64_t n;
    const float4* colxf;         // [splitx] (s, t, h, tile extent) per tile column
    const float4* rowxf;         // [splity]
    int splitx, splity;
    int resx, resy;              // tile resolution
    float lbx, lby;              // canvas lower-left, for the tile guess
    float inv_tdx, inv_tdy;      // 1 / tile extent, for the tile guess
    TierArgs tr;
    int P;
    unsigned long long* out_count;
    const float4* zones;         // zone map or null (as LabelCountArgs)
    uint64_t zrow0;
    float4 qbox;
};
int tier_lean_shapes();
size_t tier_lean_smem(bool label, int P, bool agg);
bool launch_tier_lean(int shape, bool label, const TierLeanArgs& a, const LeanCols& lc, int sms, cudaStream_t st);
int splat_lean_shapes();
// shared memory of a shape for a canvas (1 for the global-atomic shapes), 0
// when the canvas does not fit
size_t splat_lean_smem(int shape, size_t npix, bool agg);
bool launch_splat_lean(int shape, const SplatLeanArgs& a, const LeanCols& lc, int sms, cudaStream_t st);
int label_count_shapes();
size_t label_count_smem(int shape, int code_words, int P);
bool launch_label_count(int shape, const LabelCountArgs& a, int sms, cudaStream_t st);

// point side
// smem_hist: histogram capacity decision done by the launcher.
void launch_raster_splat(const PointArgs& pa, const CanvasXf& cx, uint32_t* canvas_c, long long* canvas_s,
                         int sms, cudaStream_t st);
void launch_raster_label(const PointArgs& pa, const CanvasXf& cx, const uint16_t* label, int sms,
                         cudaStream_t st);
void launch_tier_label_points(const PointArgs& pa, const CanvasXf& cx, const TierArgs& tr, int sms, cudaStream_t st);
void launch_tier_splat_points(const PointArgs& pa, const CanvasXf& cx, const TierArgs& tr, int sms, cudaStream_t st);
void launch_index_points(const PointArgs& pa, const IndexArgs& ia, int sms, cudaStream_t st);
void launch_exact_points(const PointArgs& pa, const ExactIndex& ix, int sms, cudaStream_t st);
void launch_hybrid_points(const PointArgs& pa, const ExactIndex& ix, const HybridArgs& ha, int sms,
                          cudaStream_t st);

// classified grid build
void launch_cls_classify(const ClsArgs& c, int sms, cudaStream_t st);
void launch_cls_emit(const ClsArgs& c, int sms, cudaStream_t st);   // level-1 FULL and level-2 kept pairs
void launch_cls_fill_edges(const ClsArgs& c, int sms, cudaStream_t st);
// count labelled pixels (before border marking) and mark border pixels
void launch_label_finish(uint16_t* label, const uint32_t* mask, int resx, int resy, int ntiles, int words,
                         unsigned long long* nonempty, int sms, cudaStream_t st);
void launch_cls_codes(const int* cell_start, const int4* entries, uint32_t* code, int ncells, int sms,
                      cudaStream_t st);

// ---------------------------------------------------------------------------
// Batched raster join: many queries over one resident point table in one
// launch.  Work items are blocks of rows of a "segment" (a row range that
// the same set of queries covers); a block of rows is staged in shared memory
// once and every query of its segment runs over it.
constexpr int kBatchMaxCols = 6;          // distinct scalar columns one batch may read
enum { BQ_LABEL = 0, BQ_SPLAT = 1, BQ_SKIP = 2, BQ_TLABEL = 3, BQ_TSPLAT = 4 };   // T: tiered canvas

struct BatchQuery {
    uint32_t lo[kBatchMaxCols];           // interval predicate per batch column:
    uint32_t span[kBatchMaxCols];         //   order_key(v) - lo <= span (lo 0, span ~0: none)
    int aggr_u;                           // batch column of the aggregate, -1: count only
    int aggr_typ;
    float sum_scale;                      // fixed-point scale 2^(s-32)
    int mode;                             // BQ_*
    int P;
    int hist_smem;                        // per-block shared-memory histogram (P <= capacity)
    CanvasXf cx;
    const uint16_t* label;                // BQ_LABEL: [T][resy][resx]
    uint32_t* canvas_c;                   // BQ_SPLAT: [T][resy][resx]
    long long* canvas_s;
    unsigned long long* out_count;        // [P]
    unsigned long long* out_sum;          // [P] fixed-point
    double* out_nonfinite;                // [P]
    uint32_t* out_count32;                // private splat: counts flushed into the u32 canvas
    float4 box;                           // locations that can reach the canvas (x0, y0, x1, y1)
    const float4* zones;                  // zone map (bounds per 2^kZoneShift rows), or null: no skip
    TierArgs tr;                          // BQ_TLABEL / BQ_TSPLAT
};

struct BatchSeg {
    uint64_t r0, r1;                      // rows
    uint64_t item0;                       // first work item of the segment
    int qbegin, qend;                     // queries: qlist[qbegin .. qend)
};

struct BatchArgs {
    const float2* xy;
    int nu;                               // batch columns
    const uint32_t* ucol[kBatchMaxCols];
    int utyp[kBatchMaxCols];
    const BatchQuery* q;
    const int* qlist;
    const BatchSeg* seg;
    int nseg;
    uint64_t nitems;
    unsigned long long* work;             // work-item counter (zeroed before the launch)
    int rows;                             // rows per work item
    int hist_cap;                         // shared-memory histogram entries
};

// block shape of the batched kernel (picked by the tuner)
struct BatchShape {
    int threads;                          // 256 or 512
    int rows;                             // rows per work item
    int direct;                           // 0: rows staged in shared memory; 1: streamed per query (L2 reuse)
};
size_t batch_smem_bytes(const BatchShape& s, int nu, int hist_cap);
int batch_blocks_per_sm(const BatchShape& s, int nu, int hist_cap);
bool launch_batch_points(const BatchArgs& a, const BatchShape& s, int sms, cudaStream_t st);

// time index of the resident table
void launch_time_minmax(const uint32_t* t, uint64_t n, unsigned* out_min, unsigned* out_max, int sms, cudaStream_t st);
struct PermuteCols {
    int ncol;
    const void* src[RJ_MAX_ATTRIBUTES];
    void* dst[RJ_MAX_ATTRIBUTES];
    int esz[RJ_MAX_ATTRIBUTES];           // 4 or 8 bytes
};
struct ClusterKey {
    const uint32_t* t;                    // time column, or null (spatial order only)
    uint32_t tmin, tmax;
    int nbt;                              // time buckets
    const float2* xy;
    float x0, y0, sx, sy;                 // cell = (v - v0) * s, clamped to [0, 2^cb)
    int cb;                               // cell bits per axis (0: time order only)
};
void launch_xy_bounds(const float2* xy, uint64_t n, unsigned* out, int sms, cudaStream_t st);
void launch_cluster_hist(const ClusterKey& k, uint64_t n, unsigned* hist, int sms, cudaStream_t st);
void launch_cluster_scatter(const ClusterKey& k, uint64_t n, unsigned long long* cursor, const PermuteCols& pc, int sms,
                            cudaStream_t st);
void launch_time_unsorted(const uint32_t* t, uint64_t n, uint32_t tmin, uint32_t tmax, int nb, unsigned long long* count,
                          int sms, cudaStream_t st);

}  // namespace rj
