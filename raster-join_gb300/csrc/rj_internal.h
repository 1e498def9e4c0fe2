// rj_internal.h -- host-side state shared by the runtime translation units:
// the context behind rj_ctx, polygon sets, and the helpers that plan a query
// (canvas geometry, filters, device allocation).
#pragma once
#include <atomic>
#include <cmath>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "rj_device.cuh"
#include "rj_launch.h"

namespace rjh {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct Column {
    int attrib = -1;
    int type = RJ_FLOAT;
    void* d = nullptr;           // device data, or host data of a streamed table
    bool owned = false;
    float absmax = 0.f;     // largest finite |aggregate value| (sizes the fixed-point sums)
};

// Derived structures of the bound polygon set, rebuilt on demand.
struct GridCache {
    bool valid = false;
    int res = 0;
    int clamp = 0;
    bool pair_cell = false;
    size_t nentries = 0;
};

struct ExactCache {
    bool valid = false;
    int res = 0;
    int user_res = 0;
    size_t nentries = 0, nedges = 0;
};

// One polygon collection (PolyHandler polys / pindexes / bounds,
// RasterJoin/db/PolyHandler.cpp:49-80) with its device copy.
struct PolySet {
    int P = 0, V = 0;
    std::vector<float> h_xy;
    std::vector<int> h_pindex;
    std::vector<float4> h_mbr;      // per polygon (minx, miny, maxx, maxy)
    double bbox[4] = {0, 0, 0, 0};
    float max_abs_coord = 0.f, max_edge_dx = 0.f, max_edge_dy = 0.f;
    double sum_dx = 0, sum_dy = 0;  // sums of |dx|, |dy| over all edges
    // one device allocation (d_block) holds the vertices, pindex and the
    // edge -> polygon map; d_verts, d_pindex and d_edge_poly point into it
    DevBuf d_block;
    DevBuf d_verts, d_pindex, d_edge_poly;
    uint64_t version = 0;
    // Whether two polygons share a pixel centre, per canvas geometry (a set
    // whose coverage is disjoint on one canvas can overlap on a finer one):
    // absent = unknown, 0 = disjoint, 1 = overlapping.
    std::map<uint64_t, int> overlap;
    int overlap_on(uint64_t canvas) const {
        auto it = overlap.find(canvas);
        return it == overlap.end() ? -1 : it->second;
    }
    GridCache grid;
    ExactCache exact;
};

// Time-bucketed row order of the resident table (rj_build_time_index): rows
// of bucket b are [start[b], start[b+1]); bucket of t is
// (t - tmin) * nb / (tmax - tmin + 1).
struct TimeIndex {
    bool valid = false;
    int attrib = -1;
    uint32_t tmin = 0, tmax = 0;
    int nb = 0;
    std::vector<uint64_t> start;   // nb + 1
    uint32_t bucket_of(uint32_t t) const {
        if (t <= tmin) return 0;
        if (t >= tmax) return (uint32_t)nb - 1;
        return (uint32_t)(((uint64_t)(t - tmin) * (uint64_t)nb) / ((uint64_t)(tmax - tmin) + 1));
    }
    // rows that can hold a time in [t0, t1] (a superset, multiple of 4 aligned)
    void rows(uint32_t t0, uint32_t t1, uint64_t n, uint64_t& r0, uint64_t& r1) const {
        if (t1 < t0 || t1 < tmin || t0 > tmax) { r0 = r1 = 0; return; }
        r0 = start[bucket_of(t0)] & ~3ULL;
        r1 = start[bucket_of(t1) + 1];
        if (r1 > n) r1 = n;
    }
};

}  // namespace rjh

struct rj_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sms = 1;
    int64_t budget = 0;       // bytes, 0 = unlimited
    std::atomic<size_t> used{0};
    std::string err;
    std::recursive_mutex mu;  // serialises calls that share the context's scratch

    // point table (QueryResult columns)
    uint64_t npts = 0;
    int loc_attrib = -1;
    std::vector<rjh::Column> cols;
    rjh::TimeIndex tix;
    // streamed (host-resident) table: chunks of `chunk` rows copied per query
    bool streamed = false;
    uint64_t chunk = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copied[2]{}, consumed[2]{}, copy_t0{}, copy_t1{};
    rjh::DevBuf sbuf[2];
    rjh::DevBuf zones;               // zone map of the resident table (bounds per 1024 rows)
    bool zones_valid = false;
    float4 table_box{};              // bounds of the table's finite locations (with the zone map)
    float4 qbox{};                   // locations that can reach the current query's polygons
    int passes = 1;                  // point passes of the last query
    double copy_ms = 0;              // host->device copy time of the last query

    // polygon set bound for rj_execute: the context's own (rj_set_polygons)
    // or a caller's rj_polyset (rj_use_polyset)
    rjh::PolySet own;
    rjh::PolySet* ps = &own;
    const rjh::PolySet* cache_owner = nullptr;   // set whose grid / classified grid the scratch holds
    uint64_t cache_version = 0;

    std::map<std::string, rjh::DevBuf> scratch;
    // suffix of the scratch keys: queries issued on another stream (the
    // batched plain lanes) keep their buffers apart
    std::string scratch_ns;

    rj_timings tm{};
    cudaEvent_t ev[8]{};
    int* d_err = nullptr;     // device status word of bounded waits
    int sum_shift = 0;        // fixed-point scale 2^s of the current query's sums
    uint64_t row0 = 0, row1 = ~0ULL;   // rows of the current query (time index window)
    int server_running = 0;   // a serving loop owns the context
    // kernel tuning (rj_set_tuning): forced shapes, -1 = default / autotuned
    int point_shape = -1;
    int count_shape = -1, count_bshift = -1;
    int hybrid_exact_scale = 1;
    uint64_t wait_ns = rj::kWaitLimitNs;   // bound of the pipeline's device waits
    int last_count_shape = -1, last_count_bshift = -1;
    // exact partial sums of the last query (rj_get_sum_partials)
    int forced_shift = RJ_SUM_SHIFT_AUTO;
    std::vector<long long> last_fixed;
    std::vector<double> last_nonfinite;
    int last_shift = 0;
    void* batch_engine = nullptr;   // executor of rj_execute_batch
    // prepared queries (rj_prepare): the table's buffers change generation
    // whenever they are reallocated or reordered; while a query is captured
    // into a CUDA graph, steps that would read a value back to the host
    // refuse (RJ_E_UNSUPPORTED) and the zone map is left out
    uint64_t table_gen = 0;
    uint64_t tix_gen = 0;   // bumped when the time index stops matching the rows
    unsigned long long* edge_tests_dev = nullptr;   // this query's edge-test counter, or null
    bool capturing = false;
};

// A prepared query: the device work of one rj_execute captured as a CUDA
// graph, replayed by rj_execute_prepared.
struct rj_plan {
    rj_ctx* ctx = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t stream = nullptr;
    int P = 0;
    int function_type = 0;
    int shift = 0;
    int aggr_attrib = -1;
    uint64_t table_gen = 0, ps_version = 0;
    uint64_t tix_gen = 0;
    bool uses_tix = false;   // the captured row window came from the time index
    const void* ps = nullptr;
    uint64_t npts = 0;
    // pinned host copies of the per-polygon outputs, written by the graph
    unsigned long long* hc = nullptr;
    unsigned long long* hq = nullptr;
    double* hnf = nullptr;
    long long* hb = nullptr;
    int* derr = nullptr;
};

struct rj_polyset {
    rj_ctx* ctx = nullptr;
    rjh::PolySet s;
};

namespace rjh {

// raster canvases of at least this many pixels use the tiered form (16 x 16
// blocks, per-pixel data only where polygon edges pass)
constexpr size_t kTierMinPixels = (size_t)1 << 24;
// The tiered form also costs the point pass a little per point (a block code
// before the pixel); it pays when the canvas has more pixels than about twice
// the rows the query scans (measured on GB300: flat polygon side ~1.6 ps per
// pixel, tiered point lookups ~3.1 ps per point more while the flat canvas
// stays in L2).  Beyond kTierFlatMaxPixels a flat canvas no longer stays in
// L2 and every point's lookup goes to DRAM: 2B points on a 40000 x 40000
// canvas took 53.2 ms flat against 12.5 ms tiered (260 Voronoi cells; 2000
// overlapping stars: 97.7 against 44.2 ms).
constexpr size_t kTierFlatMaxPixels = (size_t)1 << 25;
inline bool use_tier(size_t npix, uint64_t rows) {
    return npix >= kTierMinPixels && (npix > 2 * rows || npix > kTierFlatMaxPixels);
}
// the form a raster query takes: flat or tiered canvas (RJ_FLAG_FLAT_CANVAS /
// RJ_FLAG_TIERED_CANVAS force one)
inline bool query_tier(uint32_t flags, size_t npix, uint64_t rows) {
    if (flags & RJ_FLAG_FLAT_CANVAS) return false;
    if (flags & RJ_FLAG_TIERED_CANVAS) return npix >= kTierMinPixels;
    return use_tier(npix, rows);
}

int fail(rj_ctx* c, int code, const char* fmt, ...);

#define RJ_CUDA(call)                                                                         \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return ::rjh::fail(ctx, RJ_E_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                               __FILE__, __LINE__);                                           \
    } while (0)

int dev_alloc(rj_ctx* ctx, DevBuf& b, size_t bytes);
void dev_free(rj_ctx* ctx, DevBuf& b);
const Column* find_col(const rj_ctx* ctx, int attrib);
double now_ms();

// Raster canvas plan: RasterJoin::updateBuffers (RasterJoin.cpp:51-78) and
// the per-tile MVP (RasterJoin.cpp:224-231, Utils.h:36-46).
struct RasterPlan {
    double cell = 0;
    int actual_x = 0, actual_y = 0;
    int splitx = 1, splity = 1;
    int resx = 1, resy = 1;
    std::vector<float4> colxf, rowxf;
};
int plan_raster_bbox(rj_ctx* ctx, const double* bbox, const rj_query* q, RasterPlan& rp);
// identity of a canvas geometry (tiles, resolution, per-tile transforms)
uint64_t canvas_key(const std::vector<float4>& colxf, const std::vector<float4>& rowxf, int resx, int resy);
int build_filter(rj_ctx* ctx, const rj_query* q, rj::DevFilter& f, bool force_count, bool* empty);
int load_polyset(rj_ctx* ctx, PolySet& s, const float* xy, const int32_t* pindex, int32_t npolys,
                 const double* bbox);
void free_polyset(rj_ctx* ctx, PolySet& s);
// rows [r0, r1) of the resident table a query can touch (all rows without a
// time index on its time attribute)
void decode_result(int P, const unsigned long long* hc, const unsigned long long* hq, const double* hnf, int shift,
                   const long long* hb, rj_result* res);
void free_batch_engine(rj_ctx* ctx);
// One query's device work queued on ctx->stream (the readbacks some forms
// need aside, no host synchronisation) with the context's scratch and error
// word; the per-polygon outputs stay on the device for the caller to copy.
// ctx->sum_shift holds the query's fixed-point shift on return.
int enqueue_query_untimed(rj_ctx* ctx, const rj_query* q, unsigned long long** oc, unsigned long long** os,
                          double** onf, long long** ob);
void query_rows(const rj_ctx* ctx, const rj_query* q, uint64_t& r0, uint64_t& r1);
int ensure_zones(rj_ctx* ctx);

}  // namespace rjh
