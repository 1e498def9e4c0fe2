// rj_batch.cu -- polygon-set handles, the time index of the resident table,
// the batched raster join and the serving loop (C ABI in include/rj.h).
//
// A batch runs in an Engine: a stream, a device arena and pinned staging.
//   1. host planning per query: canvas plan (RasterJoin::updateBuffers,
//      RasterJoin.cpp:51-78), filters in interval form, the rows the query's
//      time window covers, arena placement of its outputs and canvas;
//   2. polygon side per query: the polygon label map of its canvas, or a
//      zeroed point canvas when two of its polygons share pixel centres;
//   3. one fused point pass for all queries (k_batch_points);
//   4. per canvas-path query, the polygon pass that reduces its canvas;
//   5. one copy of every query's per-polygon outputs back to the host.
// The serving loop runs one Engine per slot on its own thread; a slot takes
// every queued request that fits its arena when it becomes free, so batches
// grow with the arrival rate and slots overlap on the device.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <thread>
#include <unordered_map>

#include "rj_device.cuh"
#include "rj_internal.h"
#include "rj_launch.h"

using namespace rj;
using namespace rjh;

namespace {

struct Arena {
    DevBuf buf;
    size_t off = 0;
    void reset() { off = 0; }
    template <class T>
    T* take(size_t n) {
        const size_t b = (std::max<size_t>(n, 1) * sizeof(T) + 255) & ~size_t(255);
        if (off + b > buf.bytes) return nullptr;
        T* p = (T*)((char*)buf.p + off);
        off += b;
        return p;
    }
};

size_t al256(size_t b) { return (std::max<size_t>(b, 1) + 255) & ~size_t(255); }

// per-block shared histogram entries of the fused point pass (polygons of a
// label-map query, or pixels of a small splat canvas)
constexpr int kBatchHistCap = 4096;

// Streams of the queries that leave the fused pass: each lane has its own
// scratch (keys suffixed with the lane) and error word, so that the device
// work of several such queries -- and of the fused pass on the engine's own
// stream -- overlaps on the GPU.
constexpr int kLanes = 8;   // at most; rj_execute_batch's engine uses 8, a serving slot 4

struct Engine {
    rj_ctx* ctx = nullptr;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    Arena ar;
    size_t cap = 0;              // arena bytes (0: grow on demand)
    cudaEvent_t ev[6]{};
    void* h_pin = nullptr;
    size_t h_pin_bytes = 0;
    BatchShape shape{256, 16384, 1};
    bool tuned = false;
    bool lanes = false;          // may queue queries on the lanes
    int nlanes = kLanes;         // lanes in use (a serving slot takes fewer: its
                                 // requests are small, and each lane's scratch is
                                 // allocated on first use, mid-serving)
    int id = 0;                  // names the lanes' scratch apart from other engines'
    cudaStream_t lane_st[kLanes]{};
    int* lane_err = nullptr;     // device: one error word per lane
    cudaEvent_t lane_ev = nullptr;
    void* lane_pin = nullptr;    // pinned staging of the lanes' outputs
    size_t lane_pin_bytes = 0;
};

std::atomic<int> g_engine_ids{0};

int engine_init(rj_ctx* ctx, Engine& e, cudaStream_t st, size_t cap) {
    e.ctx = ctx;
    e.cap = cap;
    e.id = g_engine_ids.fetch_add(1);
    if (st) {
        e.st = st;
    } else {
        if (cudaStreamCreateWithFlags(&e.st, cudaStreamNonBlocking) != cudaSuccess) return RJ_E_CUDA;
        e.own_stream = true;
    }
    for (auto& v : e.ev)
        if (cudaEventCreate(&v) != cudaSuccess) return RJ_E_CUDA;
    return RJ_OK;
}

void engine_free(Engine& e) {
    if (e.st) cudaStreamSynchronize(e.st);
    for (auto& s : e.lane_st) {
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
        s = nullptr;
    }
    if (e.lane_err) cudaFree(e.lane_err);
    e.lane_err = nullptr;
    if (e.lane_ev) cudaEventDestroy(e.lane_ev);
    e.lane_ev = nullptr;
    if (e.lane_pin) cudaFreeHost(e.lane_pin);
    e.lane_pin = nullptr;
    if (e.ar.buf.p) dev_free(e.ctx, e.ar.buf);
    if (e.h_pin) cudaFreeHost(e.h_pin);
    e.h_pin = nullptr;
    for (auto& v : e.ev)
        if (v) cudaEventDestroy(v);
    if (e.own_stream && e.st) cudaStreamDestroy(e.st);
    e.st = nullptr;
}

void* engine_pinned(Engine& e, size_t bytes) {
    if (e.h_pin_bytes >= bytes) return e.h_pin;
    if (e.h_pin) cudaFreeHost(e.h_pin);
    e.h_pin = nullptr;
    e.h_pin_bytes = 0;
    if (cudaMallocHost(&e.h_pin, bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    e.h_pin_bytes = bytes;
    return e.h_pin;
}

// Per-query plan of one batch.
struct QPlan {
    int idx = 0;                 // position in the caller's arrays
    const rj_query* q = nullptr;
    PolySet* ps = nullptr;
    rj_polyset* set = nullptr;
    rj_result* res = nullptr;
    int status = RJ_OK;
    bool fused = false;
    RasterPlan rp;
    DevFilter f{};
    int shift = 0;
    uint64_t r0 = 0, r1 = 0;
    int mode = BQ_SKIP;
    int T = 1;
    size_t npix = 0;
    bool check_overlap = false;
    uint64_t canvas = 0;         // canvas geometry (overlap status is per canvas)
    bool tier = false;           // tiered canvas (16 x 16 blocks)
    TierArgs tr{};
    size_t nblk = 0;             // blocks of the tiered canvas
    size_t est_slots = 0;        // upper bound on its mixed blocks
    int nslots = 0;
    int* slot_buf = nullptr;
    int* scan_tmp = nullptr;
    size_t out_off = 0;          // first polygon of the query in the output block
    uint16_t* label = nullptr;
    uint32_t* cc = nullptr;
    long long* cs = nullptr;
    float4* dcol = nullptr;
    float4* drow = nullptr;
};

// bytes of a tiered canvas's canvas form (block sums + slot pixels)
size_t tier_canvas_bytes(const QPlan& p) {
    const bool agg = p.f.aggr != 0;
    return al256(p.nblk * 4) + (agg ? al256(p.nblk * 8) : 0) + al256(p.est_slots * 256 * 4) +
           (agg ? al256(p.est_slots * 256 * 8) : 0);
}

size_t canvas_bytes(const QPlan& p) {
    const bool agg = p.f.aggr != 0;
    if (p.tier) {
        const size_t base = 4 * al256(p.nblk * 4) + al256((p.nblk + 1) * 4) +
                            al256((size_t)scan_tmp_ints((int)std::max<size_t>(p.nblk, 1)) * 4);
        return base + (p.mode == BQ_TLABEL ? al256(p.est_slots * 256 * 2) : tier_canvas_bytes(p));
    }
    return p.mode == BQ_LABEL ? al256(p.npix * 2) : al256(p.npix * 4) + (agg ? al256(p.npix * 8) : 0);
}

// Host planning of one query (under the context lock: filters and canvas
// plans report errors through the context).
// Single-tile queries over at least this many rows run faster through the
// lean single-query passes (label map: block codes in shared memory, plain
// shared atomics; point canvas: canvas copies in shared memory or plain
// atomics) than in the fused pass, whose shared row reads save little: the
// per-(point, query) work dominates, not the row read.  They leave the fused
// pass.
constexpr uint64_t kLeanQueryRows = 1ull << 22;

void plan_query(rj_ctx* ctx, QPlan& p, bool no_fuse, bool fuse_all) {
    const rj_query* q = p.q;
    if (no_fuse || q->function_type != RJ_RASTER_JOIN || ctx->streamed) return;   // plain path
    int rc = plan_raster_bbox(ctx, p.ps->bbox, q, p.rp);
    if (rc) { p.status = rc; return; }
    bool empty = false;
    rc = build_filter(ctx, q, p.f, false, &empty);
    if (rc) { p.status = rc; return; }
    p.shift = p.f.aggr ? ctx->sum_shift : 0;
    if (p.f.general && !empty) return;                             // per-predicate filters: plain path
    p.T = p.rp.splitx * p.rp.splity;
    p.npix = (size_t)p.rp.resx * p.rp.resy * p.T;
    query_rows(ctx, q, p.r0, p.r1);
    // row ranges on multiples of four rows (aligned 128-bit loads in the fused
    // pass); the rows added are outside the time window and fail its predicate
    p.r0 &= ~3ULL;
    p.r1 = std::min<uint64_t>(ctx->npts, (p.r1 + 3) & ~3ULL);
    // large canvases: tiered form (per-block work instead of per-pixel work)
    p.tier = query_tier(q->flags, p.npix, p.r1 - p.r0);
    if (p.tier) {
        p.tr.bw = (p.rp.resx + 15) / 16;
        p.tr.bh = (p.rp.resy + 15) / 16;
        p.nblk = (size_t)p.T * p.tr.bw * p.tr.bh;
        if (p.nblk >= (size_t)1 << 24) return;                     // single-query path
        // mixed blocks lie on the edges (or the canvas border): blocks an edge
        // passes are at most |dx| / 16 px + |dy| / 16 px + 3
        const double pw = (p.ps->bbox[2] - p.ps->bbox[0]) / p.rp.splitx / p.rp.resx;
        const double ph = (p.ps->bbox[3] - p.ps->bbox[1]) / p.rp.splity / p.rp.resy;
        const double est = p.ps->sum_dx / (16.0 * pw) + p.ps->sum_dy / (16.0 * ph) + 3.0 * p.ps->V * p.T +
                           2.0 * p.T * (p.tr.bw + p.tr.bh) + 64.0;
        p.est_slots = (size_t)std::min<double>(est, (double)p.nblk);
    }
    p.fused = true;
    if (empty || p.r1 <= p.r0) {
        p.mode = BQ_SKIP;
        return;
    }
    const bool label_ok = !(q->flags & RJ_FLAG_FORCE_CANVAS) && p.ps->P <= kMaxLabelPolys;
    p.canvas = canvas_key(p.rp.colxf, p.rp.rowxf, p.rp.resx, p.rp.resy);
    const int known = p.ps->overlap_on(p.canvas);
    if (p.tier) {
        p.mode = (label_ok && known != 1) ? BQ_TLABEL : BQ_TSPLAT;
        p.check_overlap = p.mode == BQ_TLABEL && known != 0;
    } else {
        p.mode = (label_ok && known != 1) ? BQ_LABEL : BQ_SPLAT;
        p.check_overlap = p.mode == BQ_LABEL && known != 0;
        if (!fuse_all && (p.mode == BQ_LABEL || p.mode == BQ_SPLAT) && p.T == 1 && !p.f.general &&
            p.f.ncol <= label_lean_max_cols() && p.r1 - p.r0 >= kLeanQueryRows)
            p.fused = false;   // rj_execute's lean pass (same results)
    }
}

struct PolyScratch {
    int2* wv = nullptr;
    int4* info_a = nullptr;
    int2* info_b = nullptr;
    int* nbands = nullptr;
    int* band_start = nullptr;
    int* tmp = nullptr;
    unsigned* ctr = nullptr;
};

size_t poly_scratch_bytes(size_t TV, size_t TP) {
    return al256(TV * sizeof(int2)) + al256(TP * sizeof(int4)) + al256(TP * sizeof(int2)) + al256(TP * 4) +
           al256((TP + 1) * 4) + al256((size_t)scan_tmp_ints((int)std::max<size_t>(TP, 1)) * 4) + al256(4);
}

bool poly_scratch_take(Arena& ar, size_t TV, size_t TP, PolyScratch& s) {
    s.wv = ar.take<int2>(TV);
    s.info_a = ar.take<int4>(TP);
    s.info_b = ar.take<int2>(TP);
    s.nbands = ar.take<int>(TP);
    s.band_start = ar.take<int>(TP + 1);
    s.tmp = ar.take<int>((size_t)scan_tmp_ints((int)std::max<size_t>(TP, 1)));
    s.ctr = ar.take<unsigned>(1);
    return s.wv && s.info_a && s.info_b && s.nbands && s.band_start && s.tmp && s.ctr;
}

// Polygon pass of one query's canvas (label map or reduction).
bool query_poly_pass(Engine& e, const QPlan& p, int mode, PolyScratch& s, unsigned long long* oc,
                     unsigned long long* os, unsigned long long* covered, const TierArgs* tier = nullptr) {
    rj_ctx* ctx = e.ctx;
    const PolySet& ps = *p.ps;
    launch_transform_vertices((const float2*)ps.d_verts.p, ps.V, p.dcol, p.drow, p.rp.splitx, p.T, s.wv, nullptr,
                              ctx->sms, e.st);
    PolyPassArgs a{};
    a.wv = s.wv;
    a.pindex = (const int*)ps.d_pindex.p;
    a.P = ps.P;
    a.V = ps.V;
    a.T = p.T;
    a.resx = p.rp.resx;
    a.resy = p.rp.resy;
    a.canvas_c = tier ? nullptr : p.cc;
    a.canvas_s = tier ? nullptr : p.cs;
    a.label = mode == MODE_LABEL ? p.label : nullptr;
    a.covered = covered;
    a.out_count = oc;
    a.out_sum = os;
    a.work_ctr = s.ctr;
    a.info_a = s.info_a;
    a.info_b = s.info_b;
    a.nbands = s.nbands;
    a.band_start = s.band_start;
    cudaMemsetAsync(s.ctr, 0, sizeof(unsigned), e.st);
    launch_poly_info(mode, a, ctx->sms, e.st);
    if (!launch_exclusive_scan(s.nbands, s.band_start, a.T * a.P, s.tmp, e.st)) return false;
    if (tier) launch_tier_pass(mode, a, *tier, ctx->sms, e.st);
    else launch_poly_pass(mode, a, ctx->sms, e.st);
    return true;
}

// Rows covered by the same queries: segments + their query lists.
void build_segments(const std::vector<QPlan*>& act, std::vector<BatchSeg>& segs, std::vector<int>& qlist, int rows,
                    uint64_t& nitems, uint64_t& rows_read, uint64_t& point_queries) {
    std::vector<uint64_t> E;
    E.reserve(act.size() * 2);
    for (const QPlan* p : act) {
        E.push_back(p->r0);
        E.push_back(p->r1);
    }
    std::sort(E.begin(), E.end());
    E.erase(std::unique(E.begin(), E.end()), E.end());
    struct S { uint64_t a, b; std::vector<int> qs; };
    std::vector<S> tmp;
    for (size_t k = 0; k + 1 < E.size(); ++k) {
        S s{E[k], E[k + 1], {}};
        for (size_t i = 0; i < act.size(); ++i)
            if (act[i]->r0 <= s.a && act[i]->r1 >= s.b) s.qs.push_back((int)i);
        if (!s.qs.empty()) tmp.push_back(std::move(s));
    }
    // segments with the most queries first (their items cost the most)
    std::stable_sort(tmp.begin(), tmp.end(), [](const S& x, const S& y) { return x.qs.size() > y.qs.size(); });
    segs.clear();
    qlist.clear();
    nitems = 0;
    rows_read = 0;
    point_queries = 0;
    for (const S& s : tmp) {
        BatchSeg g{};
        g.r0 = s.a;
        g.r1 = s.b;
        g.item0 = nitems;
        g.qbegin = (int)qlist.size();
        qlist.insert(qlist.end(), s.qs.begin(), s.qs.end());
        g.qend = (int)qlist.size();
        nitems += (s.b - s.a + rows - 1) / rows;
        rows_read += s.b - s.a;
        point_queries += (s.b - s.a) * s.qs.size();
        segs.push_back(g);
    }
}

struct BatchOut {
    int fused = 0, fallback = 0, segments = 0, tuned = 0;
    uint64_t items = 0, rows_read = 0, point_queries = 0;
    double poly_ms = 0, point_ms = 0, reduce_ms = 0;
};

float ev_ms(cudaEvent_t a, cudaEvent_t b) {
    float v = 0.f;
    if (cudaEventElapsedTime(&v, a, b) != cudaSuccess) {
        cudaGetLastError();
        return 0.f;
    }
    return v;
}

// Runs the fused queries of `plans` (fused == true, status OK) in waves that
// fit the engine's arena; queries that do not fit even alone fall back.
int run_fused(Engine& e, std::vector<QPlan>& plans, uint32_t flags, BatchOut& bo) {
    rj_ctx* ctx = e.ctx;
    std::vector<QPlan*> todo;
    for (QPlan& p : plans)
        if (p.fused && p.status == RJ_OK) todo.push_back(&p);
    size_t next = 0;
    while (next < todo.size()) {
        // ---- admission: a prefix of the remaining queries that fits the arena
        std::vector<QPlan*> wave;
        size_t need = 0, maxTV = 0, maxTP = 0, outs = 0, xfs = 0;
        size_t avail = e.cap;
        if (avail == 0) {
            size_t fr = 0, tot = 0;
            cudaMemGetInfo(&fr, &tot);
            avail = (size_t)(0.5 * (double)(fr + e.ar.buf.bytes));
            if (ctx->budget > 0) avail = std::min<size_t>(avail, (size_t)std::max<int64_t>(ctx->budget - (int64_t)ctx->used + (int64_t)e.ar.buf.bytes, 0));
        }
        for (; next < todo.size(); ++next) {
            QPlan* p = todo[next];
            const size_t TV = (size_t)p->T * p->ps->V, TP = (size_t)p->T * p->ps->P;
            const size_t nmaxTV = std::max(maxTV, TV), nmaxTP = std::max(maxTP, TP);
            const size_t nouts = outs + p->ps->P, nxfs = xfs + p->rp.splitx + p->rp.splity;
            size_t cb = p->mode == BQ_SKIP ? 0 : canvas_bytes(*p);
            // a label query may need a canvas after the overlap check: reserve it
            if (p->check_overlap)
                cb += p->tier ? tier_canvas_bytes(*p) : al256(p->npix * 4) + (p->f.aggr ? al256(p->npix * 8) : 0);
            const size_t fixed = poly_scratch_bytes(nmaxTV, nmaxTP) + 3 * al256(nouts * 8) + al256(nxfs * 16) +
                                 al256((wave.size() + 1) * 16) + al256((wave.size() + 1) * sizeof(BatchQuery)) +
                                 al256((wave.size() + 1) * 2 * 2 * sizeof(BatchSeg)) +
                                 al256((wave.size() + 1) * (wave.size() + 1) * 2 * 4) + 4096;
            if (!wave.empty() && fixed + need + cb > avail) break;
            if (wave.empty() && fixed + cb > avail) {
                p->fused = false;   // too large for one pass: the plain path tiles it
                continue;
            }
            wave.push_back(p);
            need += cb;
            maxTV = nmaxTV;
            maxTP = nmaxTP;
            outs = nouts;
            xfs = nxfs;
        }
        if (wave.empty()) break;
        const size_t nw = wave.size();
        const size_t total = poly_scratch_bytes(maxTV, maxTP) + 3 * al256(outs * 8) + al256(xfs * 16) + al256(nw * 16) +
                             al256(nw * 24) +
                             al256(nw * sizeof(BatchQuery)) + al256(nw * 2 * 2 * sizeof(BatchSeg)) +
                             al256(nw * nw * 2 * 4 + 4) + need + 4096;
        if (e.ar.buf.bytes < total) {
            int rc = dev_alloc(ctx, e.ar.buf, e.cap ? std::max(e.cap, total) : total);
            if (rc) return rc;
        }
        e.ar.reset();
        Arena& ar = e.ar;
        PolyScratch ps{};
        if (!poly_scratch_take(ar, maxTV, maxTP, ps)) return fail(ctx, RJ_E_OOM, "batch arena too small");
        unsigned long long* oc = ar.take<unsigned long long>(outs);
        unsigned long long* os = ar.take<unsigned long long>(outs);
        double* onf = ar.take<double>(outs);
        float4* xf = ar.take<float4>(xfs);
        unsigned long long* lcnt = ar.take<unsigned long long>(2 * nw);
        unsigned long long* tcnt = ar.take<unsigned long long>(3 * nw);   // tiered: multi, covered, labelled
        BatchQuery* dq = ar.take<BatchQuery>(nw);
        unsigned long long* work = ar.take<unsigned long long>(1);
        if (!oc || !os || !onf || !xf || !lcnt || !tcnt || !dq || !work) return fail(ctx, RJ_E_OOM, "batch arena too small");
        // placements + transforms
        std::vector<float4> hxf;
        hxf.reserve(xfs);
        size_t o = 0;
        for (QPlan* p : wave) {
            p->out_off = o;
            o += p->ps->P;
            p->dcol = xf + hxf.size();
            hxf.insert(hxf.end(), p->rp.colxf.begin(), p->rp.colxf.end());
            p->drow = xf + hxf.size();
            hxf.insert(hxf.end(), p->rp.rowxf.begin(), p->rp.rowxf.end());
            p->label = nullptr;
            p->cc = nullptr;
            p->cs = nullptr;
            if (p->tier && p->mode != BQ_SKIP) {
                TierArgs& tr = p->tr;
                tr.full = ar.take<uint32_t>(p->nblk);
                tr.mixed = ar.take<uint32_t>(p->nblk);
                p->slot_buf = ar.take<int>(p->nblk + 1);
                tr.slot = p->slot_buf;
                tr.code = ar.take<uint32_t>(p->nblk);
                p->scan_tmp = ar.take<int>((size_t)scan_tmp_ints((int)std::max<size_t>(p->nblk, 1)));
                tr.plabel = nullptr;
                tr.bcnt = tr.pcnt = nullptr;
                tr.bsum = tr.psum = nullptr;
                if (p->mode == BQ_TLABEL) {
                    tr.plabel = ar.take<uint16_t>(p->est_slots * 256);
                } else {
                    tr.bcnt = ar.take<uint32_t>(p->nblk);
                    tr.pcnt = ar.take<uint32_t>(p->est_slots * 256);
                    if (p->f.aggr) {
                        tr.bsum = ar.take<long long>(p->nblk);
                        tr.psum = ar.take<long long>(p->est_slots * 256);
                    }
                }
                if (!tr.full || !tr.mixed || !p->slot_buf || !tr.code || !p->scan_tmp ||
                    (p->mode == BQ_TLABEL ? !tr.plabel : (!tr.bcnt || !tr.pcnt || (p->f.aggr && (!tr.bsum || !tr.psum)))))
                    return fail(ctx, RJ_E_OOM, "batch arena too small for a tiered canvas");
            } else if (p->mode == BQ_LABEL) {
                p->label = ar.take<uint16_t>(p->npix);
            } else if (p->mode == BQ_SPLAT) {
                p->cc = ar.take<uint32_t>(p->npix);
                if (p->f.aggr) p->cs = ar.take<long long>(p->npix);
            }
        }
        cudaStream_t st = e.st;
        cudaEventRecord(e.ev[0], st);
        RJ_CUDA(cudaMemcpyAsync(xf, hxf.data(), hxf.size() * sizeof(float4), cudaMemcpyHostToDevice, st));
        RJ_CUDA(cudaMemsetAsync(oc, 0, outs * 8, st));
        RJ_CUDA(cudaMemsetAsync(os, 0, outs * 8, st));
        RJ_CUDA(cudaMemsetAsync(onf, 0, outs * 8, st));
        RJ_CUDA(cudaMemsetAsync(lcnt, 0, 2 * nw * 8, st));
        RJ_CUDA(cudaMemsetAsync(tcnt, 0, 3 * nw * 8, st));
        // ---- tiered canvases: block classification, slots of the mixed blocks
        bool any_tier = false;
        for (size_t i = 0; i < nw; ++i) {
            QPlan* p = wave[i];
            if (!p->tier || p->mode == BQ_SKIP) continue;
            any_tier = true;
            RJ_CUDA(cudaMemsetAsync(p->tr.full, 0xFF, p->nblk * 4, st));
            RJ_CUDA(cudaMemsetAsync(p->tr.mixed, 0, p->nblk * 4, st));
            if (!query_poly_pass(e, *p, MODE_TIER_CLASSIFY, ps, nullptr, nullptr, nullptr, &p->tr))
                return fail(ctx, RJ_E_INVALID, "too many (tile, polygon) items");
            if (!launch_exclusive_scan((const int*)p->tr.mixed, p->slot_buf, (int)p->nblk, p->scan_tmp, st))
                return fail(ctx, RJ_E_INVALID, "tier scan failed");
            launch_tier_codes(p->tr, p->nblk, tcnt + 3 * i, ctx->sms, st);
            RJ_CUDA(cudaMemcpyAsync(&p->nslots, p->slot_buf + p->nblk, sizeof(int), cudaMemcpyDeviceToHost, st));
        }
        if (any_tier) {
            RJ_CUDA(cudaStreamSynchronize(st));
            for (size_t i = 0; i < nw; ++i) {
                QPlan* p = wave[i];
                if (!p->tier || p->mode == BQ_SKIP) continue;
                if ((size_t)p->nslots > p->est_slots)
                    return fail(ctx, RJ_E_INVALID, "tiered canvas: %d mixed blocks above the bound %zu", p->nslots,
                                p->est_slots);
                const size_t spx = (size_t)p->nslots * 256;
                if (p->mode == BQ_TLABEL) {
                    RJ_CUDA(cudaMemsetAsync(p->tr.plabel, 0xFF, std::max<size_t>(spx, 1) * 2, st));
                    if (!query_poly_pass(e, *p, MODE_TIER_LABEL, ps, nullptr, nullptr, tcnt + 3 * i + 1, &p->tr))
                        return fail(ctx, RJ_E_INVALID, "too many (tile, polygon) items");
                    if (p->check_overlap) launch_tier_nonempty(p->tr.plabel, spx, tcnt + 3 * i + 2, ctx->sms, st);
                } else {
                    RJ_CUDA(cudaMemsetAsync(p->tr.bcnt, 0, p->nblk * 4, st));
                    RJ_CUDA(cudaMemsetAsync(p->tr.pcnt, 0, std::max<size_t>(spx, 1) * 4, st));
                    if (p->tr.bsum) RJ_CUDA(cudaMemsetAsync(p->tr.bsum, 0, p->nblk * 8, st));
                    if (p->tr.psum) RJ_CUDA(cudaMemsetAsync(p->tr.psum, 0, std::max<size_t>(spx, 1) * 8, st));
                }
            }
        }
        // ---- polygon side: label maps / zeroed canvases
        bool any_check = false;
        for (size_t i = 0; i < nw; ++i) {
            QPlan* p = wave[i];
            if (p->mode == BQ_LABEL) {
                RJ_CUDA(cudaMemsetAsync(p->label, 0xFF, p->npix * 2, st));
                if (!query_poly_pass(e, *p, MODE_LABEL, ps, nullptr, nullptr, lcnt + 2 * i))
                    return fail(ctx, RJ_E_INVALID, "too many (tile, polygon) items");
                launch_label_finish(p->label, nullptr, p->rp.resx, p->rp.resy, p->T, 0, lcnt + 2 * i + 1, ctx->sms, st);
                any_check |= p->check_overlap;
            } else if (p->mode == BQ_SPLAT) {
                RJ_CUDA(cudaMemsetAsync(p->cc, 0, p->npix * 4, st));
                if (p->cs) RJ_CUDA(cudaMemsetAsync(p->cs, 0, p->npix * 8, st));
            }
        }
        RJ_CUDA(cudaGetLastError());
        for (QPlan* p : wave) any_check |= p->tier && p->check_overlap;
        if (any_check) {
            // which label maps hold every covered pixel centre exactly once
            std::vector<unsigned long long> hl(2 * nw), ht(3 * nw);
            RJ_CUDA(cudaMemcpyAsync(hl.data(), lcnt, 2 * nw * 8, cudaMemcpyDeviceToHost, st));
            RJ_CUDA(cudaMemcpyAsync(ht.data(), tcnt, 3 * nw * 8, cudaMemcpyDeviceToHost, st));
            RJ_CUDA(cudaStreamSynchronize(st));
            for (size_t i = 0; i < nw; ++i) {
                QPlan* p = wave[i];
                if (!p->check_overlap) continue;
                const bool overlap = p->tier ? (ht[3 * i] != 0 || ht[3 * i + 1] != ht[3 * i + 2])
                                             : hl[2 * i] != hl[2 * i + 1];
                if (p->tier) {
                    {
                        std::lock_guard<std::recursive_mutex> lock(ctx->mu);
                        p->ps->overlap[p->canvas] = overlap ? 1 : 0;
                    }
                    if (!overlap) continue;
                    p->mode = BQ_TSPLAT;
                    TierArgs& tr = p->tr;
                    const size_t spx = (size_t)std::max(p->nslots, 1) * 256;
                    tr.bcnt = ar.take<uint32_t>(p->nblk);
                    tr.pcnt = ar.take<uint32_t>(spx);
                    if (p->f.aggr) {
                        tr.bsum = ar.take<long long>(p->nblk);
                        tr.psum = ar.take<long long>(spx);
                    }
                    if (!tr.bcnt || !tr.pcnt || (p->f.aggr && (!tr.bsum || !tr.psum)))
                        return fail(ctx, RJ_E_OOM, "batch arena too small for a tiered canvas");
                    RJ_CUDA(cudaMemsetAsync(tr.bcnt, 0, p->nblk * 4, st));
                    RJ_CUDA(cudaMemsetAsync(tr.pcnt, 0, spx * 4, st));
                    if (tr.bsum) RJ_CUDA(cudaMemsetAsync(tr.bsum, 0, p->nblk * 8, st));
                    if (tr.psum) RJ_CUDA(cudaMemsetAsync(tr.psum, 0, spx * 8, st));
                    continue;
                }
                {
                    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
                    p->ps->overlap[p->canvas] = overlap ? 1 : 0;
                }
                if (!overlap) continue;
                p->mode = BQ_SPLAT;
                p->cc = ar.take<uint32_t>(p->npix);
                if (p->f.aggr) p->cs = ar.take<long long>(p->npix);
                if (!p->cc || (p->f.aggr && !p->cs)) return fail(ctx, RJ_E_OOM, "batch arena too small for a canvas");
                RJ_CUDA(cudaMemsetAsync(p->cc, 0, p->npix * 4, st));
                if (p->cs) RJ_CUDA(cudaMemsetAsync(p->cs, 0, p->npix * 8, st));
            }
        }
        cudaEventRecord(e.ev[1], st);
        // ---- batch columns, query descriptors, segments
        BatchArgs ba{};
        ba.xy = (const float2*)find_col(ctx, ctx->loc_attrib)->d;
        std::vector<const uint32_t*> ucols;
        std::vector<int> utyps;
        auto slot_of = [&](const uint32_t* col, int typ) {
            for (size_t u = 0; u < ucols.size(); ++u)
                if (ucols[u] == col) return (int)u;
            ucols.push_back(col);
            utyps.push_back(typ);
            return (int)ucols.size() - 1;
        };
        std::vector<BatchQuery> hq(nw);
        std::vector<QPlan*> act;
        int max_hist = 0;
        for (size_t i = 0; i < nw; ++i) {
            QPlan* p = wave[i];
            BatchQuery& d = hq[i];
            std::memset(&d, 0, sizeof d);
            for (int u = 0; u < kBatchMaxCols; ++u) {
                d.lo[u] = 0u;
                d.span[u] = 0xFFFFFFFFu;
            }
            d.mode = p->mode;
            d.P = p->ps->P;
            d.aggr_u = -1;
            d.out_count = oc + p->out_off;
            d.out_sum = os + p->out_off;
            d.out_nonfinite = onf + p->out_off;
            if (p->mode == BQ_SKIP) continue;
            std::vector<std::pair<int, int>> slots;   // (slot, filter column)
            for (int c = 0; c < p->f.ncol; ++c) slots.push_back({slot_of(p->f.col[c], p->f.ctyp[c]), c});
            if (p->f.aggr) d.aggr_u = slot_of(p->f.aggr_col, p->f.aggr_typ);
            if ((int)ucols.size() > kBatchMaxCols) return fail(ctx, RJ_E_UNSUPPORTED, "batch reads too many columns");
            for (auto& sc : slots) {
                d.lo[sc.first] = p->f.lo[sc.second];
                d.span[sc.first] = p->f.span[sc.second];
            }
            d.aggr_typ = p->f.aggr_typ;
            d.sum_scale = p->f.sum_scale;
            CanvasXf& cx = d.cx;
            cx.colxf = p->dcol;
            cx.rowxf = p->drow;
            cx.splitx = p->rp.splitx;
            cx.splity = p->rp.splity;
            cx.resx = p->rp.resx;
            cx.resy = p->rp.resy;
            cx.lbx = (float)p->ps->bbox[0];
            cx.lby = (float)p->ps->bbox[1];
            cx.tdx = p->rp.colxf[0].w;
            cx.tdy = p->rp.rowxf[0].w;
            cx.col0 = p->rp.colxf[0];
            cx.row0 = p->rp.rowxf[0];
            d.label = p->label;
            d.canvas_c = p->cc;
            d.canvas_s = p->cs;
            d.tr = p->tr;
            {
                // canvas extent plus two pixels: a location outside it maps to
                // no pixel of any tile (window range test and snapping)
                const double mx = 2.0 * (p->ps->bbox[2] - p->ps->bbox[0]) / p->rp.actual_x + 1e-3;
                const double my = 2.0 * (p->ps->bbox[3] - p->ps->bbox[1]) / p->rp.actual_y + 1e-3;
                d.box = make_float4((float)(p->ps->bbox[0] - mx), (float)(p->ps->bbox[1] - my),
                                    (float)(p->ps->bbox[2] + mx), (float)(p->ps->bbox[3] + my));
                // zone checks only when the query's reach misses part of the table
                const float4 tb = ctx->table_box;
                const bool covers = d.box.x <= tb.x && d.box.y <= tb.y && d.box.z >= tb.z && d.box.w >= tb.w;
                d.zones = (ctx->zones_valid && !covers) ? (const float4*)ctx->zones.p : nullptr;
            }
            if ((p->mode == BQ_LABEL || p->mode == BQ_TLABEL) && d.P <= kBatchHistCap) max_hist = std::max(max_hist, d.P);
            if (p->mode == BQ_SPLAT && p->T == 1 && p->npix <= (size_t)kBatchHistCap) {
                // small canvas: splat into the block's shared histogram (indexed by
                // pixel) and flush into the canvas
                d.P = (int)p->npix;
                d.out_count = nullptr;
                d.out_count32 = p->cc;
                d.out_sum = reinterpret_cast<unsigned long long*>(p->cs);
                max_hist = std::max(max_hist, d.P);
            }
            act.push_back(p);
        }
        const int hist_cap = (max_hist + 1) & ~1;
        for (size_t i = 0; i < nw; ++i)
            hq[i].hist_smem = (hq[i].mode == BQ_LABEL || hq[i].mode == BQ_TLABEL || hq[i].out_count32) &&
                                      hq[i].P <= hist_cap ? 1 : 0;
        ba.nu = (int)ucols.size();
        for (int u = 0; u < ba.nu; ++u) {
            ba.ucol[u] = ucols[u];
            ba.utyp[u] = utyps[u];
        }
        // act[] indices -> wave indices for the query lists
        std::vector<int> act_idx;
        for (size_t i = 0; i < nw; ++i)
            if (wave[i]->mode != BQ_SKIP) act_idx.push_back((int)i);
        BatchShape shape = e.shape;
        std::vector<BatchSeg> segs;
        std::vector<int> qlist;
        uint64_t nitems = 0, rows_read = 0, pq = 0;
        build_segments(act, segs, qlist, shape.rows, nitems, rows_read, pq);
        for (int& v : qlist) v = act_idx[v];
        BatchSeg* dseg = ar.take<BatchSeg>(segs.size());
        int* dql = ar.take<int>(qlist.size());
        if (!dseg || !dql) return fail(ctx, RJ_E_OOM, "batch arena too small for the work lists");
        RJ_CUDA(cudaMemcpyAsync(dq, hq.data(), nw * sizeof(BatchQuery), cudaMemcpyHostToDevice, st));
        if (!segs.empty()) {
            RJ_CUDA(cudaMemcpyAsync(dseg, segs.data(), segs.size() * sizeof(BatchSeg), cudaMemcpyHostToDevice, st));
            RJ_CUDA(cudaMemcpyAsync(dql, qlist.data(), qlist.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        }
        ba.q = dq;
        ba.qlist = dql;
        ba.seg = dseg;
        ba.nseg = (int)segs.size();
        ba.work = work;
        ba.hist_cap = hist_cap;
        // ---- block-shape tuner: time every shape that fits on this batch
        auto set_shape = [&](const BatchShape& s) {
            // item numbering depends on rows per item
            build_segments(act, segs, qlist, s.rows, nitems, rows_read, pq);
            for (int& v : qlist) v = act_idx[v];
            ba.rows = s.rows;
            ba.nitems = nitems;
            ba.nseg = (int)segs.size();
            cudaMemcpyAsync(dseg, segs.data(), segs.size() * sizeof(BatchSeg), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dql, qlist.data(), qlist.size() * sizeof(int), cudaMemcpyHostToDevice, st);
        };
        auto zero_outputs = [&]() {
            cudaMemsetAsync(oc, 0, outs * 8, st);
            cudaMemsetAsync(os, 0, outs * 8, st);
            cudaMemsetAsync(onf, 0, outs * 8, st);
            for (QPlan* p : act) {
                if (p->mode == BQ_SPLAT) {
                    cudaMemsetAsync(p->cc, 0, p->npix * 4, st);
                    if (p->cs) cudaMemsetAsync(p->cs, 0, p->npix * 8, st);
                } else if (p->mode == BQ_TSPLAT) {
                    const size_t spx = (size_t)std::max(p->nslots, 1) * 256;
                    cudaMemsetAsync(p->tr.bcnt, 0, p->nblk * 4, st);
                    cudaMemsetAsync(p->tr.pcnt, 0, spx * 4, st);
                    if (p->tr.bsum) cudaMemsetAsync(p->tr.bsum, 0, p->nblk * 8, st);
                    if (p->tr.psum) cudaMemsetAsync(p->tr.psum, 0, spx * 8, st);
                }
            }
        };
        if ((flags & RJ_BATCH_AUTOTUNE) && !e.tuned && nitems > 0) {
            static const BatchShape cands[] = {{256, 2048, 0},  {256, 4096, 0},  {256, 8192, 0},  {512, 4096, 0},
                                               {256, 8192, 1},  {256, 16384, 1}, {256, 32768, 1}, {512, 16384, 1},
                                               {512, 32768, 1}};
            float best = 1e30f;
            BatchShape bs = shape;
            for (const BatchShape& c : cands) {
                if (batch_blocks_per_sm(c, ba.nu, hist_cap) < 1) continue;
                set_shape(c);
                zero_outputs();
                cudaMemsetAsync(work, 0, 8, st);
                cudaEventRecord(e.ev[4], st);
                launch_batch_points(ba, c, ctx->sms, st);
                cudaEventRecord(e.ev[5], st);
                RJ_CUDA(cudaStreamSynchronize(st));
                RJ_CUDA(cudaGetLastError());
                const float ms = ev_ms(e.ev[4], e.ev[5]);
                if (ms < best) { best = ms; bs = c; }
            }
            shape = bs;
            e.shape = bs;
            e.tuned = true;
            bo.tuned = 1;
            zero_outputs();
        }
        if (batch_blocks_per_sm(shape, ba.nu, hist_cap) < 1) shape = {256, 2048, 0};
        set_shape(shape);
        RJ_CUDA(cudaMemsetAsync(work, 0, 8, st));
        if (!launch_batch_points(ba, shape, ctx->sms, st))
            return fail(ctx, RJ_E_CUDA, "batched point pass does not fit the device (shared memory)");
        RJ_CUDA(cudaGetLastError());
        cudaEventRecord(e.ev[2], st);
        // ---- canvas-path queries: polygon pass over their canvases
        for (QPlan* p : act) {
            if (p->mode == BQ_SPLAT) {
                if (!query_poly_pass(e, *p, MODE_REDUCE, ps, oc + p->out_off, os + p->out_off, nullptr))
                    return fail(ctx, RJ_E_INVALID, "too many (tile, polygon) items");
            } else if (p->mode == BQ_TSPLAT) {
                if (!query_poly_pass(e, *p, MODE_TIER_REDUCE, ps, oc + p->out_off, os + p->out_off, nullptr, &p->tr))
                    return fail(ctx, RJ_E_INVALID, "too many (tile, polygon) items");
            }
        }
        RJ_CUDA(cudaGetLastError());
        cudaEventRecord(e.ev[3], st);
        // ---- results
        unsigned long long* h = (unsigned long long*)engine_pinned(e, 3 * outs * 8);
        if (!h) return fail(ctx, RJ_E_OOM, "pinned host staging failed");
        RJ_CUDA(cudaMemcpyAsync(h, oc, outs * 8, cudaMemcpyDeviceToHost, st));
        RJ_CUDA(cudaMemcpyAsync(h + outs, os, outs * 8, cudaMemcpyDeviceToHost, st));
        RJ_CUDA(cudaMemcpyAsync(h + 2 * outs, onf, outs * 8, cudaMemcpyDeviceToHost, st));
        RJ_CUDA(cudaStreamSynchronize(st));
        RJ_CUDA(cudaGetLastError());
        const double* hnf = reinterpret_cast<const double*>(h + 2 * outs);
        for (QPlan* p : wave)
            decode_result(p->ps->P, h + p->out_off, h + outs + p->out_off, hnf + p->out_off, p->shift, nullptr, p->res);
        bo.fused += (int)nw;
        bo.segments += (int)segs.size();
        bo.items += nitems;
        bo.rows_read += rows_read;
        bo.point_queries += pq;
        bo.poly_ms += ev_ms(e.ev[0], e.ev[1]);
        bo.point_ms += ev_ms(e.ev[1], e.ev[2]);
        bo.reduce_ms += ev_ms(e.ev[2], e.ev[3]);
    }
    return RJ_OK;
}

// Raster queries that leave the fused pass, queued on the lanes: the device
// work of rj_execute (enqueue_query_untimed) with the query's polygon set
// bound, the outputs copied to pinned staging on the lane, nothing waited
// for.  Queries of one polygon set share a lane (the set's host-side caches
// are filled in stream order).  lanes_finish waits for the lanes and decodes.
struct LaneRun {
    std::vector<QPlan*> q;
    std::vector<size_t> off;     // staging offset of each query's outputs
    std::vector<int> shift;
    std::vector<bool> bounds;
    bool queued = false;
};

int lanes_enqueue(Engine& e, LaneRun& lr, int& launches) {
    rj_ctx* ctx = e.ctx;
    if (lr.q.empty()) return RJ_OK;
    if (!e.lane_err) {
        for (auto& s : e.lane_st)
            if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return fail(ctx, RJ_E_CUDA, "lane stream");
        if (cudaEventCreateWithFlags(&e.lane_ev, cudaEventDisableTiming) != cudaSuccess) return fail(ctx, RJ_E_CUDA, "lane event");
        if (cudaMalloc(&e.lane_err, kLanes * sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, RJ_E_OOM, "lane error words");
        }
    }
    const size_t nq = lr.q.size();
    lr.off.assign(nq, 0);
    lr.shift.assign(nq, 0);
    lr.bounds.assign(nq, false);
    size_t bytes = 0;
    for (size_t i = 0; i < nq; ++i) {
        lr.off[i] = bytes;
        lr.bounds[i] = lr.q[i]->q->function_type == RJ_RASTER_JOIN_BOUNDS;
        const size_t P = (size_t)lr.q[i]->ps->P;
        bytes += al256(P * 24 + (lr.bounds[i] ? P * 32 : 0) + 8);
    }
    if (e.lane_pin_bytes < bytes) {
        if (e.lane_pin) cudaFreeHost(e.lane_pin);
        e.lane_pin = nullptr;
        e.lane_pin_bytes = 0;
        if (cudaMallocHost(&e.lane_pin, bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, RJ_E_OOM, "pinned staging of the lanes");
        }
        e.lane_pin_bytes = bytes;
    }
    char* h = (char*)e.lane_pin;
    {
        // the lanes start after the work already queued on the context's stream
        std::lock_guard<std::recursive_mutex> lock(ctx->mu);
        RJ_CUDA(cudaEventRecord(e.lane_ev, ctx->stream));
        for (auto& s : e.lane_st) RJ_CUDA(cudaStreamWaitEvent(s, e.lane_ev, 0));
    }
    std::map<const PolySet*, int> lane_of;
    int next = 0;
    for (size_t i = 0; i < nq; ++i) {
        // the context is taken per query, so that other callers (another
        // serving slot, a submit) interleave with a long batch
        std::lock_guard<std::recursive_mutex> lock(ctx->mu);
        cudaStream_t saved_st = ctx->stream;
        int* saved_err = ctx->d_err;
        PolySet* saved_ps = ctx->ps;
        const std::string saved_ns = ctx->scratch_ns;
        QPlan& p = *lr.q[i];
        auto it = lane_of.find(p.ps);
        const int l = it != lane_of.end() ? it->second : (lane_of[p.ps] = (next++) % e.nlanes);
        ctx->stream = e.lane_st[l];
        ctx->d_err = e.lane_err + l;
        ctx->scratch_ns = "#e" + std::to_string(e.id) + "." + std::to_string(l);
        ctx->ps = p.ps;
        unsigned long long *oc = nullptr, *os = nullptr;
        double* onf = nullptr;
        long long* ob = nullptr;
        int rc = enqueue_query_untimed(ctx, p.q, &oc, &os, &onf, &ob);
        launches += g_kernel_launches;
        if (!rc) {
            lr.shift[i] = ctx->sum_shift;
            const size_t P = (size_t)p.ps->P;
            char* b = h + lr.off[i];
            cudaStream_t st = ctx->stream;
            if (cudaMemcpyAsync(b, oc, P * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaMemcpyAsync(b + P * 8, os, P * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaMemcpyAsync(b + P * 16, onf, P * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                (lr.bounds[i] && cudaMemcpyAsync(b + P * 24, ob, P * 32, cudaMemcpyDeviceToHost, st) != cudaSuccess) ||
                cudaMemcpyAsync(b + P * (lr.bounds[i] ? 56 : 24), ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost,
                                st) != cudaSuccess) {
                cudaGetLastError();
                rc = fail(ctx, RJ_E_CUDA, "query %d: copying its outputs back", p.idx);
            }
        }
        if (rc) {
            cudaStreamSynchronize(ctx->stream);
            p.status = rc;
        }
        ctx->stream = saved_st;
        ctx->d_err = saved_err;
        ctx->ps = saved_ps;
        ctx->scratch_ns = saved_ns;
    }
    lr.queued = true;
    return RJ_OK;
}

// Frees the lanes' scratch buffers of this engine (their keys carry the
// engine's lane suffix); the caller holds the context lock and no lane work
// is in flight.
void release_lane_scratch(Engine& e) {
    rj_ctx* ctx = e.ctx;
    const std::string tag = "#e" + std::to_string(e.id) + ".";
    for (auto it = ctx->scratch.begin(); it != ctx->scratch.end();) {
        if (it->first.find(tag) != std::string::npos) {
            dev_free(ctx, it->second);
            it = ctx->scratch.erase(it);
        } else {
            ++it;
        }
    }
}

int lanes_finish(Engine& e, LaneRun& lr) {
    if (!lr.queued) return RJ_OK;
    int rc = RJ_OK;
    for (auto& s : e.lane_st)
        if (s && cudaStreamSynchronize(s) != cudaSuccess) rc = RJ_E_CUDA;
    if (rc) {
        cudaGetLastError();
        for (QPlan* p : lr.q)
            if (p->status == RJ_OK) p->status = RJ_E_CUDA;
        return fail(e.ctx, RJ_E_CUDA, "a lane of the batch failed");
    }
    const char* h = (const char*)e.lane_pin;
    for (size_t i = 0; i < lr.q.size(); ++i) {
        QPlan& p = *lr.q[i];
        if (p.status != RJ_OK) continue;
        const size_t P = (size_t)p.ps->P;
        const char* b = h + lr.off[i];
        int derr = 0;
        std::memcpy(&derr, b + P * (lr.bounds[i] ? 56 : 24), sizeof derr);
        if (derr) {
            p.status = fail(e.ctx, RJ_E_TIMEOUT, "query %d: a bounded device wait ran out (status 0x%x)", p.idx, derr);
            continue;
        }
        decode_result((int)P, (const unsigned long long*)b, (const unsigned long long*)(b + P * 8),
                      (const double*)(b + P * 16), lr.shift[i],
                      lr.bounds[i] ? (const long long*)(b + P * 24) : nullptr, p.res);
    }
    lr.queued = false;
    return RJ_OK;
}

// One query through rj_execute with its polygon set bound.
int run_plain(rj_ctx* ctx, QPlan& p) {
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    PolySet* saved = ctx->ps;
    ctx->ps = p.ps;
    const int rc = rj_execute(ctx, p.q, p.res);
    ctx->ps = saved;
    return rc;
}

int execute_batch(Engine& e, int nq, const rj_query* qs, const rj_query* const* qptr, rj_polyset* const* sets,
                  rj_result* res, rj_result* const* rptr, int32_t* status, uint32_t flags, rj_batch_stats* stats) {
    rj_ctx* ctx = e.ctx;
    const double t0 = now_ms();
    std::vector<QPlan> plans(nq);
    g_kernel_launches = 0;
    // every raster query goes to the lanes unless the fused pass is asked for
    const bool lanes_all = e.lanes && !(flags & (RJ_BATCH_FUSE | RJ_BATCH_FUSE_ALL | RJ_BATCH_NO_FUSE));
    {
        std::lock_guard<std::recursive_mutex> lock(ctx->mu);
        if (ctx->npts == 0 && ctx->cols.empty()) return fail(ctx, RJ_E_NO_DATA, "point table not loaded");
        for (int i = 0; i < nq; ++i) {
            QPlan& p = plans[i];
            p.idx = i;
            p.q = qptr ? qptr[i] : qs + i;
            p.set = sets ? sets[i] : nullptr;
            p.ps = p.set ? &p.set->s : &ctx->own;
            p.res = rptr ? rptr[i] : (res ? res + i : nullptr);
            if (p.set && p.set->ctx != ctx) { p.status = fail(ctx, RJ_E_INVALID, "query %d: polygon set of another context", i); continue; }
            if (p.ps->P == 0) { p.status = fail(ctx, RJ_E_NO_DATA, "query %d: polygons not set", i); continue; }
            if (p.res && p.res->npolys != 0 && p.res->npolys != p.ps->P) {
                p.status = fail(ctx, RJ_E_INVALID, "query %d: result sized for %d polygons, set has %d", i, p.res->npolys, p.ps->P);
                continue;
            }
            plan_query(ctx, p, (flags & RJ_BATCH_NO_FUSE) != 0 || lanes_all, (flags & RJ_BATCH_FUSE_ALL) != 0);
        }
        const int zrc = ensure_zones(ctx);   // lets the point pass skip rows far from a query
        if (zrc) return zrc;
    }
    const double t_setup = now_ms();
    BatchOut bo;
    // raster queries that leave the fused pass go to the lanes first (queued,
    // not waited for), so that they overlap with the fused pass; with
    // RJ_BATCH_NO_FUSE every query runs through rj_execute in turn instead
    LaneRun lr;
    int plain_launches = 0;
    if (e.lanes && !(flags & RJ_BATCH_NO_FUSE) && !ctx->streamed)
        for (QPlan& p : plans)
            if (p.status == RJ_OK && !p.fused &&
                (p.q->function_type == RJ_RASTER_JOIN || p.q->function_type == RJ_RASTER_JOIN_BOUNDS))
                lr.q.push_back(&p);
    int rc = lanes_enqueue(e, lr, plain_launches);
    if (rc) {
        for (QPlan* p : lr.q)
            if (p->status == RJ_OK) p->status = rc;
        lr.q.clear();
    }
    g_kernel_launches = 0;
    rc = run_fused(e, plans, flags, bo);
    if (rc) {
        for (QPlan& p : plans)
            if (p.fused && p.status == RJ_OK) p.status = rc;
    }
    const int launches_fused = g_kernel_launches;
    for (QPlan& p : plans) {
        if (p.status != RJ_OK || p.fused) continue;
        if (std::find(lr.q.begin(), lr.q.end(), &p) != lr.q.end()) continue;
        p.status = run_plain(ctx, p);
        plain_launches += ctx->tm.kernel_launches;
        ++bo.fallback;
    }
    lanes_finish(e, lr);
    bo.fallback += (int)lr.q.size();
    // A query the lanes could not hold (its lane's scratch beside the other
    // lanes' exceeded the memory budget) runs again alone once the lanes'
    // scratch is released.
    bool retry = false;
    for (QPlan* p : lr.q) retry = retry || p->status == RJ_E_OOM;
    if (retry) {
        {
            std::lock_guard<std::recursive_mutex> lock(ctx->mu);
            release_lane_scratch(e);
        }
        for (QPlan* p : lr.q) {
            if (p->status != RJ_E_OOM) continue;
            p->status = run_plain(ctx, *p);
            plain_launches += ctx->tm.kernel_launches;
        }
    }
    int first = RJ_OK;
    for (QPlan& p : plans) {
        if (status) status[p.idx] = p.status;
        if (p.status != RJ_OK && first == RJ_OK) first = p.status;
    }
    if (stats) {
        std::memset(stats, 0, sizeof *stats);
        stats->nqueries = nq;
        stats->fused = bo.fused;
        stats->fallback = bo.fallback;
        stats->segments = bo.segments;
        stats->items = bo.items;
        stats->rows_read = bo.rows_read;
        stats->point_queries = bo.point_queries;
        stats->total_ms = now_ms() - t0;
        stats->setup_ms = t_setup - t0;
        stats->poly_ms = bo.poly_ms;
        stats->point_ms = bo.point_ms;
        stats->reduce_ms = bo.reduce_ms;
        stats->threads = e.shape.threads;
        stats->rows_per_item = e.shape.rows;
        stats->direct = e.shape.direct;
        stats->tuned = bo.tuned;
        stats->kernel_launches = launches_fused + plain_launches;
    }
    return first;
}

}  // namespace

namespace rjh {
void free_batch_engine(rj_ctx* ctx) {
    Engine* e = (Engine*)ctx->batch_engine;
    if (!e) return;
    engine_free(*e);
    delete e;
    ctx->batch_engine = nullptr;
}
}  // namespace rjh

// ---------------------------------------------------------------------------
// Serving loop.
namespace {

struct Request {
    uint64_t ticket = 0;
    rj_query q{};
    rj_polyset* ps = nullptr;
    rj_result* res = nullptr;
    size_t need = 0;             // arena bytes of its canvas / label map
    double submit_ms = 0, start_ms = 0, done_ms = 0;
    int batch_id = -1, batch_size = 0, status = RJ_OK;
    bool done = false;
};

}  // namespace

struct rj_server {
    rj_ctx* ctx = nullptr;
    rj_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, Request*> reqs;
    uint64_t next_ticket = 1;
    int next_batch = 0;
    bool stop = false;
    std::vector<Engine*> engines;
    std::vector<std::thread> workers;
};

namespace {

size_t request_need(rj_ctx* ctx, const rj_query* q, const PolySet& ps, bool lanes) {
    // the lanes work in the context's scratch, not in the slot's arena
    if (lanes || q->function_type != RJ_RASTER_JOIN) return 0;
    RasterPlan rp;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    if (plan_raster_bbox(ctx, ps.bbox, q, rp)) return 0;
    const size_t npix = (size_t)rp.resx * rp.resy * rp.splitx * rp.splity;
    return al256(npix * 2) + (size_t)ps.P * 24;
}

void server_worker(rj_server* s, Engine* e) {
    cudaSetDevice(s->ctx->device);
    const size_t cap = e->cap;
    for (;;) {
        std::vector<Request*> batch;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || !s->queue.empty(); });
            if (s->queue.empty()) {
                if (s->stop) return;
                continue;
            }
            if (s->cfg.max_wait_ms > 0 && (int)s->queue.size() < s->cfg.max_batch && !s->stop) {
                // hold the batch open for more arrivals, at most max_wait_ms after the oldest
                const double deadline = s->queue.front()->submit_ms + s->cfg.max_wait_ms;
                while (!s->stop && (int)s->queue.size() < s->cfg.max_batch) {
                    const double left = deadline - now_ms();
                    if (left <= 0) break;
                    s->cv_work.wait_for(lk, std::chrono::microseconds((int64_t)(left * 1000.0)));
                }
                if (s->queue.empty()) continue;
            }
            size_t used = 0;
            while (!s->queue.empty() && (int)batch.size() < s->cfg.max_batch) {
                Request* r = s->queue.front();
                if (!batch.empty() && cap && used + r->need > cap / 2) break;   // admission by canvas memory
                used += r->need;
                batch.push_back(r);
                s->queue.pop_front();
            }
            const int id = s->next_batch++;
            const double t = now_ms();
            for (Request* r : batch) {
                r->batch_id = id;
                r->batch_size = (int)batch.size();
                r->start_ms = t;
            }
        }
        const int n = (int)batch.size();
        std::vector<const rj_query*> qp(n);
        std::vector<rj_polyset*> sp(n);
        std::vector<rj_result*> rp(n);
        std::vector<int32_t> st(n, RJ_OK);
        for (int i = 0; i < n; ++i) {
            qp[i] = &batch[i]->q;
            sp[i] = batch[i]->ps;
            rp[i] = batch[i]->res;
        }
        execute_batch(*e, n, nullptr, qp.data(), sp.data(), nullptr, rp.data(), st.data(), s->cfg.batch_flags,
                      nullptr);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            const double t = now_ms();
            for (int i = 0; i < n; ++i) {
                batch[i]->status = st[i];
                batch[i]->done_ms = t;
                batch[i]->done = true;
            }
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

}  // namespace

// ===========================================================================
extern "C" {

int rj_polyset_create(rj_ctx* ctx, const float* xy, const int32_t* pindex, int32_t npolys, const double* bbox,
                      rj_polyset** out) {
    if (!ctx || !out) return RJ_E_INVALID;
    *out = nullptr;
    // no context lock: the new set is private until returned, and its upload
    // does not wait for joins in flight
    rj_polyset* ps = new rj_polyset();
    ps->ctx = ctx;
    int rc = load_polyset(ctx, ps->s, xy, pindex, npolys, bbox);
    if (rc) {
        free_polyset(ctx, ps->s);
        delete ps;
        return rc;
    }
    *out = ps;
    return RJ_OK;
}

void rj_polyset_destroy(rj_polyset* ps) {
    if (!ps) return;
    rj_ctx* ctx = ps->ctx;
    {
        std::lock_guard<std::recursive_mutex> lock(ctx->mu);
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        if (ctx->ps == &ps->s) ctx->ps = &ctx->own;
        if (ctx->cache_owner == &ps->s) ctx->cache_owner = nullptr;
        free_polyset(ctx, ps->s);
    }
    delete ps;
}

int rj_use_polyset(rj_ctx* ctx, rj_polyset* ps) {
    if (!ctx) return RJ_E_INVALID;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    if (ps && ps->ctx != ctx) return fail(ctx, RJ_E_INVALID, "polygon set belongs to another context");
    ctx->ps = ps ? &ps->s : &ctx->own;
    return RJ_OK;
}

int rj_build_time_index(rj_ctx* ctx, int32_t attrib, int32_t nbuckets) {
    return rj_cluster_points(ctx, attrib, nbuckets, 0);
}

int rj_cluster_points(rj_ctx* ctx, int32_t attrib, int32_t nbuckets, int32_t cell_bits) {
    if (!ctx) return RJ_E_INVALID;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    ctx->err.clear();
    if (ctx->server_running) return fail(ctx, RJ_E_BUSY, "a serving loop owns the context");
    if (ctx->cols.empty()) return fail(ctx, RJ_E_NO_DATA, "point table not loaded");
    if (ctx->streamed) return fail(ctx, RJ_E_UNSUPPORTED, "a streamed (host-resident) table cannot be reordered");
    const Column* tc = nullptr;
    if (attrib >= 0) {
        tc = find_col(ctx, attrib);
        if (!tc || tc->type != RJ_UINT)
            return fail(ctx, RJ_E_INVALID, "time attribute %d is not a loaded uint column", attrib);
    }
    if (cell_bits < 0 || cell_bits > 12) return fail(ctx, RJ_E_INVALID, "cell_bits must be 0..12");
    if (!tc && cell_bits == 0) return fail(ctx, RJ_E_INVALID, "nothing to order by (no time attribute, no cells)");
    const int nbt = tc ? (nbuckets > 0 ? nbuckets : 16384) : 1;
    if (nbt > (1 << 24)) return fail(ctx, RJ_E_INVALID, "too many time buckets");
    const uint64_t nkeys = (uint64_t)nbt << (2 * cell_bits);
    if (nkeys > (1ULL << 24)) return fail(ctx, RJ_E_INVALID, "time buckets x cells exceed 2^24 keys");
    cudaSetDevice(ctx->device);
    const uint64_t n = ctx->npts;
    cudaStream_t st = ctx->stream;
    const Column* loc = find_col(ctx, ctx->loc_attrib);
    TimeIndex tix;
    tix.attrib = attrib;
    tix.nb = nbt;
    tix.start.assign(nbt + 1, 0);
    if (n == 0) {
        tix.valid = tc != nullptr;
        ctx->tix = tix;
        return RJ_OK;
    }
    ClusterKey key{};
    key.nbt = nbt;
    key.cb = cell_bits;
    key.xy = (const float2*)loc->d;
    DevBuf mm;
    int rc;
    if ((rc = dev_alloc(ctx, mm, 32))) return rc;
    unsigned* dmm = (unsigned*)mm.p;
    unsigned hmm[6] = {0xFFFFFFFFu, 0u, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u};
    cudaMemcpyAsync(dmm, hmm, sizeof hmm, cudaMemcpyHostToDevice, st);
    if (tc) launch_time_minmax((const uint32_t*)tc->d, n, dmm, dmm + 1, ctx->sms, st);
    if (cell_bits) launch_xy_bounds((const float2*)loc->d, n, dmm + 2, ctx->sms, st);
    cudaMemcpyAsync(hmm, dmm, sizeof hmm, cudaMemcpyDeviceToHost, st);
    cudaError_t ce = cudaStreamSynchronize(st);
    dev_free(ctx, mm);
    if (ce != cudaSuccess) return fail(ctx, RJ_E_CUDA, "bounds reduction failed: %s", cudaGetErrorString(ce));
    if (tc) {
        key.t = (const uint32_t*)tc->d;
        key.tmin = tix.tmin = hmm[0];
        key.tmax = tix.tmax = hmm[1];
    }
    if (cell_bits) {
        auto unorder = [](unsigned u) {
            const unsigned b = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
            float f;
            std::memcpy(&f, &b, 4);
            return f;
        };
        const float lx = unorder(hmm[2]), ly = unorder(hmm[3]), hx = unorder(hmm[4]), hy = unorder(hmm[5]);
        const double cells = (double)(1 << cell_bits);
        key.x0 = std::isfinite(lx) ? lx : 0.f;
        key.y0 = std::isfinite(ly) ? ly : 0.f;
        key.sx = (std::isfinite(hx) && hx > lx) ? (float)(cells / ((double)hx - lx)) : 0.f;
        key.sy = (std::isfinite(hy) && hy > ly) ? (float)(cells / ((double)hy - ly)) : 0.f;
    }
    // key histogram -> row offsets
    DevBuf hist, cursor;
    if ((rc = dev_alloc(ctx, hist, nkeys * 4))) return rc;
    cudaMemsetAsync(hist.p, 0, nkeys * 4, st);
    launch_cluster_hist(key, n, (unsigned*)hist.p, ctx->sms, st);
    std::vector<unsigned> hh(nkeys);
    cudaMemcpyAsync(hh.data(), hist.p, nkeys * 4, cudaMemcpyDeviceToHost, st);
    ce = cudaStreamSynchronize(st);
    dev_free(ctx, hist);
    if (ce != cudaSuccess) return fail(ctx, RJ_E_CUDA, "key histogram failed: %s", cudaGetErrorString(ce));
    std::vector<uint64_t> start(nkeys + 1, 0);
    for (uint64_t b = 0; b < nkeys; ++b) start[b + 1] = start[b] + hh[b];
    if (start[nkeys] != n) return fail(ctx, RJ_E_CUDA, "key histogram does not add up");
    for (int b = 0; b <= nbt; ++b) tix.start[b] = start[(uint64_t)b << (2 * cell_bits)];
    if (tc && cell_bits == 0) {
        // a table already in bucket order keeps its row order
        DevBuf flag;
        if ((rc = dev_alloc(ctx, flag, 8))) return rc;
        cudaMemsetAsync(flag.p, 0, 8, st);
        launch_time_unsorted((const uint32_t*)tc->d, n, tix.tmin, tix.tmax, nbt, (unsigned long long*)flag.p, ctx->sms, st);
        unsigned long long unsorted = 1;
        cudaMemcpyAsync(&unsorted, flag.p, 8, cudaMemcpyDeviceToHost, st);
        ce = cudaStreamSynchronize(st);
        dev_free(ctx, flag);
        if (ce != cudaSuccess) return fail(ctx, RJ_E_CUDA, "time order check failed: %s", cudaGetErrorString(ce));
        if (unsorted == 0) {
            tix.valid = true;
            ctx->tix = tix;
            return RJ_OK;
        }
    }
    if ((rc = dev_alloc(ctx, cursor, nkeys * 8))) return rc;
    cudaMemcpyAsync(cursor.p, start.data(), nkeys * 8, cudaMemcpyHostToDevice, st);
    // new column buffers in key order
    PermuteCols pc{};
    pc.ncol = (int)ctx->cols.size();
    std::vector<void*> fresh(pc.ncol, nullptr);
    for (int c = 0; c < pc.ncol; ++c) {
        const Column& col = ctx->cols[c];
        const size_t esz = col.type == RJ_LOCATION ? 8 : 4;
        const size_t bytes = esz * ((n + 3) & ~3ULL) + 256;
        if (ctx->budget > 0 && (int64_t)(ctx->used + bytes) > ctx->budget) ce = cudaErrorMemoryAllocation;
        else ce = cudaMalloc(&fresh[c], bytes);
        if (ce != cudaSuccess) {
            cudaGetLastError();
            for (void* p : fresh)
                if (p) cudaFree(p);
            dev_free(ctx, cursor);
            return fail(ctx, RJ_E_OOM, "no device memory for the reordered table");
        }
        cudaMemsetAsync((char*)fresh[c] + esz * n, 0, bytes - esz * n, st);
        pc.src[c] = col.d;
        pc.dst[c] = fresh[c];
        pc.esz[c] = (int)esz;
    }
    launch_cluster_scatter(key, n, (unsigned long long*)cursor.p, pc, ctx->sms, st);
    ce = cudaStreamSynchronize(st);
    dev_free(ctx, cursor);
    if (ce != cudaSuccess) {
        for (void* p : fresh) cudaFree(p);
        return fail(ctx, RJ_E_CUDA, "reorder scatter failed: %s", cudaGetErrorString(ce));
    }
    for (int c = 0; c < pc.ncol; ++c) {
        Column& col = ctx->cols[c];
        const size_t esz = col.type == RJ_LOCATION ? 8 : 4;
        const size_t bytes = esz * ((n + 3) & ~3ULL) + 256;
        if (col.owned) {
            cudaFree(col.d);
            ctx->used -= bytes;
        }
        col.d = fresh[c];
        col.owned = true;
        ctx->used += bytes;
    }
    tix.valid = tc != nullptr;
    ctx->tix = tix;
    ctx->zones_valid = false;   // rows moved
    ++ctx->table_gen;
    return RJ_OK;
}

int rj_execute_batch(rj_ctx* ctx, int32_t nq, const rj_query* q, rj_polyset* const* sets, rj_result* res,
                     int32_t* status, uint32_t flags, rj_batch_stats* stats) {
    if (!ctx || nq < 0 || (nq > 0 && !q)) return RJ_E_INVALID;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    ctx->err.clear();
    if (ctx->server_running) return fail(ctx, RJ_E_BUSY, "a serving loop owns the context");
    cudaSetDevice(ctx->device);
    Engine* e = (Engine*)ctx->batch_engine;
    if (!e || e->st != ctx->stream) {
        if (e) {
            engine_free(*e);
            delete e;
        }
        e = new Engine();
        ctx->batch_engine = e;
        if (engine_init(ctx, *e, ctx->stream, 0)) {
            delete e;
            ctx->batch_engine = nullptr;
            return fail(ctx, RJ_E_CUDA, "batch engine setup failed");
        }
        e->lanes = true;
    }
    int rc = execute_batch(*e, nq, q, nullptr, sets, res, nullptr, status, flags, stats);
    // a large arena (label maps / canvases of a big batch) is not kept between calls
    if (e->ar.buf.bytes > ((size_t)1 << 30)) dev_free(ctx, e->ar.buf);
    return rc;
}

int rj_server_create(rj_ctx* ctx, const rj_server_config* cfg, rj_server** out) {
    if (!ctx || !out) return RJ_E_INVALID;
    *out = nullptr;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    if (ctx->server_running) return fail(ctx, RJ_E_BUSY, "a serving loop already owns the context");
    if (ctx->cols.empty()) return fail(ctx, RJ_E_NO_DATA, "point table not loaded");
    cudaSetDevice(ctx->device);
    rj_server* s = new rj_server();
    s->ctx = ctx;
    if (cfg) s->cfg = *cfg;
    if (s->cfg.slots <= 0) s->cfg.slots = 2;
    if (s->cfg.slots > 8) s->cfg.slots = 8;
    if (s->cfg.canvas_mb <= 0) s->cfg.canvas_mb = 8192;
    if (s->cfg.max_batch <= 0) s->cfg.max_batch = 256;
    const size_t cap = (size_t)s->cfg.canvas_mb << 20;
    for (int i = 0; i < s->cfg.slots; ++i) {
        Engine* e = new Engine();
        int rc = engine_init(ctx, *e, nullptr, cap);
        e->lanes = !(s->cfg.batch_flags & (RJ_BATCH_FUSE | RJ_BATCH_FUSE_ALL | RJ_BATCH_NO_FUSE));
        e->nlanes = 4;
        // the fused pass works in the slot's fixed arena; the lanes in scratch
        if (!rc && !e->lanes) rc = dev_alloc(ctx, e->ar.buf, cap);
        if (rc) {
            engine_free(*e);
            delete e;
            for (Engine* o : s->engines) {
                engine_free(*o);
                delete o;
            }
            delete s;
            return rc == RJ_E_CUDA ? fail(ctx, RJ_E_CUDA, "serving slot setup failed") : rc;
        }
        s->engines.push_back(e);
    }
    ctx->server_running = 1;
    for (Engine* e : s->engines) s->workers.emplace_back(server_worker, s, e);
    *out = s;
    return RJ_OK;
}

int rj_submit(rj_server* s, const rj_query* q, rj_polyset* ps, rj_result* res, uint64_t* ticket) {
    if (!s || !q) return RJ_E_INVALID;
    if (ps && ps->ctx != s->ctx) return RJ_E_INVALID;
    Request* r = new Request();
    r->q = *q;
    r->ps = ps;
    r->res = res;
    r->need = request_need(s->ctx, q, ps ? ps->s : s->ctx->own, !s->engines.empty() && s->engines[0]->lanes);
    r->submit_ms = now_ms();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            delete r;
            return RJ_E_BUSY;
        }
        r->ticket = s->next_ticket++;
        s->reqs[r->ticket] = r;
        s->queue.push_back(r);
    }
    if (ticket) *ticket = r->ticket;
    s->cv_work.notify_one();
    return RJ_OK;
}

int rj_poll(rj_server* s, uint64_t ticket, int32_t timeout_ms, rj_request_info* info) {
    if (!s) return RJ_E_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return RJ_E_INVALID;
    Request* r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return RJ_PENDING;
    if (info) {
        info->submit_ms = r->submit_ms;
        info->start_ms = r->start_ms;
        info->done_ms = r->done_ms;
        info->batch_id = r->batch_id;
        info->batch_size = r->batch_size;
        info->status = r->status;
    }
    const int st = r->status;
    s->reqs.erase(it);
    delete r;
    return st == RJ_OK ? RJ_OK : st;
}

void rj_server_destroy(rj_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (std::thread& t : s->workers) t.join();
    for (Engine* e : s->engines) {
        engine_free(*e);
        delete e;
    }
    for (auto& kv : s->reqs) delete kv.second;
    {
        std::lock_guard<std::recursive_mutex> lock(s->ctx->mu);
        s->ctx->server_running = 0;
    }
    delete s;
}

}  // extern "C"
