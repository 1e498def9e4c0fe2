// rj_runtime.cu -- host runtime behind the C ABI (include/rj.h).
//
// It plays the role of the reference's GLHandler + GLFunction layer
// (RasterJoin/join/GLHandler.cpp, GLFunction.cpp): it owns the device, a
// stream, the resident point table and polygon set, the derived per-polygon-set
// structures (grid index, label maps, masks) and plans every query into kernel
// launches.  Join types dispatch through a table indexed by the reference's
// FunctionType, like GLHandler::initFunctions (GLHandler.cpp:157-186).
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "rj_device.cuh"
#include "rj_internal.h"
#include "rj_launch.h"

using namespace rj;

namespace rjh {


int fail(rj_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) {
        std::lock_guard<std::recursive_mutex> lock(c->mu);
        c->err = buf;
    }
    return code;
}

// Steps that read a value back to the host before the work can go on cannot
// be captured into a graph (rj_prepare): they refuse while capturing.
int readback_guard(rj_ctx* ctx, const char* what) {
    if (ctx->capturing)
        return fail(ctx, RJ_E_UNSUPPORTED, "%s reads a value back to the host: this query cannot be prepared", what);
    return RJ_OK;
}

int dev_alloc(rj_ctx* ctx, DevBuf& b, size_t bytes) {
    if (b.p && b.bytes >= bytes) return RJ_OK;
    if (b.p) {
        cudaFree(b.p);
        ctx->used -= b.bytes;
        b.p = nullptr;
        b.bytes = 0;
    }
    if (bytes == 0) bytes = 16;
    bytes = (bytes + 255) & ~size_t(255);
    if (ctx->budget > 0 && (int64_t)(ctx->used + bytes) > ctx->budget)
        return fail(ctx, RJ_E_OOM, "device memory budget exceeded: need %zu more bytes, %zu of %lld in use",
                    bytes, (size_t)ctx->used.load(), (long long)ctx->budget);
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b.p = nullptr;
        return fail(ctx, RJ_E_OOM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    }
    b.bytes = bytes;
    ctx->used += bytes;
    return RJ_OK;
}

void dev_free(rj_ctx* ctx, DevBuf& b) {
    if (b.p) {
        cudaFree(b.p);
        ctx->used -= b.bytes;
    }
    b.p = nullptr;
    b.bytes = 0;
}

DevBuf& scratch_buf(rj_ctx* ctx, const char* key) {
    return ctx->scratch_ns.empty() ? ctx->scratch[key] : ctx->scratch[std::string(key) + ctx->scratch_ns];
}

int scratch(rj_ctx* ctx, const char* key, size_t bytes, void** out) {
    DevBuf& b = scratch_buf(ctx, key);
    int rc = dev_alloc(ctx, b, bytes);
    if (rc) return rc;
    *out = b.p;
    return RJ_OK;
}

template <class T>
int scratch_t(rj_ctx* ctx, const char* key, size_t count, T** out) {
    void* p = nullptr;
    int rc = scratch(ctx, key, count * sizeof(T), &p);
    *out = (T*)p;
    return rc;
}

const Column* find_col(const rj_ctx* ctx, int attrib) {
    for (const Column& c : ctx->cols)
        if (c.attrib == attrib) return &c;
    return nullptr;
}

void free_points(rj_ctx* ctx) {
    ++ctx->table_gen;
    for (Column& c : ctx->cols) {
        if (c.owned && c.d) cudaFree(c.d);
    }
    // owned column sizes are tracked in ctx->used by load_points
    ctx->cols.clear();
    ctx->npts = 0;
    ctx->loc_attrib = -1;
}

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

int plan_raster_bbox(rj_ctx* ctx, const double* bbox, const rj_query* q, RasterPlan& rp) {
    // tiles up to the reference's framebuffer side (GLFunction.hpp:14); the
    // tiered canvas's kernels hold a tile row of at most 8192 pixels
    if (q->max_fbo_size > RJ_MAX_FBO_SIZE)
        return fail(ctx, RJ_E_INVALID, "canvas tile side %d above %d", q->max_fbo_size, RJ_MAX_FBO_SIZE);
    double ground = q->ground_resolution > 0 ? q->ground_resolution : 1.0;
    double cell = q->cell_size > 0 ? q->cell_size : (q->accuracy_m / std::sqrt(2.0)) / ground;
    if (!(cell > 0) || !std::isfinite(cell)) return fail(ctx, RJ_E_INVALID, "invalid cell size %g", cell);
    double dx = bbox[2] - bbox[0], dy = bbox[3] - bbox[1];
    if (!(dx > 0 && dy > 0)) return fail(ctx, RJ_E_INVALID, "degenerate polygon bounds");
    double ax = std::ceil(dx / cell), ay = std::ceil(dy / cell);
    if (ax > 2e6 || ay > 2e6) return fail(ctx, RJ_E_INVALID, "canvas too large: %.0f x %.0f", ax, ay);
    rp.cell = cell;
    rp.actual_x = std::max(1, (int)ax);
    rp.actual_y = std::max(1, (int)ay);
    int max_res = q->max_fbo_size > 0 ? q->max_fbo_size : RJ_MAX_FBO_SIZE;
    rp.splitx = (int)std::ceil(double(rp.actual_x) / max_res);
    rp.splity = (int)std::ceil(double(rp.actual_y) / max_res);
    rp.resx = (int)std::ceil(double(rp.actual_x) / rp.splitx);
    rp.resy = (int)std::ceil(double(rp.actual_y) / rp.splity);
    if ((size_t)rp.splitx * rp.splity > 65536) return fail(ctx, RJ_E_INVALID, "too many canvas tiles");
    double tdx = dx / rp.splitx, tdy = dy / rp.splity;
    rp.colxf.resize(rp.splitx);
    rp.rowxf.resize(rp.splity);
    for (int c = 0; c < rp.splitx; ++c) {
        double lb = bbox[0] + c * tdx, rt = lb + tdx;
        double origin = (rt + lb) / 2, half = (rt - lb) / 2;
        float s = (float)(1.0 / half);
        float t = s * (float)(-origin);
        rp.colxf[c] = make_float4(s, t, rp.resx * 0.5f, (float)tdx);
    }
    for (int r = 0; r < rp.splity; ++r) {
        double lb = bbox[1] + r * tdy, rt = lb + tdy;
        double origin = (rt + lb) / 2, half = (rt - lb) / 2;
        float s = (float)(1.0 / half);
        float t = s * (float)(-origin);
        rp.rowxf[r] = make_float4(s, t, rp.resy * 0.5f, (float)tdy);
    }
    return RJ_OK;
}

int plan_raster(rj_ctx* ctx, const rj_query* q, RasterPlan& rp) { return plan_raster_bbox(ctx, ctx->ps->bbox, q, rp); }

uint64_t canvas_key(const std::vector<float4>& colxf, const std::vector<float4>& rowxf, int resx, int resy) {
    uint64_t h = 1469598103934665603ULL;   // FNV-1a
    auto mix = [&](const void* p, size_t n) {
        for (size_t i = 0; i < n; ++i) h = (h ^ ((const unsigned char*)p)[i]) * 1099511628211ULL;
    };
    const int dims[4] = {(int)colxf.size(), (int)rowxf.size(), resx, resy};
    mix(dims, sizeof dims);
    mix(colxf.data(), colxf.size() * sizeof(float4));
    mix(rowxf.data(), rowxf.size() * sizeof(float4));
    return h;
}

// Filter + aggregation (GLFunction::setupPoints GLFunction.cpp:199-344).
int build_filter(rj_ctx* ctx, const rj_query* q, DevFilter& f, bool force_count, bool* empty = nullptr) {
    if (empty) *empty = false;
    std::memset(&f, 0, sizeof f);
    if (q->n_constraints < 0) return fail(ctx, RJ_E_INVALID, "negative constraint count");
    if (q->n_constraints > RJ_MAX_CONSTRAINTS)
        return fail(ctx, RJ_E_TOO_MANY_CONSTRAINTS, "%d constraints, at most %d supported", q->n_constraints,
                    RJ_MAX_CONSTRAINTS);
    // predicates, then grouped by the column they read (each column is loaded once)
    struct Pred { const uint32_t* col; int op, typ; uint32_t val; bool compat; };
    std::vector<Pred> preds;
    for (int i = 0; i < q->n_constraints; ++i) {
        const rj_constraint& c = q->constraints[i];
        const Column* col = find_col(ctx, c.attrib_id);
        if (!col) return fail(ctx, RJ_E_INVALID, "constraint %d: unknown attribute %d", i, c.attrib_id);
        if (col->type == RJ_LOCATION)
            return fail(ctx, RJ_E_UNSUPPORTED, "constraint %d: location attributes cannot be filtered", i);
        if (c.type < RJ_EQ || c.type > RJ_GTE)
            return fail(ctx, RJ_E_INVALID, "constraint %d: bad constraint type %d", i, c.type);
        preds.push_back({(const uint32_t*)col->d, c.type, col->type, c.val.uval, (q->flags & RJ_FLAG_COMPAT_FLOAT_EQ) != 0});
    }
    if (q->time_attrib >= 0) {
        const Column* col = find_col(ctx, q->time_attrib);
        if (!col || col->type == RJ_LOCATION)
            return fail(ctx, RJ_E_INVALID, "time attribute %d is not a loaded scalar column", q->time_attrib);
        preds.push_back({(const uint32_t*)col->d, RJ_GTE, col->type, q->t_start, false});
        preds.push_back({(const uint32_t*)col->d, RJ_LTE, col->type, q->t_end, false});
    }
    int k = 0;
    f.ncol = 0;
    std::vector<bool> used(preds.size(), false);
    for (size_t i = 0; i < preds.size(); ++i) {
        if (used[i]) continue;
        const int c = f.ncol++;
        f.col[c] = preds[i].col;
        f.pstart[c] = k;
        for (size_t j = i; j < preds.size(); ++j) {
            if (used[j] || preds[j].col != preds[i].col) continue;
            used[j] = true;
            f.op[k] = preds[j].op;
            f.typ[k] = preds[j].typ;
            f.val[k] = preds[j].val;
            if (preds[j].compat) f.compat_mask |= 1u << k;
            ++k;
        }
    }
    f.pstart[f.ncol] = k;
    // interval form of every column's predicates (unsatisfiable -> *empty)
    f.general = 0;
    for (int c = 0; c < f.ncol; ++c) {
        uint32_t lo = 0u, hi = 0xFFFFFFFFu;
        const int t = f.typ[f.pstart[c]];
        f.ctyp[c] = t;
        if (t == RJ_FLOAT) {
            lo = order_key(RJ_FLOAT, 0xFF800000u);   // -inf
            hi = order_key(RJ_FLOAT, 0x7F800000u);   // +inf
        }
        for (int j = f.pstart[c]; j < f.pstart[c + 1]; ++j) {
            if (f.compat_mask & (1u << j)) f.general = 1;
            const uint32_t v = f.val[j];
            uint32_t elo, ehi;   // keys of the values equal to v
            if (t == RJ_FLOAT) {
                float fv;
                std::memcpy(&fv, &v, 4);
                if (std::isnan(fv)) { lo = 1; hi = 0; continue; }   // every comparison with NaN fails
                if (fv == 0.0f) { elo = order_key(RJ_FLOAT, 0x80000000u); ehi = order_key(RJ_FLOAT, 0u); }
                else elo = ehi = order_key(RJ_FLOAT, v);
            } else {
                elo = ehi = order_key(t, v);
            }
            uint64_t plo = lo, phi = hi;
            const uint64_t kmin = (t == RJ_FLOAT) ? order_key(RJ_FLOAT, 0xFF800000u) : 0u;
            const uint64_t kmax = (t == RJ_FLOAT) ? order_key(RJ_FLOAT, 0x7F800000u) : 0xFFFFFFFFu;
            int64_t a = (int64_t)kmin, b = (int64_t)kmax;
            switch (f.op[j]) {
                case RJ_EQ: a = elo; b = ehi; break;
                case RJ_LT: b = (int64_t)elo - 1; break;
                case RJ_LTE: b = ehi; break;
                case RJ_GT: a = (int64_t)ehi + 1; break;
                case RJ_GTE: a = elo; break;
            }
            plo = std::max<int64_t>((int64_t)plo, a);
            phi = std::min<int64_t>((int64_t)phi, b);
            if ((int64_t)phi < (int64_t)plo || b < a) { lo = 1; hi = 0; continue; }
            lo = (uint32_t)plo;
            hi = (uint32_t)phi;
        }
        if (hi < lo) {
            // unsatisfiable: evaluate the predicates one by one (they reject every point)
            f.general = 1;
            f.lo[c] = 0;
            f.span[c] = 0;
            if (empty) *empty = true;
        } else {
            f.lo[c] = lo;
            f.span[c] = hi - lo;
        }
    }
    f.n = k;
    f.aggr_ci = -1;
    if (!force_count && q->aggregation != RJ_COUNT) {
        if (q->aggregation != RJ_AVG && q->aggregation != RJ_SUM)
            return fail(ctx, RJ_E_INVALID, "bad aggregation %d", q->aggregation);
        const Column* col = find_col(ctx, q->aggr_attrib);
        if (!col) return fail(ctx, RJ_E_INVALID, "aggregation attribute %d not loaded", q->aggr_attrib);
        if (col->type == RJ_LOCATION)
            return fail(ctx, RJ_E_UNSUPPORTED, "cannot aggregate a location attribute");
        f.aggr = 1;
        f.aggr_typ = col->type;
        f.aggr_col = (const uint32_t*)col->d;
        f.aggr_ci = -1;
        for (int c = 0; c < f.ncol; ++c)
            if (f.col[c] == f.aggr_col) f.aggr_ci = c;
        // fixed-point sums: |v| * 2^s * n < 2^62 for every value and any subset
        int shift = rj_sum_shift_for((double)col->absmax, ctx->npts);
        if (ctx->forced_shift != RJ_SUM_SHIFT_AUTO) {
            if (ctx->forced_shift > shift)
                return fail(ctx, RJ_E_INVALID, "sum shift %d too fine for this table (values up to %g over %llu rows: %d)",
                            ctx->forced_shift, (double)col->absmax, (unsigned long long)ctx->npts, shift);
            shift = ctx->forced_shift;
        }
        ctx->sum_shift = shift;
        f.sum_scale = std::ldexp(1.0f, shift - 32);
    }
    return RJ_OK;
}

struct Phase {
    rj_ctx* ctx;
    bool on;
    explicit Phase(rj_ctx* c, bool enabled) : ctx(c), on(enabled) {}
    void mark(int i) {
        if (on) cudaEventRecord(ctx->ev[i], ctx->stream);
    }
    double ms(int a, int b) {
        if (!on) return 0.0;
        float v = 0.f;
        cudaEventElapsedTime(&v, ctx->ev[a], ctx->ev[b]);
        return v;
    }
};

// Window-space vertices of the polygon set for every canvas tile.
int transform_vertices(rj_ctx* ctx, const std::vector<float4>& colxf, const std::vector<float4>& rowxf,
                       int2** wv, float2** wf, bool want_float) {
    const int T = (int)(colxf.size() * rowxf.size());
    float4 *dcol, *drow;
    int rc;
    if ((rc = scratch_t(ctx, "colxf", colxf.size(), &dcol))) return rc;
    if ((rc = scratch_t(ctx, "rowxf", rowxf.size(), &drow))) return rc;
    if (ctx->capturing) {
        // a graph must not copy from host memory that is gone when it
        // replays: the transforms travel as kernel arguments instead
        if (colxf.size() > (size_t)kXfArgs || rowxf.size() > (size_t)kXfArgs)
            return fail(ctx, RJ_E_UNSUPPORTED, "more than %d canvas tiles per axis: this query cannot be prepared", kXfArgs);
        XfArgs ca{}, ra{};
        for (size_t i = 0; i < colxf.size(); ++i) ca.v[i] = colxf[i];
        for (size_t i = 0; i < rowxf.size(); ++i) ra.v[i] = rowxf[i];
        launch_write_xf(ca, (int)colxf.size(), dcol, ctx->stream);
        launch_write_xf(ra, (int)rowxf.size(), drow, ctx->stream);
    } else {
        RJ_CUDA(cudaMemcpyAsync(dcol, colxf.data(), colxf.size() * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
        RJ_CUDA(cudaMemcpyAsync(drow, rowxf.data(), rowxf.size() * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
    }
    if ((rc = scratch_t(ctx, "wv", (size_t)T * ctx->ps->V, wv))) return rc;
    *wf = nullptr;
    if (want_float && (rc = scratch_t(ctx, "wf", (size_t)T * ctx->ps->V, wf))) return rc;
    launch_transform_vertices((const float2*)ctx->ps->d_verts.p, ctx->ps->V, dcol, drow, (int)colxf.size(), T, *wv,
                              want_float ? *wf : nullptr, ctx->sms, ctx->stream);
    RJ_CUDA(cudaGetLastError());
    return RJ_OK;
}

// Grid index (GLFunction::createPolyIndex GLFunction.cpp:65-156).
int build_grid(rj_ctx* ctx, int res, int clamp, IndexArgs& ia, bool with_pair_cell = false) {
    if (res <= 0 || res > 8192) return fail(ctx, RJ_E_INVALID, "grid resolution %d out of range", res);
    GridCache& g = ctx->ps->grid;
    const double dx = ctx->ps->bbox[2] - ctx->ps->bbox[0], dy = ctx->ps->bbox[3] - ctx->ps->bbox[1];
    const float lbx = (float)ctx->ps->bbox[0], lby = (float)ctx->ps->bbox[1];
    const float csx = (float)(dx / res), csy = (float)(dy / res);
    int *cell_start, *entries;
    int rc;
    const size_t ncells = (size_t)res * res;
    if (!(g.valid && g.res == res && g.clamp == clamp && (g.pair_cell || !with_pair_cell))) {
        int *cnt, *cursor, *tmp;
        if ((rc = scratch_t(ctx, "grid_cnt", ncells, &cnt))) return rc;
        if ((rc = scratch_t(ctx, "grid_start", ncells + 1, &cell_start))) return rc;
        if ((rc = scratch_t(ctx, "grid_tmp", (size_t)scan_tmp_ints((int)ncells), &tmp))) return rc;
        RJ_CUDA(cudaMemsetAsync(cnt, 0, ncells * sizeof(int), ctx->stream));
        GridArgs ga{};
        ga.verts = (const float2*)ctx->ps->d_verts.p;
        ga.pindex = (const int*)ctx->ps->d_pindex.p;
        ga.P = ctx->ps->P;
        ga.lbx = lbx; ga.lby = lby; ga.csx = csx; ga.csy = csy;
        ga.res = res;
        ga.compat_clamp = clamp;
        ga.cell_count = cnt;
        launch_grid_count(ga, ctx->sms, ctx->stream);
        if (!launch_exclusive_scan(cnt, cell_start, (int)ncells, tmp, ctx->stream))
            return fail(ctx, RJ_E_INVALID, "grid too large to scan");
        int total = 0;
        if ((rc = readback_guard(ctx, "building the grid index"))) return rc;
        RJ_CUDA(cudaMemcpyAsync(&total, cell_start + ncells, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        RJ_CUDA(cudaStreamSynchronize(ctx->stream));
        if ((rc = scratch_t(ctx, "grid_entries", (size_t)std::max(total, 1), &entries))) return rc;
        if ((rc = scratch_t(ctx, "grid_cursor", ncells, &cursor))) return rc;
        RJ_CUDA(cudaMemsetAsync(cursor, 0, ncells * sizeof(int), ctx->stream));
        ga.cell_start = cell_start;
        ga.cursor = cursor;
        ga.entries = entries;
        ga.pair_cell = nullptr;
        if (with_pair_cell && (rc = scratch_t(ctx, "grid_pair_cell", (size_t)std::max(total, 1), &ga.pair_cell))) return rc;
        launch_grid_fill(ga, ctx->sms, ctx->stream);
        launch_grid_sort(cell_start, entries, (int)ncells, ctx->sms, ctx->stream);
        RJ_CUDA(cudaGetLastError());
        g.valid = true;
        g.res = res;
        g.clamp = clamp;
        g.nentries = (size_t)total;
        g.pair_cell = with_pair_cell;
    } else {
        if ((rc = scratch_t(ctx, "grid_start", ncells + 1, &cell_start))) return rc;
        if ((rc = scratch_t(ctx, "grid_entries", std::max<size_t>(g.nentries, 1), &entries))) return rc;
    }
    ia.verts = (const float2*)ctx->ps->d_verts.p;
    ia.pindex = (const int*)ctx->ps->d_pindex.p;
    ia.cell_start = cell_start;
    ia.entries = entries;
    ia.lbx = lbx; ia.lby = lby; ia.csx = csx; ia.csy = csy;
    ia.res = res;
    return RJ_OK;
}

// Resolution of the classified grid: the query grid times 2^k, about 1024
// cells across, with cells much larger than the fp32 error of the test.
int exact_res(const rj_ctx* ctx, int res, int max_scale) {
    const double ext = std::max(ctx->ps->bbox[2] - ctx->ps->bbox[0], ctx->ps->bbox[3] - ctx->ps->bbox[1]);
    const double err = std::ldexp(1.0, -21) * (ctx->ps->max_abs_coord + 6.0 * std::max(ctx->ps->max_edge_dx, ctx->ps->max_edge_dy) + 1.0);
    int g = res;
    while (g * 2 <= 1024 && g * 2 <= res * max_scale && ext / (g * 2) > 64.0 * err) g *= 2;
    return g;
}

// Classified grid (FULL / OUT / EDGE per cell and candidate polygon).  The
// candidates of a cell are exactly the reference's: polygons whose MBR cell
// range on the query grid (index-size.glsl:50-68, upper bound clamped to the
// grid) contains the query-grid cell holding it; every query-grid cell is a
// block of 2^k x 2^k classified cells.
// max_scale: finest refinement of the query grid (the hybrid join tests only
// the points near an outline, so a coarser classified grid is cheaper overall).
int build_exact(rj_ctx* ctx, int user_res, ExactIndex& ix, int max_scale = 1024) {
    int rc;
    const int G = exact_res(ctx, user_res, max_scale);
    const int scale = G / user_res;
    ExactCache& xc = ctx->ps->exact;
    const size_t ncells = (size_t)G * G;
    const double dx = ctx->ps->bbox[2] - ctx->ps->bbox[0], dy = ctx->ps->bbox[3] - ctx->ps->bbox[1];
    const float lbx = (float)ctx->ps->bbox[0], lby = (float)ctx->ps->bbox[1];
    const float csx = (float)(dx / G), csy = (float)(dy / G);
    int* start2;
    int4* entries2;
    float4* edges;
    if (!(xc.valid && xc.res == G && xc.user_res == user_res)) {
        // candidate ranges on the query grid, in fp32 as the reference computes them
        const float rcsx = (float)(dx / user_res), rcsy = (float)(dy / user_res);
        const int P = ctx->ps->P;
        std::vector<int> off(P + 1);
        std::vector<int4> rng(P);
        long long total = 0;
        for (int p = 0; p < P; ++p) {
            off[p] = (int)total;
            const float4 m = ctx->ps->h_mbr[p];
            int stx = 0, sty = 0, enx = 0, eny = 0;
            if (ctx->ps->h_pindex[p + 1] > ctx->ps->h_pindex[p]) {
                volatile float ax = m.x - lbx, ay = m.y - lby, bx = m.z - lbx, by = m.w - lby;
                volatile float qx0 = ax / rcsx, qy0 = ay / rcsy, qx1 = bx / rcsx, qy1 = by / rcsy;
                stx = (int)qx0; sty = (int)qy0;
                enx = (int)qx1 + 1; eny = (int)qy1 + 1;
                if (enx >= user_res) enx = user_res;
                if (eny >= user_res) eny = user_res;
                if (stx < 0) stx = 0;
                if (sty < 0) sty = 0;
                if (enx < stx) enx = stx;
                if (eny < sty) eny = sty;
            }
            rng[p] = make_int4(stx, enx, sty, eny);
            total += (long long)(enx - stx) * (eny - sty);
        }
        off[P] = (int)total;
        const long long max_fine = total * scale * scale;
        if (max_fine > (1LL << 30)) return fail(ctx, RJ_E_UNSUPPORTED, "too many cell/polygon candidate pairs (%lld)", max_fine);
        const int npairs1 = (int)total;
        int *doff, *cell_kept, *cursor, *tmp, *plist_n;
        int4 *drng, *info1;
        int2* plist;
        if ((rc = scratch_t(ctx, "cls_off", (size_t)P + 1, &doff))) return rc;
        if ((rc = scratch_t(ctx, "cls_rng", (size_t)P, &drng))) return rc;
        if ((rc = scratch_t(ctx, "cls_info1", (size_t)std::max(npairs1, 1), &info1))) return rc;
        if ((rc = scratch_t(ctx, "cls_plist", (size_t)std::max<long long>(max_fine, 1), &plist))) return rc;
        if ((rc = scratch_t(ctx, "cls_plist_n", 1, &plist_n))) return rc;
        if ((rc = scratch_t(ctx, "cls_kept", ncells, &cell_kept))) return rc;
        if ((rc = scratch_t(ctx, "cls_cursor", ncells, &cursor))) return rc;
        if ((rc = scratch_t(ctx, "cls_start", ncells + 1, &start2))) return rc;
        RJ_CUDA(cudaMemcpyAsync(doff, off.data(), sizeof(int) * (P + 1), cudaMemcpyHostToDevice, ctx->stream));
        RJ_CUDA(cudaMemcpyAsync(drng, rng.data(), sizeof(int4) * P, cudaMemcpyHostToDevice, ctx->stream));
        RJ_CUDA(cudaMemsetAsync(cell_kept, 0, ncells * sizeof(int), ctx->stream));
        RJ_CUDA(cudaMemsetAsync(cursor, 0, ncells * sizeof(int), ctx->stream));
        RJ_CUDA(cudaMemsetAsync(plist_n, 0, sizeof(int), ctx->stream));
        ClsArgs c{};
        c.verts = (const float2*)ctx->ps->d_verts.p;
        c.pindex = (const int*)ctx->ps->d_pindex.p;
        c.P = P;
        c.pair_off = doff;
        c.prange = drng;
        c.plist = plist;
        c.plist_n = plist_n;
        c.scale = scale;
        c.lbx = lbx; c.lby = lby; c.csx = csx; c.csy = csy;
        c.res = G;
        const double U = std::ldexp(1.0, -24);
        const double Mc = std::max<double>(ctx->ps->max_abs_coord, std::max(std::fabs(ctx->ps->bbox[0]), std::fabs(ctx->ps->bbox[2])));
        const double E = 8.0 * U * (Mc + 6.0 * std::max(ctx->ps->max_edge_dx, ctx->ps->max_edge_dy));
        const double delta = 8.0 * U * (2.0 * Mc + G * std::max((double)csx, (double)csy));
        const double rel = 8.0 * U * (Mc + G * std::max((double)csx, (double)csy));
        c.margin = (float)(2.0 * (E + delta + rel) + 1e-7 * std::max(dx, dy));
        c.cell_kept = cell_kept;
        c.cell_start = start2;
        c.cursor = cursor;
        // level 1: coarse pairs
        ClsArgs c1 = c;
        c1.level = 1;
        c1.npairs = npairs1;
        c1.info = info1;
        if (npairs1 > 0) launch_cls_classify(c1, ctx->sms, ctx->stream);
        // level 2: fine cells of the coarse EDGE pairs.  Its pair count stays on
        // the device; buffers are sized for the upper bound (every coarse pair
        // refined) so no host round trip is needed before the scans.
        const int npairs2 = (int)max_fine;
        int4* info2;
        int *ecount, *eoff;
        if ((rc = scratch_t(ctx, "cls_info2", (size_t)std::max(npairs2, 1), &info2))) return rc;
        if ((rc = scratch_t(ctx, "cls_ecount", (size_t)std::max(npairs2, 1), &ecount))) return rc;
        if ((rc = scratch_t(ctx, "cls_eoff", (size_t)npairs2 + 1, &eoff))) return rc;
        const int ntmp = std::max(scan_tmp_ints((int)ncells), scan_tmp_ints(std::max(npairs2, 1)));
        if ((rc = scratch_t(ctx, "cls_tmp", (size_t)ntmp, &tmp))) return rc;
        RJ_CUDA(cudaMemsetAsync(ecount, 0, sizeof(int) * (size_t)std::max(npairs2, 1), ctx->stream));
        ClsArgs c2 = c;
        c2.level = 2;
        c2.npairs = npairs2;
        c2.info = info2;
        c2.ecount = ecount;
        c2.eoff = eoff;
        if (npairs2 > 0) launch_cls_classify(c2, ctx->sms, ctx->stream);
        if (!launch_exclusive_scan(cell_kept, start2, (int)ncells, tmp, ctx->stream))
            return fail(ctx, RJ_E_INVALID, "classified grid too large");
        int totals[2] = {0, 0};
        if ((rc = readback_guard(ctx, "building the classified grid"))) return rc;
        if (npairs2 > 0) {
            if (!launch_exclusive_scan(ecount, eoff, npairs2, tmp, ctx->stream))
                return fail(ctx, RJ_E_UNSUPPORTED, "too many cell/polygon pairs to scan (%d)", npairs2);
            RJ_CUDA(cudaMemcpyAsync(&totals[1], eoff + npairs2, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        }
        RJ_CUDA(cudaMemcpyAsync(&totals[0], start2 + ncells, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        RJ_CUDA(cudaStreamSynchronize(ctx->stream));
        if ((rc = scratch_t(ctx, "cls_entries", (size_t)std::max(totals[0], 1), &entries2))) return rc;
        if ((rc = scratch_t(ctx, "cls_edges", (size_t)std::max(totals[1], 1), &edges))) return rc;
        c1.entries = c2.entries = entries2;
        c2.edges = edges;
        uint32_t* code;
        if ((rc = scratch_t(ctx, "cls_code", ncells, &code))) return rc;
        if (npairs1 > 0) launch_cls_emit(c1, ctx->sms, ctx->stream);
        if (npairs2 > 0) {
            launch_cls_emit(c2, ctx->sms, ctx->stream);
            launch_cls_fill_edges(c2, ctx->sms, ctx->stream);
        }
        launch_cls_codes(start2, entries2, code, (int)ncells, ctx->sms, ctx->stream);
        RJ_CUDA(cudaGetLastError());
        xc.valid = true;
        xc.res = G;
        xc.user_res = user_res;
        xc.nentries = (size_t)totals[0];
        xc.nedges = (size_t)totals[1];
    } else {
        if ((rc = scratch_t(ctx, "cls_start", ncells + 1, &start2))) return rc;
        if ((rc = scratch_t(ctx, "cls_entries", std::max<size_t>(xc.nentries, 1), &entries2))) return rc;
        if ((rc = scratch_t(ctx, "cls_edges", std::max<size_t>(xc.nedges, 1), &edges))) return rc;
    }
    ix.code = (const uint32_t*)scratch_buf(ctx, "cls_code").p;
    ix.cell_start = start2;
    ix.entries = entries2;
    ix.edges = edges;
    ix.lbx = lbx;
    ix.lby = lby;
    ix.csx = csx;
    ix.csy = csy;
    ix.res = G;
    return RJ_OK;
}

PointArgs make_point_args(rj_ctx* ctx, const DevFilter& f, unsigned long long* oc, unsigned long long* os) {
    PointArgs pa{};
    const Column* loc = find_col(ctx, ctx->loc_attrib);
    // rows the query can touch (time index window; the exact time predicate still applies)
    const uint64_t r0 = std::min(ctx->row0, ctx->npts), r1 = std::max(r0, std::min(ctx->row1, ctx->npts));
    pa.xy = (const float2*)loc->d + r0;
    pa.n = r1 - r0;
    pa.f = f;
    for (int c = 0; c < pa.f.ncol; ++c) pa.f.col[c] += r0;
    if (pa.f.aggr_col) pa.f.aggr_col += r0;
    pa.P = ctx->ps->P;
    pa.out_count = oc;
    pa.out_sum = os;
    pa.out_nonfinite = (double*)scratch_buf(ctx, "out_nonfinite").p;
    pa.err = ctx->d_err;
    pa.shape = ctx->point_shape;
    pa.wait_ns = ctx->wait_ns;
    // the zone check costs a dependent load per iteration: skip it when the
    // query's reach holds every finite location of the table (nothing to skip)
    const float4 tb = ctx->table_box, qb = ctx->qbox;
    const bool covers = qb.x <= tb.x && qb.y <= tb.y && qb.z >= tb.z && qb.w >= tb.w;
    if (ctx->zones_valid && !ctx->streamed && !covers && !ctx->capturing) {
        pa.zones = (const float4*)ctx->zones.p;
        pa.row0 = r0;
        pa.qbox = ctx->qbox;
    }
    return pa;
}

// The point pass of one query: one launch over the resident table, or, for a
// streamed table, one launch per chunk of rows, each chunk's columns copied
// into one of two device buffers on a copy stream while the previous chunk
// is processed (the reference's memory passes, GLFunction.cpp:330-337 and
// RasterJoin.cpp:215-236).
template <class Launch>
int point_pass(rj_ctx* ctx, const DevFilter& f, unsigned long long* oc, unsigned long long* os, Launch&& launch) {
    ctx->passes = 1;
    ctx->copy_ms = 0;
    PointArgs pa = make_point_args(ctx, f, oc, os);
    if (!ctx->streamed) {
        launch(pa);
        return RJ_OK;
    }
    // host columns the query reads: location, filter columns, aggregate
    std::vector<const char*> src;
    std::vector<size_t> esz;
    auto slot = [&](const void* p, size_t e) {
        for (size_t i = 0; i < src.size(); ++i)
            if (src[i] == (const char*)p) return (int)i;
        src.push_back((const char*)p);
        esz.push_back(e);
        return (int)src.size() - 1;
    };
    const Column* loc = find_col(ctx, ctx->loc_attrib);
    slot(loc->d, 8);
    int cslot[kMaxFilters];
    for (int c = 0; c < f.ncol; ++c) cslot[c] = slot(f.col[c], 4);
    const int aslot = f.aggr_col ? slot(f.aggr_col, 4) : -1;
    size_t rec = 0;
    for (size_t e : esz) rec += e;
    const uint64_t n = ctx->npts;
    const uint64_t chunk = std::max<uint64_t>(4, ctx->chunk & ~3ULL);
    int rc;
    for (int b = 0; b < 2; ++b)
        if ((rc = dev_alloc(ctx, ctx->sbuf[b], chunk * rec + 256 * src.size()))) return rc;
    if (!ctx->copy_stream) {
        RJ_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        for (int b = 0; b < 2; ++b) {
            RJ_CUDA(cudaEventCreateWithFlags(&ctx->copied[b], cudaEventDisableTiming));
            RJ_CUDA(cudaEventCreateWithFlags(&ctx->consumed[b], cudaEventDisableTiming));
        }
        RJ_CUDA(cudaEventCreate(&ctx->copy_t0));
        RJ_CUDA(cudaEventCreate(&ctx->copy_t1));
    }
    // buffers are free once the work queued so far on the stream has run
    for (int b = 0; b < 2; ++b) RJ_CUDA(cudaEventRecord(ctx->consumed[b], ctx->stream));
    RJ_CUDA(cudaEventRecord(ctx->copy_t0, ctx->copy_stream));
    int passes = 0;
    for (uint64_t r0 = 0; r0 < n; r0 += chunk, ++passes) {
        const int b = passes & 1;
        const uint64_t rows = std::min(chunk, n - r0);
        RJ_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->consumed[b], 0));
        std::vector<char*> dst(src.size());
        char* base = (char*)ctx->sbuf[b].p;
        for (size_t i = 0; i < src.size(); ++i) {
            dst[i] = base;
            base += ((chunk * esz[i]) + 255) & ~(size_t)255;
            RJ_CUDA(cudaMemcpyAsync(dst[i], src[i] + r0 * esz[i], rows * esz[i], cudaMemcpyHostToDevice, ctx->copy_stream));
        }
        RJ_CUDA(cudaEventRecord(ctx->copied[b], ctx->copy_stream));
        RJ_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->copied[b], 0));
        PointArgs pc = pa;
        pc.xy = (const float2*)dst[0];
        pc.n = rows;
        for (int c = 0; c < f.ncol; ++c) pc.f.col[c] = (const uint32_t*)dst[cslot[c]];
        if (aslot >= 0) pc.f.aggr_col = (const uint32_t*)dst[aslot];
        launch(pc);
        RJ_CUDA(cudaEventRecord(ctx->consumed[b], ctx->stream));
    }
    RJ_CUDA(cudaEventRecord(ctx->copy_t1, ctx->copy_stream));
    ctx->passes = std::max(passes, 1);
    RJ_CUDA(cudaGetLastError());
    return RJ_OK;
}

CanvasXf make_canvas_xf(rj_ctx* ctx, const RasterPlan& rp, const float4* dcol, const float4* drow) {
    CanvasXf cx{};
    cx.colxf = dcol;
    cx.rowxf = drow;
    cx.splitx = rp.splitx;
    cx.splity = rp.splity;
    cx.resx = rp.resx;
    cx.resy = rp.resy;
    cx.lbx = (float)ctx->ps->bbox[0];
    cx.lby = (float)ctx->ps->bbox[1];
    cx.tdx = rp.colxf[0].w;
    cx.tdy = rp.rowxf[0].w;
    cx.col0 = rp.colxf[0];
    cx.row0 = rp.rowxf[0];
    return cx;
}

// ---------------------------------------------------------------------------
// Join operators.  Each fills out_count / out_sum (and out_bounds) on device.
struct ExecState {
    unsigned long long* out_count;
    unsigned long long* out_sum;
    long long* out_bounds;
    Phase* ph;
    int passes = 1;
};

int poly_pass(rj_ctx* ctx, int mode, PolyPassArgs& a, const TierArgs* tier = nullptr) {
    unsigned int* ctr;
    int rc;
    const int TP = a.T * a.P;
    int4* info_a;
    int2* info_b;
    int *nbands, *band_start, *tmp;
    if ((rc = scratch_t(ctx, "work_ctr", 1, &ctr))) return rc;
    if ((rc = scratch_t(ctx, "pp_info_a", TP, &info_a))) return rc;
    if ((rc = scratch_t(ctx, "pp_info_b", TP, &info_b))) return rc;
    if ((rc = scratch_t(ctx, "pp_nbands", TP, &nbands))) return rc;
    if ((rc = scratch_t(ctx, "pp_band_start", (size_t)TP + 1, &band_start))) return rc;
    if ((rc = scratch_t(ctx, "pp_tmp", (size_t)scan_tmp_ints(TP), &tmp))) return rc;
    RJ_CUDA(cudaMemsetAsync(ctr, 0, sizeof(unsigned), ctx->stream));
    a.work_ctr = ctr;
    a.info_a = info_a;
    a.info_b = info_b;
    a.nbands = nbands;
    a.band_start = band_start;
    launch_poly_info(mode, a, ctx->sms, ctx->stream);
    if (!launch_exclusive_scan(nbands, band_start, TP, tmp, ctx->stream))
        return fail(ctx, RJ_E_INVALID, "too many (tile, polygon) items");
    if (tier) launch_tier_pass(mode, a, *tier, ctx->sms, ctx->stream);
    else launch_poly_pass(mode, a, ctx->sms, ctx->stream);
    RJ_CUDA(cudaGetLastError());
    return RJ_OK;
}

// Tiered canvas of a large raster canvas: classification of 16 x 16 blocks,
// then the label form (disjoint coverage) or the canvas form.  Results equal
// the flat canvas's; polygon-side work follows the perimeters.
int tier_lean_pass(rj_ctx* ctx, const DevFilter& f, const RasterPlan& rp, const CanvasXf& cx, const TierArgs& tr,
                   bool label, size_t nblk, size_t spx, ExecState& es, bool* done);   // below

int exec_raster_tier(rj_ctx* ctx, const rj_query* q, const RasterPlan& rp, const DevFilter& f, ExecState& es,
                     PolyPassArgs& a, const CanvasXf& cx, uint64_t ckey, bool bounds) {
    int rc;
    TierArgs tr{};
    tr.bw = (rp.resx + 15) / 16;
    tr.bh = (rp.resy + 15) / 16;
    const size_t nblk = (size_t)a.T * tr.bw * tr.bh;
    if (nblk >= (size_t)1 << 24) return fail(ctx, RJ_E_UNSUPPORTED, "canvas too large for the tiered form");
    int* slot;
    int* tmp;
    unsigned long long* cnt;   // multi blocks, covered pixel writes, labelled pixels
    if ((rc = scratch_t(ctx, "tier_full", nblk, &tr.full))) return rc;
    if ((rc = scratch_t(ctx, "tier_mixed", nblk, &tr.mixed))) return rc;
    if ((rc = scratch_t(ctx, "tier_slot", nblk + 1, &slot))) return rc;
    if ((rc = scratch_t(ctx, "tier_code", nblk, &tr.code))) return rc;
    if ((rc = scratch_t(ctx, "tier_tmp", (size_t)scan_tmp_ints((int)nblk), &tmp))) return rc;
    if ((rc = scratch_t(ctx, "tier_cnt", 3, &cnt))) return rc;
    tr.slot = slot;
    // error bounds: the blocks the outline pass reads are mixed too
    tr.outline = bounds ? 1 : 0;
    RJ_CUDA(cudaMemsetAsync(tr.full, 0xFF, nblk * 4, ctx->stream));
    RJ_CUDA(cudaMemsetAsync(tr.mixed, 0, nblk * 4, ctx->stream));
    RJ_CUDA(cudaMemsetAsync(cnt, 0, 3 * 8, ctx->stream));
    a.outline_rows = tr.outline;
    rc = poly_pass(ctx, MODE_TIER_CLASSIFY, a, &tr);
    a.outline_rows = 0;
    if (rc) return rc;
    if (!launch_exclusive_scan((const int*)tr.mixed, slot, (int)nblk, tmp, ctx->stream))
        return fail(ctx, RJ_E_INVALID, "tier scan failed");
    launch_tier_codes(tr, nblk, cnt, ctx->sms, ctx->stream);
    int nslots = 0;
    if ((rc = readback_guard(ctx, "the tiered canvas"))) return rc;
    RJ_CUDA(cudaMemcpyAsync(&nslots, slot + nblk, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    RJ_CUDA(cudaStreamSynchronize(ctx->stream));
    const size_t spx = (size_t)std::max(nslots, 1) * 256;
    bool label = !bounds && !(q->flags & RJ_FLAG_FORCE_CANVAS) && ctx->ps->overlap_on(ckey) != 1 &&
                 ctx->ps->P <= kMaxLabelPolys;
    if (label) {
        if ((rc = scratch_t(ctx, "tier_plabel", spx, &tr.plabel))) return rc;
        RJ_CUDA(cudaMemsetAsync(tr.plabel, 0xFF, spx * 2, ctx->stream));
        a.covered = cnt + 1;
        if ((rc = poly_pass(ctx, MODE_TIER_LABEL, a, &tr))) return rc;
        if (ctx->ps->overlap_on(ckey) == -1) {
            launch_tier_nonempty(tr.plabel, (size_t)nslots * 256, cnt + 2, ctx->sms, ctx->stream);
            unsigned long long hc[3] = {0, 0, 0};
            RJ_CUDA(cudaMemcpyAsync(hc, cnt, sizeof hc, cudaMemcpyDeviceToHost, ctx->stream));
            RJ_CUDA(cudaStreamSynchronize(ctx->stream));
            ctx->ps->overlap[ckey] = (hc[0] != 0 || hc[1] != hc[2]) ? 1 : 0;
        }
        label = ctx->ps->overlap_on(ckey) == 0;
    }
    es.ph->mark(2);
    if (label) {
        bool lean = false;
        if ((rc = tier_lean_pass(ctx, f, rp, cx, tr, true, nblk, spx, es, &lean))) return rc;
        if (!lean && (rc = point_pass(ctx, f, es.out_count, es.out_sum, [&](const PointArgs& pa) {
                          launch_tier_label_points(pa, cx, tr, ctx->sms, ctx->stream);
                      })))
            return rc;
        es.ph->mark(3);
        es.ph->mark(4);
        return RJ_OK;
    }
    // canvas form: block sums + pixel canvases of the mixed blocks
    if ((rc = scratch_t(ctx, "tier_bcnt", nblk, &tr.bcnt))) return rc;
    if ((rc = scratch_t(ctx, "tier_pcnt", spx, &tr.pcnt))) return rc;
    RJ_CUDA(cudaMemsetAsync(tr.bcnt, 0, nblk * 4, ctx->stream));
    RJ_CUDA(cudaMemsetAsync(tr.pcnt, 0, spx * 4, ctx->stream));
    if (f.aggr) {
        if ((rc = scratch_t(ctx, "tier_bsum", nblk, &tr.bsum))) return rc;
        if ((rc = scratch_t(ctx, "tier_psum", spx, &tr.psum))) return rc;
        RJ_CUDA(cudaMemsetAsync(tr.bsum, 0, nblk * 8, ctx->stream));
        RJ_CUDA(cudaMemsetAsync(tr.psum, 0, spx * 8, ctx->stream));
    }
    bool lean = false;
    if ((rc = tier_lean_pass(ctx, f, rp, cx, tr, false, nblk, spx, es, &lean))) return rc;
    if (!lean && (rc = point_pass(ctx, f, es.out_count, es.out_sum, [&](const PointArgs& pa) {
                      launch_tier_splat_points(pa, cx, tr, ctx->sms, ctx->stream);
                  })))
        return rc;
    es.ph->mark(3);
    a.canvas_c = nullptr;
    a.canvas_s = nullptr;
    a.label = nullptr;
    if ((rc = poly_pass(ctx, MODE_TIER_REDUCE, a, &tr))) return rc;
    if (bounds) {
        // the outline pass of the error bounds over the mixed blocks' counts
        a.tier_code = tr.code;
        a.tier_pcnt = tr.pcnt;
        a.tier_bw = tr.bw;
        a.tier_bh = tr.bh;
        a.err = ctx->d_err;
        rc = poly_pass(ctx, MODE_BOUNDS, a);
        a.tier_code = nullptr;
        a.tier_pcnt = nullptr;
        if (rc) return rc;
    }
    es.ph->mark(4);
    return RJ_OK;
}

// Polygon label map of a canvas (MODE_LABEL).  Returns 1 in *overlap when
// some pixel centre lies in two polygons (the label map cannot represent the
// set; the canvas path is used instead).
int label_map(rj_ctx* ctx, PolyPassArgs& a, const char* key, size_t npix, const uint32_t* mask, int words,
              uint64_t canvas, uint16_t** out, int* overlap) {
    int rc;
    uint16_t* label;
    unsigned long long* cnt;
    if ((rc = scratch_t(ctx, key, npix, &label))) return rc;
    if ((rc = scratch_t(ctx, "label_counts", 2, &cnt))) return rc;
    RJ_CUDA(cudaMemsetAsync(label, 0xFF, npix * sizeof(uint16_t), ctx->stream));
    RJ_CUDA(cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), ctx->stream));
    a.label = label;
    a.covered = cnt;
    if ((rc = poly_pass(ctx, MODE_LABEL, a))) return rc;
    launch_label_finish(label, mask, a.resx, a.resy, a.T, words, cnt + 1, ctx->sms, ctx->stream);
    RJ_CUDA(cudaGetLastError());
    // The first label map of a polygon set decides whether its coverage
    // overlaps (every covered pixel centre counted once per polygon vs the
    // labelled pixels); the answer is kept with the set.
    if (ctx->ps->overlap_on(canvas) == -1) {
        if ((rc = readback_guard(ctx, "the first label map of a polygon set on a canvas"))) return rc;
        unsigned long long lc[2] = {0, 0};
        RJ_CUDA(cudaMemcpyAsync(lc, cnt, sizeof lc, cudaMemcpyDeviceToHost, ctx->stream));
        RJ_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->ps->overlap[canvas] = (lc[0] != lc[1]) ? 1 : 0;
    }
    *overlap = ctx->ps->overlap_on(canvas) == 1 ? 1 : 0;
    *out = label;
    a.label = nullptr;
    return RJ_OK;
}

// The lean passes' autotuner keys a choice by query class: the form, and
// the polygon count, canvas size and table size in octave buckets.  Scans
// below kTuneMinPoints take the default shape without timing anything.
constexpr uint64_t kTuneMinPoints = 1ull << 22;
constexpr int kCountDefaultShape = 5;     // 1024 threads, 4 pairs, block codes, per-warp histograms
inline int tune_bucket(double v) { return (int)std::floor(std::log2(std::max(v, 1.0))); }

// Filters and aggregate of a query in the lean passes' form (interval
// predicates on value pairs); false when a column is not 8-byte aligned.
bool lean_cols_of(const PointArgs& pa, unsigned long long* out_sum, LeanCols& lc) {
    lc = LeanCols{};
    lc.ncol = pa.f.ncol;
    for (int c = 0; c < lc.ncol; ++c) {
        if (((uintptr_t)pa.f.col[c] & 7) != 0) return false;
        lc.col[c] = reinterpret_cast<const uint2*>(pa.f.col[c]);
        lc.lo[c] = pa.f.lo[c];
        lc.span[c] = pa.f.span[c];
        const int t = pa.f.ctyp[c];
        lc.fm[c] = (t == RJ_FLOAT) ? 0x7FFFFFFFu : 0u;
        lc.xm[c] = (t == RJ_FLOAT || t == RJ_INT) ? 0x80000000u : 0u;
    }
    lc.aggr = pa.f.aggr ? 1 : 0;
    if (lc.aggr) {
        lc.aggr_ci = pa.f.aggr_ci;
        if (lc.aggr_ci < 0) {
            if (((uintptr_t)pa.f.aggr_col & 7) != 0) return false;
            lc.aggr_col = reinterpret_cast<const uint2*>(pa.f.aggr_col);
        }
        lc.aggr_typ = pa.f.aggr_typ;
        lc.scale = pa.f.sum_scale;
        lc.nonfinite = pa.out_nonfinite;
        lc.out_sum = out_sum;
    }
    return true;
}

// Autotuned choices per device and query class, shared by every context of
// the process: a choice depends on the GPU and the class, not on the context.
std::mutex g_tune_mu;
std::map<std::string, int> g_tuned;
bool tuned_get(const rj_ctx* ctx, const std::string& key, int* v) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tuned.find(std::to_string(ctx->device) + "/" + key);
    if (it == g_tuned.end()) return false;
    *v = it->second;
    return true;
}
void tuned_put(const rj_ctx* ctx, const std::string& key, int v) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned[std::to_string(ctx->device) + "/" + key] = v;
}

// The autotuner of the lean passes: the candidate kept for `key`, else each
// candidate timed once by `timed(i)` (CUDA events on the context's stream;
// returns false when it cannot run), the fastest kept.  Returns the index,
// or -1 when none ran.
template <class Timed>
int tune_pick(rj_ctx* ctx, const std::string& key, size_t ncand, Timed&& timed) {
    if (ncand == 1) return 0;
    int known = 0;
    if (tuned_get(ctx, key, &known)) return std::min<int>(known, (int)ncand - 1);
    if (ctx->capturing) return -1;   // nothing is timed inside a capture
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return -1;
    float best = 1e30f;
    int besti = -1;
    for (size_t i = 0; i < ncand; ++i) {
        cudaEventRecord(e0, ctx->stream);
        if (!timed(i)) continue;
        cudaEventRecord(e1, ctx->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            besti = (int)i;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (besti >= 0) tuned_put(ctx, key, besti);
    return besti;
}

// Lean label pass (rj_count_kernels.cu for a plain count, rj_lean_kernels.cu
// with interval-form filters on up to four columns and / or a summed
// aggregate): one canvas tile, a resident table.  Builds the block-code
// map(s) of the label map and runs the pass; the shape and block size are the
// ones forced with rj_set_tuning, else autotuned: on the first query of its
// class (form, polygons, canvas, table size) on this context every candidate
// is timed once on the table itself, into scratch outputs, and the fastest is
// kept.  *done = false: the pass does not apply (the caller takes the generic
// label pass).
int label_count_pass(rj_ctx* ctx, const DevFilter& f, const RasterPlan& rp, const uint16_t* label, ExecState& es,
                     bool* done) {
    *done = false;
    ctx->last_count_shape = ctx->last_count_bshift = -1;
    if (rp.splitx != 1 || rp.splity != 1 || ctx->streamed) return RJ_OK;
    if (f.general || f.ncol > label_lean_max_cols()) return RJ_OK;
    const bool plain = f.ncol == 0 && !f.aggr;
    PointArgs pa = make_point_args(ctx, f, es.out_count, es.out_sum);
    if (((uintptr_t)pa.xy & 15) != 0) return RJ_OK;
    LeanCols lc{};
    if (!plain && !lean_cols_of(pa, es.out_sum, lc)) return RJ_OK;
    const int P = ctx->ps->P;
    LabelCountArgs a{};
    a.xy = reinterpret_cast<const float4*>(pa.xy);
    a.n = pa.n;
    a.col0 = rp.colxf[0];
    a.row0 = rp.rowxf[0];
    a.resx = rp.resx;
    a.resy = rp.resy;
    a.label = label;
    a.P = P;
    a.out_count = es.out_count;
    a.zones = pa.zones;
    a.zrow0 = pa.row0;
    a.qbox = pa.qbox;
    auto code_words = [&](int bs) {
        const long long nbx = ((long long)rp.resx + (1 << bs) - 1) >> bs, nby = ((long long)rp.resy + (1 << bs) - 1) >> bs;
        return (nbx * nby + 1) / 2;
    };
    // candidate block sizes: the smallest whose code map leaves room in
    // shared memory for the histograms, and the next one
    int bs0 = 4;
    while (bs0 < 8 && code_words(bs0) * 4 + (long long)P * 12 > 160 * 1024) ++bs0;
    std::vector<int> bss;
    if (ctx->count_bshift >= 4 && ctx->count_bshift <= 8) bss.push_back(ctx->count_bshift);
    else {
        bss.push_back(bs0);
        if (bs0 < 8) bss.push_back(bs0 + 1);
    }
    const int nshapes = plain ? label_count_shapes() : label_lean_shapes();
    auto smem_of = [&](int sh, int bs) {
        return plain ? label_count_smem(sh, (int)code_words(bs), P)
                     : label_lean_smem(sh, (int)code_words(bs), P, lc.aggr != 0);
    };
    std::vector<std::pair<int, int>> cands;   // (shape, bs)
    for (int bs : bss)
        for (int sh = 0; sh < nshapes; ++sh)
            if (ctx->count_shape < 0 || ctx->count_shape == sh)
                if (smem_of(sh, bs) > 0 && smem_of(sh, bs) <= 200 * 1024) cands.push_back({sh, bs});
    if (cands.empty()) return RJ_OK;
    int rc;
    char tkey[200];
    std::snprintf(tkey, sizeof tkey, "lean:%d:%d:%d:%d:%d:%d:%d:%d:%d", plain ? 0 : 1, lc.ncol, lc.aggr, lc.aggr_ci >= 0,
                  tune_bucket((double)P), tune_bucket((double)rp.resx * rp.resy), tune_bucket((double)a.n),
                  ctx->count_shape, ctx->count_bshift);
    int tuned_i = -1;
    const bool have = tuned_get(ctx, tkey, &tuned_i);
    // small scans are not worth timing candidates for: the default shape
    const bool small = a.n < kTuneMinPoints;
    const bool known = cands.size() == 1 || have || small || ctx->capturing;
    std::pair<int, int> pick = cands[0];
    if (cands.size() > 1 && have)
        pick = cands[std::min<size_t>((size_t)tuned_i, cands.size() - 1)];
    else if (small)
        for (const auto& c : cands)
            if (c.first == (plain ? kCountDefaultShape : 0) && c.second == bss.back()) pick = c;
    // code maps: the chosen block size only, or every candidate's for the tuner
    std::map<int, uint16_t*> codes;
    for (int bs : bss) {
        if (known && bs != pick.second) continue;
        const int nbx = (rp.resx + (1 << bs) - 1) >> bs, nby = (rp.resy + (1 << bs) - 1) >> bs;
        uint16_t* c;
        char key[32];
        std::snprintf(key, sizeof key, "label_codes%d", bs);
        if ((rc = scratch_t(ctx, key, (size_t)code_words(bs) * 2, &c))) return rc;
        launch_block_codes(label, rp.resx, rp.resy, bs, nbx, nby, c, ctx->sms, ctx->stream);
        codes[bs] = c;
    }
    es.ph->mark(2);   // the code maps belong to the polygon side
    auto args_for = [&](int bs) {
        LabelCountArgs b = a;
        b.bs = bs;
        b.nbx = (rp.resx + (1 << bs) - 1) >> bs;
        b.codes = codes[bs];
        b.code_words = (int)code_words(bs);
        return b;
    };
    auto launch = [&](int sh, const LabelCountArgs& b, const LeanCols& l) {
        return plain ? launch_label_count(sh, b, ctx->sms, ctx->stream)
                     : launch_label_lean(sh, b, l, ctx->sms, ctx->stream);
    };
    if (!known) {
        // time each candidate once on (a prefix of) the table, into scratch outputs
        unsigned long long *tout, *tsum;
        double* tnf;
        if ((rc = scratch_t(ctx, "tune_count", (size_t)P, &tout))) return rc;
        if ((rc = scratch_t(ctx, "tune_sum", (size_t)P, &tsum))) return rc;
        if ((rc = scratch_t(ctx, "tune_nonfinite", (size_t)P, &tnf))) return rc;
        LeanCols tl = lc;
        tl.out_sum = tsum;
        tl.nonfinite = tnf;
        const uint64_t tn = std::min<uint64_t>(a.n & ~1ULL, 1ULL << 28);
        cudaEvent_t e0, e1;
        RJ_CUDA(cudaEventCreate(&e0));
        RJ_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        int besti = -1;
        for (size_t i = 0; i < cands.size(); ++i) {
            LabelCountArgs b = args_for(cands[i].second);
            b.out_count = tout;
            // first launch of a shape loads it: a tiny warm-up launch
            LabelCountArgs w = b;
            w.n = std::min<uint64_t>(b.n & ~1ULL, 1ULL << 16);
            if (!launch(cands[i].first, w, tl)) continue;
            b.n = tn;
            RJ_CUDA(cudaEventRecord(e0, ctx->stream));
            launch(cands[i].first, b, tl);
            RJ_CUDA(cudaEventRecord(e1, ctx->stream));
            RJ_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            RJ_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                besti = (int)i;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        RJ_CUDA(cudaGetLastError());
        if (besti < 0) return RJ_OK;
        tuned_put(ctx, tkey, besti);
        pick = cands[(size_t)besti];
    }
    ctx->passes = 1;
    ctx->copy_ms = 0;
    if (!launch(pick.first, args_for(pick.second), lc)) return RJ_OK;
    RJ_CUDA(cudaGetLastError());
    ctx->last_count_shape = pick.first;
    ctx->last_count_bshift = pick.second;
    *done = true;
    return RJ_OK;
}

// Lean point pass of the hybrid join over its label map (rj_hybrid_lean.cu):
// a resident table, interval-form filters on at most four columns, count or
// sum.  Shapes and block sizes as for the lean raster pass (forced with
// rj_set_tuning, else autotuned per query class).  *done = false: the pass
// does not apply (the caller takes the generic hybrid pass).
// mode 0: the hybrid canvas h with its label map; mode 1: the classified
// grid ix with its cell labels (index join).
int hybrid_lean_pass(rj_ctx* ctx, const DevFilter& f, int mode, const HybXf& h, const uint16_t* label,
                     const ExactIndex& ix, ExecState& es, bool* done) {
    *done = false;
    ctx->last_count_shape = ctx->last_count_bshift = -1;
    if (ctx->streamed || f.general || f.ncol > label_lean_max_cols()) return RJ_OK;
    PointArgs pa = make_point_args(ctx, f, es.out_count, es.out_sum);
    if (((uintptr_t)pa.xy & 15) != 0) return RJ_OK;
    LeanCols lc;
    if (!lean_cols_of(pa, es.out_sum, lc)) return RJ_OK;
    const int P = ctx->ps->P;
    HybLeanArgs a{};
    a.xy = reinterpret_cast<const float4*>(pa.xy);
    a.n = pa.n;
    a.h = h;
    a.label = label;
    a.P = P;
    a.out_count = es.out_count;
    a.zones = pa.zones;
    a.zrow0 = pa.row0;
    a.qbox = pa.qbox;
    a.ix = ix;
    a.mode = mode;
    const int resx = mode == 0 ? h.resx : ix.res, resy = mode == 0 ? h.resy : ix.res;
    if (mode == 0) {
        // pixel coordinate = (u + 1) / 2 * res with u = (v - o) / d
        const double ax = (double)h.resx / (2.0 * h.dx), ay = (double)h.resy / (2.0 * h.dy);
        a.fast = make_float4((float)ax, (float)(0.5 * h.resx - ax * h.ox), (float)ay, (float)(0.5 * h.resy - ay * h.oy));
    }
    auto code_words = [&](int bs) {
        const long long nbx = ((long long)resx + (1 << bs) - 1) >> bs, nby = ((long long)resy + (1 << bs) - 1) >> bs;
        return (nbx * nby + 1) / 2;
    };
    int bs0 = mode == 0 ? 4 : 3;
    while (bs0 < 8 && code_words(bs0) * 4 > 64 * 1024) ++bs0;
    std::vector<int> bss;
    if (ctx->count_bshift >= 4 && ctx->count_bshift <= 8) bss.push_back(ctx->count_bshift);
    else {
        bss.push_back(bs0);
        if (bs0 < 8) bss.push_back(bs0 + 1);
    }
    std::vector<std::pair<int, int>> cands;
    for (int bs : bss)
        for (int sh = 0; sh < hybrid_lean_shapes(); ++sh)
            if (ctx->count_shape < 0 || ctx->count_shape == sh) {
                const size_t sm = hybrid_lean_smem(sh, (int)code_words(bs), P, lc.aggr != 0);
                if (sm > 0 && sm <= 200 * 1024) cands.push_back({sh, bs});
            }
    if (cands.empty()) return RJ_OK;
    char key[200];
    std::snprintf(key, sizeof key, "hyb:%d:%d:%d:%d:%d:%d:%d:%d:%d", mode, lc.ncol, lc.aggr, lc.aggr_ci >= 0,
                  tune_bucket((double)P), tune_bucket((double)resx * resy), tune_bucket((double)a.n), ctx->count_shape,
                  ctx->count_bshift);
    int tuned_i = -1;
    const bool have = tuned_get(ctx, key, &tuned_i);
    const bool small = a.n < kTuneMinPoints;
    const bool known = cands.size() == 1 || have || small;
    int rc;
    std::map<int, uint16_t*> codes;
    for (int bs : bss) {
        if (known && bs != cands[have ? std::min<size_t>((size_t)tuned_i, cands.size() - 1) : 0].second)
            continue;   // (a small scan takes the first candidate)
        const int nbx = (resx + (1 << bs) - 1) >> bs, nby = (resy + (1 << bs) - 1) >> bs;
        uint16_t* c;
        char ck[32];
        std::snprintf(ck, sizeof ck, "hyb_codes%d_%d", mode, bs);
        if ((rc = scratch_t(ctx, ck, (size_t)code_words(bs) * 2, &c))) return rc;
        launch_block_codes(label, resx, resy, bs, nbx, nby, c, ctx->sms, ctx->stream);
        codes[bs] = c;
    }
    es.ph->mark(2);   // the code maps belong to the polygon side
    auto args_for = [&](int bs) {
        HybLeanArgs b = a;
        b.bs = bs;
        b.nbx = (resx + (1 << bs) - 1) >> bs;
        b.codes = codes[bs];
        b.code_words = (int)code_words(bs);
        return b;
    };
    unsigned long long *tout = nullptr, *tsum = nullptr;
    double* tnf = nullptr;
    if (!known) {
        if ((rc = scratch_t(ctx, "tune_count", (size_t)P, &tout))) return rc;
        if ((rc = scratch_t(ctx, "tune_sum", (size_t)P, &tsum))) return rc;
        if ((rc = scratch_t(ctx, "tune_nonfinite", (size_t)P, &tnf))) return rc;
    }
    LeanCols tl = lc;
    tl.out_sum = tsum;
    tl.nonfinite = tnf;
    const int pi = small && !have ? 0 : tune_pick(ctx, key, cands.size(), [&](size_t i) {
        HybLeanArgs b = args_for(cands[i].second);
        b.out_count = tout;
        HybLeanArgs w = b;
        w.n = std::min<uint64_t>(b.n & ~1ULL, 1ULL << 16);   // first launch of a shape loads it
        if (!launch_hybrid_lean(cands[i].first, w, tl, ctx->sms, ctx->stream)) return false;
        b.n = std::min<uint64_t>(a.n & ~1ULL, 1ULL << 27);
        return launch_hybrid_lean(cands[i].first, b, tl, ctx->sms, ctx->stream);
    });
    RJ_CUDA(cudaGetLastError());
    if (pi < 0) return RJ_OK;
    const std::pair<int, int> pick = cands[(size_t)pi];
    ctx->passes = 1;
    ctx->copy_ms = 0;
    if (!launch_hybrid_lean(pick.first, args_for(pick.second), lc, ctx->sms, ctx->stream)) return RJ_OK;
    RJ_CUDA(cudaGetLastError());
    ctx->last_count_shape = pick.first;
    ctx->last_count_bshift = pick.second;
    *done = true;
    return RJ_OK;
}

// Lean point pass onto the point canvas (rj_splat_kernels.cu): one canvas
// tile, a resident table, interval-form filters on at most four columns,
// count or sum.  The shape (canvas copies in shared memory, or atomics
// straight into the canvas; block size) is the one forced with rj_set_tuning
// (RJ_TUNE_COUNT_SHAPE), else autotuned per query class.  Tuning runs write
// into the canvas, which is cleared again after them.  *done = false: the
// pass does not apply (the caller takes the generic splat).
int splat_lean_pass(rj_ctx* ctx, const DevFilter& f, const RasterPlan& rp, uint32_t* canvas_c, long long* canvas_s,
                    ExecState& es, bool* done) {
    *done = false;
    ctx->last_count_shape = ctx->last_count_bshift = -1;
    if (rp.splitx != 1 || rp.splity != 1 || ctx->streamed) return RJ_OK;
    if (f.general || f.ncol > label_lean_max_cols()) return RJ_OK;
    PointArgs pa = make_point_args(ctx, f, es.out_count, es.out_sum);
    if (((uintptr_t)pa.xy & 15) != 0) return RJ_OK;
    LeanCols lc{};
    if (!lean_cols_of(pa, es.out_sum, lc)) return RJ_OK;
    SplatLeanArgs a{};
    a.xy = reinterpret_cast<const float4*>(pa.xy);
    a.n = pa.n;
    a.col0 = rp.colxf[0];
    a.row0 = rp.rowxf[0];
    a.resx = rp.resx;
    a.resy = rp.resy;
    a.canvas_c = canvas_c;
    a.canvas_s = reinterpret_cast<unsigned long long*>(canvas_s);
    a.zones = pa.zones;
    a.zrow0 = pa.row0;
    a.qbox = pa.qbox;
    const size_t npix = (size_t)rp.resx * rp.resy;
    const bool agg = lc.aggr != 0;
    std::vector<int> cands;
    for (int sh = 0; sh < splat_lean_shapes(); ++sh)
        if (ctx->count_shape < 0 || ctx->count_shape == sh) {
            const size_t sm = splat_lean_smem(sh, npix, agg);
            if (sm > 0 && sm <= 200 * 1024) cands.push_back(sh);
        }
    if (cands.empty()) return RJ_OK;
    char key[200];
    std::snprintf(key, sizeof key, "splat:%d:%d:%d:%d:%d:%d", lc.ncol, lc.aggr, lc.aggr_ci >= 0,
                  tune_bucket((double)npix), tune_bucket((double)a.n), ctx->count_shape);
    int tuned_i = -1;
    const bool have = tuned_get(ctx, key, &tuned_i);
    const bool small = a.n < kTuneMinPoints;
    bool timed_any = false;
    const int pi = small && !have ? 0 : tune_pick(ctx, key, cands.size(), [&](size_t i) {
        timed_any = true;
        SplatLeanArgs w = a;
        w.n = std::min<uint64_t>(a.n & ~1ULL, 1ULL << 16);   // first launch of a shape loads it
        if (!launch_splat_lean(cands[i], w, lc, ctx->sms, ctx->stream)) return false;
        SplatLeanArgs b = a;
        b.n = std::min<uint64_t>(a.n & ~1ULL, 1ULL << 27);
        return launch_splat_lean(cands[i], b, lc, ctx->sms, ctx->stream);
    });
    RJ_CUDA(cudaGetLastError());
    if (timed_any) {
        RJ_CUDA(cudaMemsetAsync(canvas_c, 0, npix * sizeof(uint32_t), ctx->stream));
        if (canvas_s) RJ_CUDA(cudaMemsetAsync(canvas_s, 0, npix * sizeof(long long), ctx->stream));
    }
    if (pi < 0) return RJ_OK;
    ctx->passes = 1;
    ctx->copy_ms = 0;
    if (!launch_splat_lean(cands[(size_t)pi], a, lc, ctx->sms, ctx->stream)) return RJ_OK;
    RJ_CUDA(cudaGetLastError());
    ctx->last_count_shape = cands[(size_t)pi];
    *done = true;
    return RJ_OK;
}

// Lean point pass over the tiered canvas (rj_tier_lean.cu): a resident
// table, interval-form filters on at most four columns, count or sum; label
// form into the per-polygon outputs, canvas form into the block and slot
// sums.  Shapes forced with rj_set_tuning (RJ_TUNE_COUNT_SHAPE), else
// autotuned per query class; tuning runs of the canvas form write into its
// sums, which are cleared again after them.  *done = false: the pass does
// not apply (the caller takes the generic pass).
int tier_lean_pass(rj_ctx* ctx, const DevFilter& f, const RasterPlan& rp, const CanvasXf& cx, const TierArgs& tr,
                   bool label, size_t nblk, size_t spx, ExecState& es, bool* done) {
    *done = false;
    ctx->last_count_shape = ctx->last_count_bshift = -1;
    if (ctx->streamed || f.general || f.ncol > label_lean_max_cols()) return RJ_OK;
    PointArgs pa = make_point_args(ctx, f, es.out_count, es.out_sum);
    if (((uintptr_t)pa.xy & 15) != 0) return RJ_OK;
    LeanCols lc{};
    if (!lean_cols_of(pa, es.out_sum, lc)) return RJ_OK;
    TierLeanArgs a{};
    a.xy = reinterpret_cast<const float4*>(pa.xy);
    a.n = pa.n;
    a.colxf = cx.colxf;
    a.rowxf = cx.rowxf;
    a.splitx = rp.splitx;
    a.splity = rp.splity;
    a.resx = rp.resx;
    a.resy = rp.resy;
    a.lbx = cx.lbx;
    a.lby = cx.lby;
    a.inv_tdx = (float)(1.0 / (double)cx.tdx);
    a.inv_tdy = (float)(1.0 / (double)cx.tdy);
    a.tr = tr;
    a.P = ctx->ps->P;
    a.out_count = es.out_count;
    a.zones = pa.zones;
    a.zrow0 = pa.row0;
    a.qbox = pa.qbox;
    const bool agg = lc.aggr != 0;
    std::vector<int> cands;
    for (int sh = 0; sh < tier_lean_shapes(); ++sh)
        if (ctx->count_shape < 0 || ctx->count_shape == sh) cands.push_back(sh);
    if (cands.empty() || tier_lean_smem(label, a.P, agg) > 200 * 1024) return RJ_OK;
    char key[200];
    std::snprintf(key, sizeof key, "tier:%d:%d:%d:%d:%d:%d:%d:%d:%d", label ? 1 : 0, lc.ncol, lc.aggr,
                  lc.aggr_ci >= 0, rp.splitx * rp.splity, tune_bucket((double)a.P), tune_bucket((double)nblk),
                  tune_bucket((double)a.n), ctx->count_shape);
    int tuned_i = -1;
    const bool have = tuned_get(ctx, key, &tuned_i);
    const bool small = a.n < kTuneMinPoints;
    int rc;
    unsigned long long *tout = nullptr, *tsum = nullptr;
    double* tnf = nullptr;
    if (!have && !small && label) {
        if ((rc = scratch_t(ctx, "tune_count", (size_t)a.P, &tout))) return rc;
        if ((rc = scratch_t(ctx, "tune_sum", (size_t)a.P, &tsum))) return rc;
        if ((rc = scratch_t(ctx, "tune_nonfinite", (size_t)a.P, &tnf))) return rc;
    }
    bool timed_any = false;
    const int pi = small && !have ? 0 : tune_pick(ctx, key, cands.size(), [&](size_t i) {
        timed_any = true;
        TierLeanArgs b = a;
        LeanCols tl = lc;
        if (label) {
            b.out_count = tout;
            tl.out_sum = tsum;
            tl.nonfinite = tnf;
        }
        TierLeanArgs w = b;
        w.n = std::min<uint64_t>(a.n & ~1ULL, 1ULL << 16);   // first launch of a shape loads it
        if (!launch_tier_lean(cands[i], label, w, tl, ctx->sms, ctx->stream)) return false;
        b.n = std::min<uint64_t>(a.n & ~1ULL, 1ULL << 27);
        return launch_tier_lean(cands[i], label, b, tl, ctx->sms, ctx->stream);
    });
    RJ_CUDA(cudaGetLastError());
    if (timed_any && !label) {
        RJ_CUDA(cudaMemsetAsync(tr.bcnt, 0, nblk * 4, ctx->stream));
        RJ_CUDA(cudaMemsetAsync(tr.pcnt, 0, spx * 4, ctx->stream));
        if (tr.bsum) RJ_CUDA(cudaMemsetAsync(tr.bsum, 0, nblk * 8, ctx->stream));
        if (tr.psum) RJ_CUDA(cudaMemsetAsync(tr.psum, 0, spx * 8, ctx->stream));
    }
    if (pi < 0) return RJ_OK;
    ctx->passes = 1;
    ctx->copy_ms = 0;
    if (!launch_tier_lean(cands[(size_t)pi], label, a, lc, ctx->sms, ctx->stream)) return RJ_OK;
    RJ_CUDA(cudaGetLastError());
    ctx->last_count_shape = cands[(size_t)pi];
    *done = true;
    return RJ_OK;
}

// Raster join (RasterJoin::performJoin RasterJoin.cpp:196-243) and the
// error-bounds join (RasterJoinBounds::performJoin RasterJoinBounds.cpp:306-381).
int exec_raster(rj_ctx* ctx, const rj_query* q, ExecState& es, bool bounds) {
    int rc;
    RasterPlan rp;
    if ((rc = plan_raster(ctx, q, rp))) return rc;
    DevFilter f;
    if ((rc = build_filter(ctx, q, f, bounds))) return rc;   // bounds: count only (RasterJoinBounds.cpp:124)
    const int T = rp.splitx * rp.splity;
    const size_t tile_px = (size_t)rp.resx * rp.resy;
    const size_t npix = tile_px * T;
    {
        // canvas plus two pixels: locations outside reach no pixel of any tile
        const double* bb = ctx->ps->bbox;
        const double mx = 2.0 * (bb[2] - bb[0]) / rp.actual_x + 1e-3, my = 2.0 * (bb[3] - bb[1]) / rp.actual_y + 1e-3;
        ctx->qbox = make_float4((float)(bb[0] - mx), (float)(bb[1] - my), (float)(bb[2] + mx), (float)(bb[3] + my));
    }

    es.ph->mark(1);
    int2* wv;
    float2* wf;
    if ((rc = transform_vertices(ctx, rp.colxf, rp.rowxf, &wv, &wf, bounds))) return rc;
    const float4* dcol = (const float4*)scratch_buf(ctx, "colxf").p;
    const float4* drow = (const float4*)scratch_buf(ctx, "rowxf").p;
    CanvasXf cx = make_canvas_xf(ctx, rp, dcol, drow);

    PolyPassArgs a{};
    a.wv = wv;
    a.wf = wf;
    a.pindex = (const int*)ctx->ps->d_pindex.p;
    a.P = ctx->ps->P;
    a.V = ctx->ps->V;
    a.T = T;
    a.resx = rp.resx;
    a.resy = rp.resy;
    a.out_count = es.out_count;
    a.out_sum = es.out_sum;
    a.out_bounds = es.out_bounds;
    a.line_filter = (q->flags & RJ_FLAG_LINE_FILTER) ? 1 : 0;

    const uint64_t ckey = canvas_key(rp.colxf, rp.rowxf, rp.resx, rp.resy);
    const uint64_t rows = std::min(ctx->row1, ctx->npts) - std::min(ctx->row0, ctx->npts);
    if (query_tier(q->flags, npix, rows)) return exec_raster_tier(ctx, q, rp, f, es, a, cx, ckey, bounds);
    bool use_label = !bounds && !(q->flags & RJ_FLAG_FORCE_CANVAS) && ctx->ps->overlap_on(ckey) != 1 &&
                     ctx->ps->P <= kMaxLabelPolys;
    if (use_label) {
        uint16_t* label;
        int overlap = 0;
        if ((rc = label_map(ctx, a, "label", npix, nullptr, 0, ckey, &label, &overlap))) return rc;
        es.ph->mark(2);
        if (!overlap) {
            bool lean = false;
            if ((rc = label_count_pass(ctx, f, rp, label, es, &lean))) return rc;
            if (!lean && (rc = point_pass(ctx, f, es.out_count, es.out_sum, [&](const PointArgs& pa) {
                              launch_raster_label(pa, cx, label, ctx->sms, ctx->stream);
                          })))
                return rc;
            RJ_CUDA(cudaGetLastError());
            es.ph->mark(3);
            es.ph->mark(4);
            return RJ_OK;
        }
    } else {
        es.ph->mark(2);
    }
    // canvas path: point pass (additive splat) then polygon pass
    uint32_t* canvas_c;
    long long* canvas_s = nullptr;
    if ((rc = scratch_t(ctx, "canvas_c", npix, &canvas_c))) return rc;
    RJ_CUDA(cudaMemsetAsync(canvas_c, 0, npix * sizeof(uint32_t), ctx->stream));
    if (f.aggr) {
        if ((rc = scratch_t(ctx, "canvas_s", npix, &canvas_s))) return rc;
        RJ_CUDA(cudaMemsetAsync(canvas_s, 0, npix * sizeof(long long), ctx->stream));
    }
    bool lean = false;
    if ((rc = splat_lean_pass(ctx, f, rp, canvas_c, canvas_s, es, &lean))) return rc;
    if (!lean && (rc = point_pass(ctx, f, es.out_count, es.out_sum, [&](const PointArgs& pa) {
                      launch_raster_splat(pa, cx, canvas_c, canvas_s, ctx->sms, ctx->stream);
                  })))
        return rc;
    RJ_CUDA(cudaGetLastError());
    es.ph->mark(3);
    a.canvas_c = canvas_c;
    a.canvas_s = canvas_s;
    a.label = nullptr;
    if ((rc = poly_pass(ctx, bounds ? MODE_BOUNDS : MODE_REDUCE, a))) return rc;
    es.ph->mark(4);
    return RJ_OK;
}

// Index join (IndexJoin::performJoin IndexJoin.cpp:156-166).  Default: the
// classified grid; RJ_FLAG_NO_CELL_CLASSIFY / RJ_FLAG_COMPAT_INDEX_CLAMP: the
// plain candidate lists with the full crossing test per candidate.
// Locations that can lie inside a polygon of the set: its bounds plus a
// margin far above the fp32 rounding of the crossing test.
void exact_qbox(rj_ctx* ctx) {
    const double* bb = ctx->ps->bbox;
    const double m = 1e-4 * std::max(bb[2] - bb[0], bb[3] - bb[1]) + 1e-3;
    ctx->qbox = make_float4((float)(bb[0] - m), (float)(bb[1] - m), (float)(bb[2] + m), (float)(bb[3] + m));
}

// RJ_FLAG_COUNT_EDGE_TESTS: a zeroed device counter for the exact tests of
// this query (read back into rj_timings.edge_tests).
int edge_test_counter(rj_ctx* ctx, const rj_query* q, ExactIndex& ix) {
    ix.tests = nullptr;
    if (!(q->flags & RJ_FLAG_COUNT_EDGE_TESTS) || ctx->capturing) return RJ_OK;
    int rc;
    if ((rc = scratch_t(ctx, "edge_tests", 1, &ctx->edge_tests_dev))) return rc;
    RJ_CUDA(cudaMemsetAsync(ctx->edge_tests_dev, 0, sizeof(unsigned long long), ctx->stream));
    ix.tests = ctx->edge_tests_dev;
    return RJ_OK;
}

int exec_index(rj_ctx* ctx, const rj_query* q, ExecState& es) {
    int rc;
    exact_qbox(ctx);
    DevFilter f;
    if ((rc = build_filter(ctx, q, f, false))) return rc;
    if (q->grid_res <= 0 || q->grid_res > 8192) return fail(ctx, RJ_E_INVALID, "grid resolution %d out of range", q->grid_res);
    es.ph->mark(1);
    const bool plain = (q->flags & (RJ_FLAG_NO_CELL_CLASSIFY | RJ_FLAG_COMPAT_INDEX_CLAMP)) != 0;
    if (plain) {
        IndexArgs ia{};
        if ((rc = build_grid(ctx, q->grid_res, (q->flags & RJ_FLAG_COMPAT_INDEX_CLAMP) ? 1 : 0, ia))) return rc;
        es.ph->mark(2);
        if ((rc = point_pass(ctx, f, es.out_count, es.out_sum, [&](const PointArgs& pa) {
                 launch_index_points(pa, ia, ctx->sms, ctx->stream);
             })))
            return rc;
    } else {
        ExactIndex ix{};
        if ((rc = build_exact(ctx, q->grid_res, ix))) return rc;
        if ((rc = edge_test_counter(ctx, q, ix))) return rc;
        es.ph->mark(2);
        // the lean pass over the grid's cell labels; else the generic pass
        bool lean = false;
        if (ctx->ps->P <= kMaxLabelPolys && !ctx->streamed) {
            uint16_t* cl;
            const int ncells = ix.res * ix.res;
            if ((rc = scratch_t(ctx, "cls_label16", (size_t)ncells, &cl))) return rc;
            launch_cell_labels(ix.code, ncells, cl, ctx->sms, ctx->stream);
            if ((rc = hybrid_lean_pass(ctx, f, 1, HybXf{}, cl, ix, es, &lean))) return rc;
        }
        if (!lean && (rc = point_pass(ctx, f, es.out_count, es.out_sum, [&](const PointArgs& pa) {
                          launch_exact_points(pa, ix, ctx->sms, ctx->stream);
                      })))
            return rc;
    }
    RJ_CUDA(cudaGetLastError());
    es.ph->mark(3);
    es.ph->mark(4);
    return RJ_OK;
}

// Hybrid join (HybridJoin::performJoin HybridJoin.cpp:339-359): points on
// non-border pixels take the pixel's polygon (label map, or canvas + polygon
// pass for overlapping polygon sets); points near an outline take the exact
// test through the grid.
int exec_hybrid(rj_ctx* ctx, const rj_query* q, ExecState& es) {
    int rc;
    exact_qbox(ctx);
    DevFilter f;
    if ((rc = build_filter(ctx, q, f, false))) return rc;
    if (q->grid_res <= 0 || q->grid_res > 8192) return fail(ctx, RJ_E_INVALID, "grid resolution %d out of range", q->grid_res);
    es.ph->mark(1);
    ExactIndex ix{};
    // refinement of the query grid for the exact tests (RJ_TUNE_HYBRID_EXACT_SCALE)
    if ((rc = build_exact(ctx, q->grid_res, ix, ctx->hybrid_exact_scale))) return rc;
    if ((rc = edge_test_counter(ctx, q, ix))) return rc;

    // canvas: getResolution(bbox, fboSize) (HybridJoin.cpp:62-66, Utils.h:29-34)
    const double dx = ctx->ps->bbox[2] - ctx->ps->bbox[0], dy = ctx->ps->bbox[3] - ctx->ps->bbox[1];
    const int fbo = q->hybrid_canvas > 0 ? q->hybrid_canvas : 4096;
    const float cellf = (float)std::max(dx / fbo, dy / fbo);
    const int resx = std::max(1, (int)std::fabs(std::ceil(dx / cellf)));
    const int resy = std::max(1, (int)std::fabs(std::ceil(dy / cellf)));
    HybXf h{};
    {
        float lbx = (float)ctx->ps->bbox[0], lby = (float)ctx->ps->bbox[1];
        float rtx = (float)ctx->ps->bbox[2], rty = (float)ctx->ps->bbox[3];
        volatile float sx = rtx + lbx, sy = rty + lby, qx = rtx - lbx, qy = rty - lby;
        h.ox = sx / 2.0f;
        h.oy = sy / 2.0f;
        h.dx = qx / 2.0f;
        h.dy = qy / 2.0f;
        h.resx = resx;
        h.resy = resy;
    }
    // Border mask: conservative outline + dilation.  A pixel is safe when no
    // edge comes within `radius` pixels; the radius covers the fp32 error of
    // the crossing test expressed in pixels (isBorder's 3x3 for radius 1).
    const int words = (resx + 31) / 32;
    uint32_t *mraw, *mask;
    if ((rc = scratch_t(ctx, "hyb_mraw", (size_t)words * resy, &mraw))) return rc;
    if ((rc = scratch_t(ctx, "hyb_mask", (size_t)words * resy, &mask))) return rc;
    RJ_CUDA(cudaMemsetAsync(mraw, 0, (size_t)words * resy * 4, ctx->stream));
    const double pix_w = std::min(dx / resx, dy / resy);
    const double err_world = std::ldexp(1.0, -21) * (ctx->ps->max_abs_coord + 6.0 * std::max(ctx->ps->max_edge_dx, ctx->ps->max_edge_dy) + 1.0);
    const int radius = std::max(1, (int)std::ceil(err_world / pix_w + 0.05));
    if (radius > 31) return fail(ctx, RJ_E_UNSUPPORTED, "hybrid canvas too fine for fp32 coordinates (radius %d)", radius);
    launch_outline_mask((const float2*)ctx->ps->d_verts.p, (const int*)ctx->ps->d_pindex.p, ctx->ps->P,
                        (const int*)ctx->ps->d_edge_poly.p, ctx->ps->V, h, 0.05f, mraw, words, ctx->sms, ctx->stream);
    launch_dilate_mask(mraw, mask, resx, resy, words, radius, ctx->sms, ctx->stream);
    RJ_CUDA(cudaGetLastError());

    // polygon coverage of the hybrid canvas (getMVP(bbox), HybridJoin.cpp:63)
    std::vector<float4> colxf(1), rowxf(1);
    {
        double ox = (ctx->ps->bbox[2] + ctx->ps->bbox[0]) / 2, hx = (ctx->ps->bbox[2] - ctx->ps->bbox[0]) / 2;
        double oy = (ctx->ps->bbox[3] + ctx->ps->bbox[1]) / 2, hy = (ctx->ps->bbox[3] - ctx->ps->bbox[1]) / 2;
        float sx = (float)(1.0 / hx), sy = (float)(1.0 / hy);
        colxf[0] = make_float4(sx, sx * (float)(-ox), resx * 0.5f, (float)dx);
        rowxf[0] = make_float4(sy, sy * (float)(-oy), resy * 0.5f, (float)dy);
    }
    int2* wv;
    float2* wf;
    if ((rc = transform_vertices(ctx, colxf, rowxf, &wv, &wf, false))) return rc;
    PolyPassArgs a{};
    a.wv = wv;
    a.pindex = (const int*)ctx->ps->d_pindex.p;
    a.P = ctx->ps->P;
    a.V = ctx->ps->V;
    a.T = 1;
    a.resx = resx;
    a.resy = resy;
    a.out_count = es.out_count;
    a.out_sum = es.out_sum;
    const size_t npix = (size_t)resx * resy;

    HybridArgs ha{};
    ha.h = h;
    ha.border = mask;
    ha.words = words;
    const uint64_t ckey = canvas_key(colxf, rowxf, resx, resy);
    bool use_label = !(q->flags & RJ_FLAG_FORCE_CANVAS) && ctx->ps->overlap_on(ckey) != 1 && ctx->ps->P <= kMaxLabelPolys;
    if (use_label) {
        uint16_t* label;
        int overlap = 0;
        if ((rc = label_map(ctx, a, "hyb_label", npix, mask, words, ckey, &label, &overlap))) return rc;
        if (overlap) use_label = false;
        else ha.label = label;
    }
    es.ph->mark(2);
    if (use_label) {
        bool lean = false;
        if ((rc = hybrid_lean_pass(ctx, f, 0, h, ha.label, ix, es, &lean))) return rc;
        if (!lean && (rc = point_pass(ctx, f, es.out_count, es.out_sum, [&](const PointArgs& pa) {
                          launch_hybrid_points(pa, ix, ha, ctx->sms, ctx->stream);
                      })))
            return rc;
        RJ_CUDA(cudaGetLastError());
        es.ph->mark(3);
        es.ph->mark(4);
        return RJ_OK;
    }
    uint32_t* canvas_c;
    long long* canvas_s = nullptr;
    if ((rc = scratch_t(ctx, "hyb_canvas_c", npix, &canvas_c))) return rc;
    RJ_CUDA(cudaMemsetAsync(canvas_c, 0, npix * sizeof(uint32_t), ctx->stream));
    if (f.aggr) {
        if ((rc = scratch_t(ctx, "hyb_canvas_s", npix, &canvas_s))) return rc;
        RJ_CUDA(cudaMemsetAsync(canvas_s, 0, npix * sizeof(long long), ctx->stream));
    }
    ha.canvas_c = canvas_c;
    ha.canvas_s = canvas_s;
    ha.scale = f.sum_scale;
    ha.label = nullptr;
    if ((rc = point_pass(ctx, f, es.out_count, es.out_sum, [&](const PointArgs& pa) {
             launch_hybrid_points(pa, ix, ha, ctx->sms, ctx->stream);
         })))
        return rc;
    RJ_CUDA(cudaGetLastError());
    es.ph->mark(3);
    // polygon-inside pass over non-border pixels (polygon-inside.frag:30-57)
    a.label = nullptr;
    a.canvas_c = canvas_c;
    a.canvas_s = canvas_s;
    a.border = mask;
    a.border_words = words;
    if ((rc = poly_pass(ctx, MODE_REDUCE, a))) return rc;
    es.ph->mark(4);
    return RJ_OK;
}

// Polygon collection -> PolySet (PolyHandler::addPolygonCollection
// PolyHandler.cpp:49-80; bounds as readPolygons PolyHandler.cpp:178-186).
int load_polyset(rj_ctx* ctx, PolySet& s, const float* xy, const int32_t* pindex, int32_t npolys,
                 const double* bbox) {
    if (npolys <= 0 || !pindex || !xy) return fail(ctx, RJ_E_INVALID, "empty polygon set");
    if (pindex[0] != 0) return fail(ctx, RJ_E_INVALID, "pindex[0] must be 0");
    for (int i = 0; i < npolys; ++i)
        if (pindex[i + 1] < pindex[i]) return fail(ctx, RJ_E_INVALID, "pindex not monotone at %d", i);
    const int V = pindex[npolys];
    double bb[4] = {INFINITY, INFINITY, -INFINITY, -INFINITY};
    float maxabs = 0.f, mdx = 0.f, mdy = 0.f;
    for (int i = 0; i < npolys; ++i) {
        const int v0 = pindex[i], n = pindex[i + 1] - v0;
        for (int k = 0; k < n; ++k) {
            float x = xy[2 * (v0 + k)], y = xy[2 * (v0 + k) + 1];
            if (!std::isfinite(x) || !std::isfinite(y)) return fail(ctx, RJ_E_INVALID, "non-finite vertex in polygon %d", i);
            bb[0] = std::min(bb[0], (double)x); bb[1] = std::min(bb[1], (double)y);
            bb[2] = std::max(bb[2], (double)x); bb[3] = std::max(bb[3], (double)y);
            maxabs = std::max(maxabs, std::max(std::fabs(x), std::fabs(y)));
            int kn = (k + 1 == n) ? 0 : k + 1;
            mdx = std::max(mdx, std::fabs(xy[2 * (v0 + kn)] - x));
            mdy = std::max(mdy, std::fabs(xy[2 * (v0 + kn) + 1] - y));
        }
    }
    if (bbox) {
        for (int i = 0; i < 4; ++i) bb[i] = bbox[i];
        maxabs = std::max(maxabs, (float)std::max(std::max(std::fabs(bb[0]), std::fabs(bb[1])),
                                                   std::max(std::fabs(bb[2]), std::fabs(bb[3]))));
    }
    if (!(bb[2] > bb[0] && bb[3] > bb[1]))
        return fail(ctx, RJ_E_INVALID, "polygon bounds are empty");   // CPUJoin.cpp:51-54
    cudaSetDevice(ctx->device);
    int rc;
    // one allocation and one copy for the three arrays (a served request
    // brings a new set: fewer driver calls per request)
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t o_pidx = al((size_t)V * 8), o_edge = o_pidx + al((size_t)(npolys + 1) * 4);
    const size_t total = o_edge + (size_t)V * 4;
    if ((rc = dev_alloc(ctx, s.d_block, total))) return rc;
    char* base = (char*)s.d_block.p;
    s.d_verts = DevBuf{base, (size_t)V * 8};
    s.d_pindex = DevBuf{base + o_pidx, (size_t)(npolys + 1) * 4};
    s.d_edge_poly = DevBuf{base + o_edge, (size_t)V * 4};
    std::vector<char> pack(total);
    std::memcpy(pack.data(), xy, (size_t)V * 8);
    std::memcpy(pack.data() + o_pidx, pindex, (size_t)(npolys + 1) * 4);
    int* edge_poly = reinterpret_cast<int*>(pack.data() + o_edge);
    for (int i = 0; i < npolys; ++i)
        for (int k = pindex[i]; k < pindex[i + 1]; ++k) edge_poly[k] = i;
    s.h_xy.assign(xy, xy + 2 * (size_t)V);
    s.h_pindex.assign(pindex, pindex + npolys + 1);
    s.h_mbr.assign(npolys, make_float4(0.f, 0.f, 0.f, 0.f));
    for (int i = 0; i < npolys; ++i) {
        float a = INFINITY, b = INFINITY, c = -INFINITY, d = -INFINITY;
        for (int k = pindex[i]; k < pindex[i + 1]; ++k) {
            a = std::min(a, xy[2 * k]); c = std::max(c, xy[2 * k]);
            b = std::min(b, xy[2 * k + 1]); d = std::max(d, xy[2 * k + 1]);
        }
        s.h_mbr[i] = make_float4(a, b, c, d);
    }
    // a synchronous copy on the default stream: it does not wait for the
    // context's (non-blocking) streams, so a set can be uploaded while joins run
    RJ_CUDA(cudaMemcpy(s.d_block.p, pack.data(), total, cudaMemcpyHostToDevice));
    double sdx = 0, sdy = 0;   // total edge extents: bound on the canvas blocks edges cross
    for (int i = 0; i < npolys; ++i) {
        const int v0 = pindex[i], n = pindex[i + 1] - v0;
        for (int k = 0; k < n; ++k) {
            const int kn = (k + 1 == n) ? 0 : k + 1;
            sdx += std::fabs((double)xy[2 * (v0 + kn)] - xy[2 * (v0 + k)]);
            sdy += std::fabs((double)xy[2 * (v0 + kn) + 1] - xy[2 * (v0 + k) + 1]);
        }
    }
    s.sum_dx = sdx;
    s.sum_dy = sdy;
    s.P = npolys;
    s.V = V;
    for (int i = 0; i < 4; ++i) s.bbox[i] = bb[i];
    s.max_abs_coord = maxabs;
    s.max_edge_dx = mdx;
    s.max_edge_dy = mdy;
    static std::atomic<uint64_t> g_set_version{0};
    s.version = ++g_set_version;
    s.overlap.clear();
    s.grid.valid = false;
    s.exact.valid = false;
    return RJ_OK;
}

void free_polyset(rj_ctx* ctx, PolySet& s) {
    dev_free(ctx, s.d_block);
    s.d_verts = s.d_pindex = s.d_edge_poly = DevBuf{};
    s.P = s.V = 0;
}

// Zone map of an owned resident table and the bounds of its finite locations
// (built once per table order; caller-held columns may change between calls,
// so they get none).  Complete on return, for kernels on any stream.
int ensure_zones(rj_ctx* ctx) {
    bool owned_all = !ctx->streamed;
    for (const Column& c : ctx->cols) owned_all = owned_all && c.owned;
    if (!owned_all) ctx->zones_valid = false;
    if (ctx->zones_valid || !owned_all || ctx->npts == 0 || ctx->capturing) return RJ_OK;
    const uint64_t nz = (ctx->npts + (1ull << kZoneShift) - 1) >> kZoneShift;
    int rc;
    // zones, then the bounds of the whole table's finite locations after them
    if ((rc = dev_alloc(ctx, ctx->zones, nz * sizeof(float4) + 16))) return rc;
    const float2* xy = (const float2*)find_col(ctx, ctx->loc_attrib)->d;
    launch_zone_boxes(xy, ctx->npts, (float4*)ctx->zones.p, ctx->sms, ctx->stream);
    unsigned* dbox = (unsigned*)((char*)ctx->zones.p + nz * sizeof(float4));
    unsigned hb[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u};
    RJ_CUDA(cudaMemcpyAsync(dbox, hb, sizeof hb, cudaMemcpyHostToDevice, ctx->stream));
    launch_xy_bounds(xy, ctx->npts, dbox, ctx->sms, ctx->stream);
    RJ_CUDA(cudaMemcpyAsync(hb, dbox, sizeof hb, cudaMemcpyDeviceToHost, ctx->stream));
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return fail(ctx, RJ_E_CUDA, "zone map build failed");
    auto unorder = [](unsigned u) {   // inverse of the kernel's order-preserving map
        const unsigned b = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
        float f;
        std::memcpy(&f, &b, 4);
        return f;
    };
    // no finite location: an empty box (lo > hi) that every query box contains
    ctx->table_box = hb[0] > hb[2] ? make_float4(INFINITY, INFINITY, -INFINITY, -INFINITY)
                                   : make_float4(unorder(hb[0]), unorder(hb[1]), unorder(hb[2]), unorder(hb[3]));
    ctx->zones_valid = true;
    return RJ_OK;
}

void query_rows(const rj_ctx* ctx, const rj_query* q, uint64_t& r0, uint64_t& r1) {
    r0 = 0;
    r1 = ctx->npts;
    if (ctx->tix.valid && q->time_attrib >= 0 && q->time_attrib == ctx->tix.attrib)
        ctx->tix.rows(q->t_start, q->t_end, ctx->npts, r0, r1);
}

// Per-polygon device outputs -> rj_result: exact counts, sums decoded from
// int64 fixed point (2^-shift) plus the fp64 sum of non-finite values, the
// reference's int32[3P] layout and the int32[4P] bounds.
void decode_result(int P, const unsigned long long* hc, const unsigned long long* hq, const double* hnf, int shift,
                   const long long* hb, rj_result* res) {
    if (!res) return;
    if (res->count) for (int i = 0; i < P; ++i) res->count[i] = hc[i];
    if (res->sum || res->compat3) {
        for (int i = 0; i < P; ++i) {
            const double s = std::ldexp((double)(long long)hq[i], -shift) + hnf[i];
            if (res->sum) res->sum[i] = s;
            if (res->compat3) {
                // [count | sum/100 | decimal*10], decodable by printResults (main.cpp:206-208)
                const double hi = std::trunc(s / 100.0);
                const double lo = std::nearbyint((s - 100.0 * hi) * 10.0);
                res->compat3[i] = (int32_t)std::min<unsigned long long>(hc[i], 0x7fffffffULL);
                res->compat3[P + i] = (int32_t)std::max(-2147483647.0, std::min(2147483647.0, hi));
                res->compat3[2 * P + i] = (int32_t)lo;
            }
        }
    }
    if (res->bounds)
        for (size_t i = 0; i < (size_t)4 * P; ++i) res->bounds[i] = hb ? (int32_t)std::min<long long>(hb[i], 0x7fffffffLL) : 0;
}

}  // namespace rjh

using namespace rjh;

// The device work of one query, queued on the context's stream: cache
// upkeep, the outputs zeroed, the join's kernels.  The per-polygon outputs
// stay on the device (oc, os, onf, ob) for the caller to copy back.
int enqueue_query(rj_ctx* ctx, const rj_query* q, Phase& ph, unsigned long long** poc, unsigned long long** pos,
                  double** ponf, long long** pob, double* t_setup) {
    int rc;
    const int P = ctx->ps->P;
    if (ctx->cache_owner != ctx->ps || ctx->cache_version != ctx->ps->version) {
        // the scratch holds another polygon set's grid structures
        ctx->ps->grid.valid = false;
        ctx->ps->exact.valid = false;
        ctx->cache_owner = ctx->ps;
        ctx->cache_version = ctx->ps->version;
    }
    query_rows(ctx, q, ctx->row0, ctx->row1);
    if ((rc = ensure_zones(ctx))) return rc;
    if (q->flags & RJ_FLAG_NO_CACHE) {
        ctx->ps->grid.valid = false;
        ctx->ps->exact.valid = false;
    }
    g_kernel_launches = 0;
    ctx->edge_tests_dev = nullptr;
    unsigned long long* oc;
    unsigned long long* os;
    double* onf;
    long long* ob;
    if ((rc = scratch_t(ctx, "out_count", P, &oc))) return rc;
    if ((rc = scratch_t(ctx, "out_sum", P, &os))) return rc;
    if ((rc = scratch_t(ctx, "out_nonfinite", P, &onf))) return rc;
    if ((rc = scratch_t(ctx, "out_bounds", (size_t)4 * P, &ob))) return rc;
    ph.mark(0);
    RJ_CUDA(cudaMemsetAsync(oc, 0, P * sizeof(unsigned long long), ctx->stream));
    RJ_CUDA(cudaMemsetAsync(os, 0, P * sizeof(unsigned long long), ctx->stream));
    RJ_CUDA(cudaMemsetAsync(onf, 0, P * sizeof(double), ctx->stream));
    ctx->sum_shift = 0;
    RJ_CUDA(cudaMemsetAsync(ob, 0, (size_t)4 * P * sizeof(long long), ctx->stream));
    RJ_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    ExecState es{oc, os, ob, &ph};
    *t_setup = now_ms();
    switch (q->function_type) {
        case RJ_RASTER_JOIN: rc = exec_raster(ctx, q, es, false); break;
        case RJ_INDEX_JOIN: rc = exec_index(ctx, q, es); break;
        case RJ_HYBRID_JOIN: rc = exec_hybrid(ctx, q, es); break;
        default: rc = exec_raster(ctx, q, es, true); break;
    }
    if (rc) return rc;
    *poc = oc;
    *pos = os;
    *ponf = onf;
    *pob = ob;
    return RJ_OK;
}

namespace rjh {
int enqueue_query_untimed(rj_ctx* ctx, const rj_query* q, unsigned long long** oc, unsigned long long** os,
                          double** onf, long long** ob) {
    Phase ph(ctx, false);
    double t_setup = 0;
    return enqueue_query(ctx, q, ph, oc, os, onf, ob, &t_setup);
}
}  // namespace rjh

// ===========================================================================
// C ABI
extern "C" {

int rj_abi_version(void) { return RJ_ABI_VERSION; }

void rj_query_init(rj_query* q) {
    if (!q) return;
    std::memset(q, 0, sizeof *q);
    q->function_type = RJ_RASTER_JOIN;
    q->aggregation = RJ_COUNT;
    q->aggr_attrib = -1;
    q->accuracy_m = 100.0;
    q->ground_resolution = 1.0;
    q->grid_res = 256;
    q->max_fbo_size = RJ_MAX_FBO_SIZE;
    q->time_attrib = -1;
    q->hybrid_canvas = 4096;
}

int rj_create(const rj_config* cfg, rj_ctx** out) {
    if (!out) return RJ_E_INVALID;
    *out = nullptr;
    rj_ctx* ctx = new rj_ctx();
    int dev = cfg ? cfg->device : 0;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        delete ctx;
        return RJ_E_CUDA;
    }
    if (dev < 0 || dev >= ndev) {
        delete ctx;
        return RJ_E_INVALID;
    }
    ctx->device = dev;
    if (cudaSetDevice(dev) != cudaSuccess) {
        delete ctx;
        return RJ_E_CUDA;
    }
    cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, dev);
    if (cfg && cfg->gpu_mem_mb > 0) ctx->budget = cfg->gpu_mem_mb * 1024LL * 1024LL;
    if (cfg && cfg->stream) {
        ctx->stream = (cudaStream_t)cfg->stream;
    } else {
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        ctx->own_stream = true;
    }
    for (auto& ev : ctx->ev) cudaEventCreate(&ev);
    if (cudaMalloc(&ctx->d_err, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        rj_destroy(ctx);
        return RJ_E_OOM;
    }
    *out = ctx;
    return RJ_OK;
}

void rj_destroy(rj_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_batch_engine(ctx);
    free_points(ctx);
    for (auto& b : ctx->sbuf) dev_free(ctx, b);
    dev_free(ctx, ctx->zones);
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
        for (int b = 0; b < 2; ++b) {
            cudaEventDestroy(ctx->copied[b]);
            cudaEventDestroy(ctx->consumed[b]);
        }
        cudaEventDestroy(ctx->copy_t0);
        cudaEventDestroy(ctx->copy_t1);
    }
    free_polyset(ctx, ctx->own);
    for (auto& kv : ctx->scratch) dev_free(ctx, kv.second);
    for (auto& ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* rj_last_error(const rj_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int rj_set_stream(rj_ctx* ctx, void* stream) {
    if (!ctx) return RJ_E_INVALID;
    cudaSetDevice(ctx->device);
    if (ctx->own_stream && ctx->stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
        ctx->own_stream = false;
    }
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
    } else {
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        ctx->own_stream = true;
    }
    return RJ_OK;
}

// Largest finite |aggregate value| of every scalar column.
static int column_stats(rj_ctx* ctx) {
    unsigned* bits;
    int rc;
    const int nc = (int)ctx->cols.size();
    if ((rc = scratch_t(ctx, "col_absmax", (size_t)std::max(nc, 1), &bits))) return rc;
    RJ_CUDA(cudaMemsetAsync(bits, 0, sizeof(unsigned) * std::max(nc, 1), ctx->stream));
    for (int i = 0; i < nc; ++i)
        if (ctx->cols[i].type != RJ_LOCATION && ctx->npts)
            launch_col_absmax((const uint32_t*)ctx->cols[i].d, ctx->cols[i].type, ctx->npts, bits + i, ctx->sms, ctx->stream);
    std::vector<unsigned> h(std::max(nc, 1));
    RJ_CUDA(cudaMemcpyAsync(h.data(), bits, sizeof(unsigned) * std::max(nc, 1), cudaMemcpyDeviceToHost, ctx->stream));
    RJ_CUDA(cudaStreamSynchronize(ctx->stream));
    RJ_CUDA(cudaGetLastError());
    for (int i = 0; i < nc; ++i) std::memcpy(&ctx->cols[i].absmax, &h[i], 4);
    return RJ_OK;
}

// Largest finite |value| of every scalar column of a host-resident table
// (several threads over row ranges).
static void column_stats_host(rj_ctx* ctx) {
    const uint64_t n = ctx->npts;
    for (Column& c : ctx->cols) {
        if (c.type == RJ_LOCATION || n == 0) continue;
        const int nt = (int)std::max<uint64_t>(1, std::min<uint64_t>(16, n / (1 << 20)));
        std::vector<float> part(nt, 0.f);
        std::vector<std::thread> th;
        for (int k = 0; k < nt; ++k) {
            th.emplace_back([&, k] {
                const uint64_t a = n * k / nt, b = n * (k + 1) / nt;
                const uint32_t* v = (const uint32_t*)c.d;
                float m = 0.f;
                for (uint64_t i = a; i < b; ++i) {
                    float x;
                    if (c.type == RJ_FLOAT) std::memcpy(&x, v + i, 4);
                    else if (c.type == RJ_INT) x = (float)(int32_t)v[i];
                    else x = (float)v[i];
                    x = std::fabs(x);
                    if (std::isfinite(x)) m = std::max(m, x);
                }
                part[k] = m;
            });
        }
        for (auto& t : th) t.join();
        c.absmax = *std::max_element(part.begin(), part.end());
    }
}

static int load_points_impl(rj_ctx* ctx, const rj_column* cols, int32_t ncols, uint64_t npoints, int32_t loc,
                            bool device, bool streamed = false, uint64_t chunk = 0) {
    if (!ctx) return RJ_E_INVALID;
    ctx->err.clear();
    if (!cols || ncols <= 0 || ncols > RJ_MAX_ATTRIBUTES)
        return fail(ctx, RJ_E_INVALID, "ncols must be 1..%d", RJ_MAX_ATTRIBUTES);
    int nloc = 0;
    for (int i = 0; i < ncols; ++i) {
        if (cols[i].type < RJ_LOCATION || cols[i].type > RJ_FLOAT)
            return fail(ctx, RJ_E_INVALID, "column %d: bad type %d", i, cols[i].type);
        if (!cols[i].data && npoints) return fail(ctx, RJ_E_INVALID, "column %d: null data", i);
        for (int j = 0; j < i; ++j)
            if (cols[j].attrib_id == cols[i].attrib_id)
                return fail(ctx, RJ_E_INVALID, "duplicate attribute id %d", cols[i].attrib_id);
        if (cols[i].attrib_id == loc) {
            if (cols[i].type != RJ_LOCATION) return fail(ctx, RJ_E_INVALID, "location attribute must have type LOCATION");
            ++nloc;
        }
        if (device && ((uintptr_t)cols[i].data & 15))
            return fail(ctx, RJ_E_INVALID, "column %d: device pointer not 16-byte aligned", i);
    }
    if (nloc != 1) return fail(ctx, RJ_E_INVALID, "location attribute %d not among the columns", loc);
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    if (ctx->server_running) return fail(ctx, RJ_E_BUSY, "a serving loop owns the context");
    cudaSetDevice(ctx->device);
    if (ctx->tix.valid) ++ctx->tix_gen;   // row ranges of time windows change meaning
    ctx->tix.valid = false;
    ctx->zones_valid = false;
    const bool was_streamed = ctx->streamed;
    ctx->streamed = false;
    // same layout as the resident table: copy into the existing buffers
    bool same = !device && !streamed && !was_streamed && (int)ctx->cols.size() == ncols && ctx->npts == npoints &&
                ctx->loc_attrib == loc;
    for (int i = 0; same && i < ncols; ++i)
        same = ctx->cols[i].owned && ctx->cols[i].attrib == cols[i].attrib_id && ctx->cols[i].type == cols[i].type;
    if (same) {
        for (int i = 0; i < ncols; ++i) {
            const size_t esz = cols[i].type == RJ_LOCATION ? 8 : 4;
            if (npoints)
                RJ_CUDA(cudaMemcpyAsync(ctx->cols[i].d, cols[i].data, esz * npoints, cudaMemcpyHostToDevice, ctx->stream));
        }
        return column_stats(ctx);
    }
    // release the previous table
    ++ctx->table_gen;
    for (Column& c : ctx->cols) {
        if (c.owned && c.d) {
            cudaFree(c.d);
            ctx->used -= (c.type == RJ_LOCATION ? 8 : 4) * ((ctx->npts + 3) & ~3ULL) + 256;
        }
    }
    ctx->cols.clear();
    ctx->npts = 0;
    ctx->loc_attrib = -1;
    for (int i = 0; i < ncols; ++i) {
        Column c;
        c.attrib = cols[i].attrib_id;
        c.type = cols[i].type;
        const size_t esz = c.type == RJ_LOCATION ? 8 : 4;
        if (device || streamed) {
            c.d = const_cast<void*>(cols[i].data);
            c.owned = false;
        } else {
            // padded to a multiple of four points so 128-bit loads stay in bounds
            const size_t bytes = esz * ((npoints + 3) & ~3ULL) + 256;
            if (ctx->budget > 0 && (int64_t)(ctx->used + bytes) > ctx->budget) {
                for (Column& o : ctx->cols) if (o.owned) cudaFree(o.d);
                ctx->cols.clear();
                return fail(ctx, RJ_E_OOM, "point table exceeds the device memory budget");
            }
            cudaError_t e = cudaMalloc(&c.d, bytes);
            if (e != cudaSuccess) {
                cudaGetLastError();
                for (Column& o : ctx->cols) if (o.owned) cudaFree(o.d);
                ctx->cols.clear();
                return fail(ctx, RJ_E_OOM, "cudaMalloc for column %d failed: %s", i, cudaGetErrorString(e));
            }
            ctx->used += bytes;
            c.owned = true;
            if (npoints) RJ_CUDA(cudaMemcpyAsync(c.d, cols[i].data, esz * npoints, cudaMemcpyHostToDevice, ctx->stream));
        }
        ctx->cols.push_back(c);
    }
    ctx->npts = npoints;
    ctx->loc_attrib = loc;
    RJ_CUDA(cudaStreamSynchronize(ctx->stream));
    if (streamed) {
        ctx->streamed = true;
        uint64_t c = chunk;
        if (c == 0) {
            // two chunk buffers of every column within half the free budget
            size_t rec = 0;
            for (const Column& col : ctx->cols) rec += col.type == RJ_LOCATION ? 8 : 4;
            size_t fr = 0, tot = 0;
            cudaMemGetInfo(&fr, &tot);
            size_t room = fr / 4;
            if (ctx->budget > 0) room = std::min<size_t>(room, (size_t)std::max<int64_t>(ctx->budget - (int64_t)ctx->used, 0) / 2);
            c = std::max<uint64_t>(1 << 20, std::min<uint64_t>(1ULL << 28, room / 2 / std::max<size_t>(rec, 1)));
        }
        ctx->chunk = std::max<uint64_t>(4, c & ~3ULL);
        column_stats_host(ctx);
        return RJ_OK;
    }
    return column_stats(ctx);
}

int rj_load_points(rj_ctx* ctx, const rj_column* cols, int32_t ncols, uint64_t npoints, int32_t loc_attrib) {
    return load_points_impl(ctx, cols, ncols, npoints, loc_attrib, false);
}

int rj_attach_points_device(rj_ctx* ctx, const rj_column* cols, int32_t ncols, uint64_t npoints,
                            int32_t loc_attrib) {
    return load_points_impl(ctx, cols, ncols, npoints, loc_attrib, true);
}

int rj_attach_points_host(rj_ctx* ctx, const rj_column* cols, int32_t ncols, uint64_t npoints, int32_t loc_attrib,
                          uint64_t chunk_points) {
    return load_points_impl(ctx, cols, ncols, npoints, loc_attrib, false, true, chunk_points);
}

int rj_attach_points_mapped(rj_ctx* ctx, const rj_column* cols, int32_t ncols, uint64_t npoints,
                            int32_t loc_attrib) {
    if (!ctx) return RJ_E_INVALID;
    if (!cols || ncols <= 0 || ncols > RJ_MAX_ATTRIBUTES)
        return fail(ctx, RJ_E_INVALID, "ncols must be 1..%d", RJ_MAX_ATTRIBUTES);
    cudaSetDevice(ctx->device);
    // page-locked host memory is addressable by the device: its device address
    std::vector<rj_column> dcols(cols, cols + ncols);
    for (int i = 0; i < ncols; ++i) {
        if (!npoints) continue;
        cudaPointerAttributes at{};
        if (!cols[i].data || cudaPointerGetAttributes(&at, cols[i].data) != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, RJ_E_INVALID, "column %d: not page-locked host memory", i);
        }
        if (at.type != cudaMemoryTypeHost || !at.devicePointer)
            return fail(ctx, RJ_E_INVALID, "column %d: not page-locked host memory the device can address", i);
        dcols[i].data = at.devicePointer;
    }
    return load_points_impl(ctx, dcols.data(), ncols, npoints, loc_attrib, true);
}

int rj_free_points(rj_ctx* ctx) {
    if (!ctx) return RJ_E_INVALID;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    if (ctx->server_running) return fail(ctx, RJ_E_BUSY, "a serving loop owns the context");
    ctx->tix.valid = false;
    ctx->zones_valid = false;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (Column& c : ctx->cols) {
        if (c.owned && c.d) {
            cudaFree(c.d);
            ctx->used -= (c.type == RJ_LOCATION ? 8 : 4) * ((ctx->npts + 3) & ~3ULL) + 256;
        }
    }
    ctx->cols.clear();
    ctx->npts = 0;
    ctx->loc_attrib = -1;
    ctx->streamed = false;
    return RJ_OK;
}

int rj_set_polygons(rj_ctx* ctx, const float* xy, const int32_t* pindex, int32_t npolys, const double* bbox) {
    if (!ctx) return RJ_E_INVALID;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    ctx->err.clear();
    if (ctx->server_running) return fail(ctx, RJ_E_BUSY, "a serving loop owns the context");
    int rc = load_polyset(ctx, ctx->own, xy, pindex, npolys, bbox);
    if (rc) return rc;
    ctx->ps = &ctx->own;
    return RJ_OK;
}

int rj_execute(rj_ctx* ctx, const rj_query* q, rj_result* res) {
    if (!ctx || !q) return RJ_E_INVALID;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    ctx->err.clear();
    const double t0 = now_ms();
    if (ctx->npts == 0 && ctx->cols.empty()) return fail(ctx, RJ_E_NO_DATA, "point table not loaded");
    if (ctx->ps->P == 0) return fail(ctx, RJ_E_NO_DATA, "polygons not set");
    if (res && res->npolys != 0 && res->npolys != ctx->ps->P)
        return fail(ctx, RJ_E_INVALID, "result sized for %d polygons, polygon set has %d", res->npolys, ctx->ps->P);
    if (q->function_type < RJ_RASTER_JOIN || q->function_type > RJ_RASTER_JOIN_BOUNDS)
        return fail(ctx, RJ_E_UNSUPPORTED, "function type %d not supported", q->function_type);   // GLHandler.cpp:201
    cudaSetDevice(ctx->device);
    int rc;
    const int P = ctx->ps->P;
    Phase ph(ctx, (q->flags & RJ_FLAG_PHASE_TIMING) != 0);
    unsigned long long *oc, *os;
    double* onf;
    long long* ob;
    double t_setup = 0;
    if ((rc = enqueue_query(ctx, q, ph, &oc, &os, &onf, &ob, &t_setup))) {
        cudaStreamSynchronize(ctx->stream);
        return rc;
    }
    std::vector<unsigned long long> hc(P), hq(P);
    std::vector<double> hnf(P);
    std::vector<long long> hb;
    int derr = 0;
    RJ_CUDA(cudaMemcpyAsync(hc.data(), oc, P * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    RJ_CUDA(cudaMemcpyAsync(hq.data(), os, P * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    RJ_CUDA(cudaMemcpyAsync(hnf.data(), onf, P * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (q->function_type == RJ_RASTER_JOIN_BOUNDS && res && res->bounds) {
        hb.resize((size_t)4 * P);
        RJ_CUDA(cudaMemcpyAsync(hb.data(), ob, (size_t)4 * P * sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
    }
    RJ_CUDA(cudaMemcpyAsync(&derr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ph.mark(5);
    RJ_CUDA(cudaStreamSynchronize(ctx->stream));
    RJ_CUDA(cudaGetLastError());
    if (derr & 4) return fail(ctx, RJ_E_INVALID, "error-bound outline read outside the tiered canvas's slots");
    if (derr) return fail(ctx, RJ_E_TIMEOUT, "a bounded device wait ran out (status 0x%x)", derr);
    decode_result(P, hc.data(), hq.data(), hnf.data(), ctx->sum_shift, hb.empty() ? nullptr : hb.data(), res);
    ctx->last_fixed.assign(hq.begin(), hq.end());
    ctx->last_nonfinite = hnf;
    ctx->last_shift = ctx->sum_shift;
    // timings (GLHandler::printTimeStats fields)
    rj_timings& t = ctx->tm;
    std::memset(&t, 0, sizeof t);
    t.pts_size = ctx->npts;
    t.poly_size = P;
    t.function = q->function_type;
    t.no_pt_passes = ctx->passes;
    t.no_constraints = q->n_constraints;
    t.setup_ms = t_setup - t0;
    t.poly_index_ms = (q->function_type == RJ_INDEX_JOIN || q->function_type == RJ_HYBRID_JOIN) ? ph.ms(1, 2) : 0.0;
    t.poly_render_ms = (q->function_type == RJ_INDEX_JOIN || q->function_type == RJ_HYBRID_JOIN) ? ph.ms(3, 4) : ph.ms(1, 2) + ph.ms(3, 4);
    t.pt_render_ms = ph.ms(2, 3);
    t.poly_mem_ms = ph.ms(4, 5);
    if (ctx->streamed && ctx->copy_t0) {
        float cm = 0.f;
        if (cudaEventElapsedTime(&cm, ctx->copy_t0, ctx->copy_t1) == cudaSuccess) t.pt_mem_ms = cm;
        else cudaGetLastError();
    }
    t.execute_ms = now_ms() - t0;
    t.accuracy = (q->function_type == RJ_RASTER_JOIN) ? (int)q->accuracy_m : 0;
    t.kernel_launches = g_kernel_launches;
    if (ctx->edge_tests_dev)
        RJ_CUDA(cudaMemcpy(&t.edge_tests, ctx->edge_tests_dev, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    return RJ_OK;
}

int32_t rj_sum_shift_for(double max_abs, uint64_t rows) {
    const double amax = std::max(std::isfinite(max_abs) ? std::fabs(max_abs) : 0.0, 1e-30);
    const int shift = (int)std::floor(62.0 - std::log2(amax) - std::log2((double)rows + 1.0));
    return std::max(-90, std::min(150, shift));
}

int rj_set_sum_shift(rj_ctx* ctx, int32_t shift) {
    if (!ctx) return RJ_E_INVALID;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    if (shift != RJ_SUM_SHIFT_AUTO && (shift < -90 || shift > 150))
        return fail(ctx, RJ_E_INVALID, "sum shift %d out of range -90..150", shift);
    ctx->forced_shift = shift;
    return RJ_OK;
}

int rj_get_sum_partials(const rj_ctx* ctx, int64_t* fixed, double* nonfinite, int32_t* shift) {
    if (!ctx) return RJ_E_INVALID;
    const size_t P = ctx->last_fixed.size();
    if (fixed && P) std::memcpy(fixed, ctx->last_fixed.data(), P * sizeof(int64_t));
    if (nonfinite && P) std::memcpy(nonfinite, ctx->last_nonfinite.data(), P * sizeof(double));
    if (shift) *shift = ctx->last_shift;
    return RJ_OK;
}

int rj_column_absmax(const rj_ctx* ctx, int32_t attrib_id, double* out) {
    if (!ctx || !out) return RJ_E_INVALID;
    const Column* c = find_col(ctx, attrib_id);
    if (!c) return RJ_E_INVALID;
    *out = (double)c->absmax;
    return RJ_OK;
}

static void plan_free(rj_plan* p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    cudaFreeHost(p->hc);
    cudaFreeHost(p->hq);
    cudaFreeHost(p->hnf);
    cudaFreeHost(p->hb);
    cudaFreeHost(p->derr);
    delete p;
}

int rj_prepare(rj_ctx* ctx, const rj_query* q, rj_plan** out) {
    if (!ctx || !q || !out) return RJ_E_INVALID;
    *out = nullptr;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    if (ctx->streamed) return fail(ctx, RJ_E_UNSUPPORTED, "a host-streamed table cannot be prepared");
    if (ctx->server_running) return fail(ctx, RJ_E_BUSY, "a serving loop owns the context");
    // one ordinary run settles the caches the capture relies on: polygon-side
    // structures, the set's overlap status on this canvas, the tuned shapes
    int rc = rj_execute(ctx, q, nullptr);
    if (rc) return rc;
    const int P = ctx->ps->P;
    rj_plan* p = new rj_plan();
    p->ctx = ctx;
    p->stream = ctx->stream;
    p->P = P;
    p->function_type = q->function_type;
    p->aggr_attrib = q->aggregation != RJ_COUNT ? q->aggr_attrib : -1;
    p->table_gen = ctx->table_gen;
    p->tix_gen = ctx->tix_gen;
    p->uses_tix = ctx->tix.valid && q->time_attrib >= 0 && q->time_attrib == ctx->tix.attrib;
    p->ps = ctx->ps;
    p->ps_version = ctx->ps->version;
    p->npts = ctx->npts;
    if (cudaHostAlloc(&p->hc, P * sizeof(unsigned long long), 0) != cudaSuccess ||
        cudaHostAlloc(&p->hq, P * sizeof(unsigned long long), 0) != cudaSuccess ||
        cudaHostAlloc(&p->hnf, P * sizeof(double), 0) != cudaSuccess ||
        cudaHostAlloc(&p->hb, (size_t)4 * P * sizeof(long long), 0) != cudaSuccess ||
        cudaHostAlloc(&p->derr, sizeof(int), 0) != cudaSuccess) {
        cudaGetLastError();
        plan_free(p);
        return fail(ctx, RJ_E_OOM, "pinned result buffers of the plan");
    }
    rj_query qc = *q;
    qc.flags &= ~RJ_FLAG_PHASE_TIMING;
    Phase ph(ctx, false);
    unsigned long long *oc = nullptr, *os = nullptr;
    double* onf = nullptr;
    long long* ob = nullptr;
    double t_setup = 0;
    cudaError_t ce = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        plan_free(p);
        return fail(ctx, RJ_E_CUDA, "cudaStreamBeginCapture: %s", cudaGetErrorString(ce));
    }
    ctx->capturing = true;
    rc = enqueue_query(ctx, &qc, ph, &oc, &os, &onf, &ob, &t_setup);
    if (!rc) {
        cudaMemcpyAsync(p->hc, oc, P * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(p->hq, os, P * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(p->hnf, onf, P * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(p->hb, ob, (size_t)4 * P * sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(p->derr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    }
    p->shift = ctx->sum_shift;
    ctx->capturing = false;
    cudaGraph_t g = nullptr;
    ce = cudaStreamEndCapture(ctx->stream, &g);
    if (rc || ce != cudaSuccess || !g) {
        cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        plan_free(p);
        if (rc) return rc;
        return fail(ctx, RJ_E_UNSUPPORTED, "the query's work could not be captured: %s", cudaGetErrorString(ce));
    }
    p->graph = g;
    ce = cudaGraphInstantiate(&p->exec, g, 0);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        plan_free(p);
        return fail(ctx, RJ_E_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(ce));
    }
    *out = p;
    return RJ_OK;
}

int rj_execute_prepared(rj_plan* p, rj_result* res) {
    if (!p || !p->ctx) return RJ_E_INVALID;
    rj_ctx* ctx = p->ctx;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    ctx->err.clear();
    const double t0 = now_ms();
    if (res && res->npolys != 0 && res->npolys != p->P)
        return fail(ctx, RJ_E_INVALID, "result sized for %d polygons, the plan has %d", res->npolys, p->P);
    if (ctx->table_gen != p->table_gen || ctx->npts != p->npts || ctx->ps != p->ps || ctx->ps->version != p->ps_version ||
        ctx->stream != p->stream || (p->uses_tix && ctx->tix_gen != p->tix_gen))
        return fail(ctx, RJ_E_INVALID, "the table, the polygon set or the stream changed since rj_prepare");
    if (p->aggr_attrib >= 0) {
        // a reload in place may change the aggregate's range and so the shift
        const Column* col = find_col(ctx, p->aggr_attrib);
        const int shift = ctx->forced_shift != RJ_SUM_SHIFT_AUTO
                              ? ctx->forced_shift
                              : rj_sum_shift_for(col ? (double)col->absmax : 0.0, ctx->npts);
        if (shift != p->shift)
            return fail(ctx, RJ_E_INVALID, "the aggregate's fixed-point scale changed since rj_prepare (%d -> %d)",
                        p->shift, shift);
    }
    cudaSetDevice(ctx->device);
    RJ_CUDA(cudaGraphLaunch(p->exec, ctx->stream));
    RJ_CUDA(cudaStreamSynchronize(ctx->stream));
    if (*p->derr) return fail(ctx, RJ_E_TIMEOUT, "a bounded device wait ran out (status 0x%x)", *p->derr);
    const int P = p->P;
    decode_result(P, p->hc, p->hq, p->hnf, p->shift, p->function_type == RJ_RASTER_JOIN_BOUNDS ? p->hb : nullptr,
                  res);
    ctx->last_fixed.assign(p->hq, p->hq + P);
    ctx->last_nonfinite.assign(p->hnf, p->hnf + P);
    ctx->last_shift = p->shift;
    rj_timings& t = ctx->tm;
    std::memset(&t, 0, sizeof t);
    t.pts_size = ctx->npts;
    t.poly_size = P;
    t.function = p->function_type;
    t.no_pt_passes = 1;
    t.execute_ms = now_ms() - t0;
    t.kernel_launches = 0;
    return RJ_OK;
}

void rj_plan_destroy(rj_plan* p) {
    if (!p) return;
    if (p->ctx) {
        std::lock_guard<std::recursive_mutex> lock(p->ctx->mu);
        cudaSetDevice(p->ctx->device);
        plan_free(p);
        return;
    }
    plan_free(p);
}

int rj_selftest_bounded_wait(rj_ctx* ctx, uint32_t limit_us) {
    if (!ctx) return RJ_E_INVALID;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    ctx->err.clear();
    if (limit_us < 1) return fail(ctx, RJ_E_INVALID, "limit must be at least 1 us");
    cudaSetDevice(ctx->device);
    int derr = 0;
    RJ_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    launch_wait_selftest(ctx->d_err, (uint64_t)limit_us * 1000ull, ctx->stream);
    RJ_CUDA(cudaGetLastError());
    RJ_CUDA(cudaMemcpyAsync(&derr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    RJ_CUDA(cudaStreamSynchronize(ctx->stream));
    if (derr) return fail(ctx, RJ_E_TIMEOUT, "a bounded device wait ran out after %u us (status 0x%x)", limit_us, derr);
    return RJ_OK;
}

int rj_set_tuning(rj_ctx* ctx, int32_t knob, int32_t value) {
    if (!ctx) return RJ_E_INVALID;
    std::lock_guard<std::recursive_mutex> lock(ctx->mu);
    switch (knob) {
        case RJ_TUNE_POINT_SHAPE:
            if (value != -1 && value != 0 && value != 2 && value != 3)
                return fail(ctx, RJ_E_INVALID, "point shape %d: -1, 0, 2 or 3", value);
            ctx->point_shape = value;
            return RJ_OK;
        case RJ_TUNE_COUNT_SHAPE:
            if (value < -1 || value >= label_count_shapes())
                return fail(ctx, RJ_E_INVALID, "count shape %d: -1..%d", value, label_count_shapes() - 1);
            ctx->count_shape = value;
            return RJ_OK;
        case RJ_TUNE_COUNT_BLOCK_SHIFT:
            if (value != -1 && (value < 4 || value > 8))
                return fail(ctx, RJ_E_INVALID, "count block shift %d: -1 or 4..8", value);
            ctx->count_bshift = value;
            return RJ_OK;
        case RJ_TUNE_WAIT_LIMIT:
            if (value < 1) return fail(ctx, RJ_E_INVALID, "wait limit %d us: at least 1", value);
            ctx->wait_ns = (uint64_t)value * 1000ull;
            return RJ_OK;
        case RJ_TUNE_HYBRID_EXACT_SCALE:
            if (value != 1 && value != 2 && value != 4)
                return fail(ctx, RJ_E_INVALID, "hybrid exact scale %d: 1, 2 or 4", value);
            ctx->hybrid_exact_scale = value;
            ctx->ps->exact.valid = false;
            return RJ_OK;
        default:
            return fail(ctx, RJ_E_INVALID, "unknown tuning knob %d", knob);
    }
}

int rj_get_tuning(const rj_ctx* ctx, int32_t knob, int32_t* value) {
    if (!ctx || !value) return RJ_E_INVALID;
    switch (knob) {
        case RJ_TUNE_POINT_SHAPE: *value = ctx->point_shape; return RJ_OK;
        case RJ_TUNE_COUNT_SHAPE: *value = ctx->last_count_shape; return RJ_OK;
        case RJ_TUNE_COUNT_BLOCK_SHIFT: *value = ctx->last_count_bshift; return RJ_OK;
        case RJ_TUNE_HYBRID_EXACT_SCALE: *value = ctx->hybrid_exact_scale; return RJ_OK;
        case RJ_TUNE_COUNT_SHAPES: *value = label_count_shapes(); return RJ_OK;
        case RJ_TUNE_LEAN_SHAPES: *value = label_lean_shapes(); return RJ_OK;
        case RJ_TUNE_SPLAT_SHAPES: *value = splat_lean_shapes(); return RJ_OK;
        case RJ_TUNE_HYBRID_SHAPES: *value = hybrid_lean_shapes(); return RJ_OK;
        case RJ_TUNE_WAIT_LIMIT: *value = (int32_t)std::min<uint64_t>(ctx->wait_ns / 1000ull, 0x7FFFFFFFull); return RJ_OK;
        default: return RJ_E_INVALID;
    }
}

int rj_get_timings(const rj_ctx* ctx, rj_timings* out) {
    if (!ctx || !out) return RJ_E_INVALID;
    *out = ctx->tm;
    return RJ_OK;
}

int rj_format_time_stats(const rj_ctx* ctx, char* buf, size_t buflen) {
    if (!ctx || !buf || buflen == 0) return RJ_E_INVALID;
    const rj_timings& t = ctx->tm;
    const int fn = t.function == RJ_RASTER_JOIN_BOUNDS ? 5 : t.function;   // GLHandler.cpp:228
    snprintf(buf, buflen, "%llu\t\t%d\t%d\t%d\t%d\t%lld\t%lld\t%lld\t%lld\t%lld\t%lld\t%lld\t%lld\t%lld\t%d",
             (unsigned long long)t.pts_size, t.poly_size, fn, t.no_pt_passes, t.no_constraints,
             (long long)std::llround(t.execute_ms), (long long)std::llround(t.pt_mem_ms),
             (long long)std::llround(t.pt_render_ms), (long long)std::llround(t.poly_mem_ms),
             (long long)std::llround(t.poly_render_ms), (long long)std::llround(t.setup_ms),
             (long long)std::llround(t.triangulation_ms), (long long)std::llround(t.poly_index_ms),
             (long long)std::llround(t.backend_query_ms), t.accuracy);
    return RJ_OK;
}

}  // extern "C"
