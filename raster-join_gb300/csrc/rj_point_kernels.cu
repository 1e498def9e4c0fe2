// rj_point_kernels.cu -- point-side kernels (the hot path).
//
// One streaming pass over the resident point table per query.  Each thread
// takes groups of four consecutive points: the location column is read as two
// 128-bit loads, every constraint / aggregate column as one 128-bit load.
// Predicates follow points.vert:138-159; the per-point mapping differs per
// join:
//   * raster splat : pixel of the point in every canvas tile, atomic add into
//                    the tile canvas (points.vert + additive blending,
//                    RasterJoin.cpp:91-148)
//   * raster label : pixel -> polygon label -> per-block shared histogram
//                    (the point pass and polygon pass fused for polygon sets
//                    whose coverage does not overlap)
//   * index        : grid cell -> candidate polygons -> fp32 crossing-number
//                    test (index.glsl:339-402)
//   * hybrid       : hybrid canvas pixel; border pixels take the index path,
//                    the others the canvas / label path (hybrid.glsl:224-300)
// Per-polygon results accumulate in shared memory (count u32, sum f64) and are
// flushed once per block with global atomics.
#include "rj_device.cuh"
#include "rj_launch.h"

namespace rj {

constexpr int kPointThreads = 512;
// deferred-point queue: < kPointThreads left over + 4 per thread per iteration
constexpr int kQueueCap = kPointThreads * 5;

// ---------------------------------------------------------------------------
template <bool AGG, bool SMEM>
struct Hist {
    uint32_t* s_cnt;
    double* s_sum;
    unsigned long long* g_cnt;
    double* g_sum;
    __device__ __forceinline__ void add(int p, float v) const {
        if (SMEM) {
            atomicAdd(s_cnt + p, 1u);
            if (AGG) atomicAdd(s_sum + p, (double)v);
        } else {
            atomicAdd(g_cnt + p, 1ull);
            if (AGG) atomicAdd(g_sum + p, (double)v);
        }
    }
};

// Visit every canvas tile whose window contains the point: fn(tile, px, py).
// A point near a tile seam may land in two tiles, as it would when every tile
// is rendered with all points (RasterJoin.cpp:224-231).
struct TileHit { int t; int px; };

__device__ __forceinline__ int axis_hits(float v, const float4* __restrict__ xf, int split, float lb, float td,
                                         int res, const float4& xf0, TileHit* out) {
    int nh = 0;
    if (split == 1) {
        float w = win_coord(v, xf0.x, xf0.y, xf0.z);
        if (w > -1.0f && w < (float)res + 1.0f) {
            int p = pix_of(snap_win(w));
            if (p >= 0 && p < res) { out[0].t = 0; out[0].px = p; nh = 1; }
        }
        return nh;
    }
    float g = floorf(__fdiv_rn(__fsub_rn(v, lb), td));
    int c0 = (g > -2.0f && g < (float)split + 1.0f) ? (int)g : -1000000;
    #pragma unroll
    for (int d = -1; d <= 1; ++d) {
        int c = c0 + d;
        if (c < 0 || c >= split) continue;
        float4 x = __ldg(xf + c);
        float w = win_coord(v, x.x, x.y, x.z);
        if (w > -1.0f && w < (float)res + 1.0f) {
            int p = pix_of(snap_win(w));
            if (p >= 0 && p < res) { out[nh].t = c; out[nh].px = p; ++nh; }
        }
    }
    return nh;
}

template <class F>
__device__ __forceinline__ void canvas_visit(const CanvasXf& c, float x, float y, F&& fn) {
    TileHit hx[3], hy[3];
    int nx = axis_hits(x, c.colxf, c.splitx, c.lbx, c.tdx, c.resx, c.col0, hx);
    if (nx == 0) return;
    int ny = axis_hits(y, c.rowxf, c.splity, c.lby, c.tdy, c.resy, c.row0, hy);
    for (int a = 0; a < nx; ++a)
        for (int b = 0; b < ny; ++b)
            fn(hy[b].t * c.splitx + hx[a].t, hx[a].px, hy[b].px);
}

// Border points collected per block in shared memory and processed in full
// warps (a few lanes of a warp taking the exact test would stall the other
// 31 lanes of the streaming pass).
struct DeferQ {
    float* qx;
    float* qy;
    float* qv;
    int* qn;
    __device__ __forceinline__ void push(float x, float y, float v) const {
        int s = atomicAdd(qn, 1);
        qx[s] = x;
        qy[s] = y;
        qv[s] = v;
    }
};

// ---------------------------------------------------------------------------
struct SplatMapper {
    static constexpr bool kDefer = false;
    CanvasXf cx;
    uint32_t* canvas_c;
    double* canvas_s;
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H&, const DeferQ&) const {
        const size_t tile_px = (size_t)cx.resx * cx.resy;
        canvas_visit(cx, x, y, [&](int t, int px, int py) {
            size_t pix = (size_t)t * tile_px + (size_t)py * cx.resx + px;
            atomicAdd(canvas_c + pix, 1u);
            if (canvas_s) atomicAdd(canvas_s + pix, (double)v);
        });
    }
    template <class H>
    __device__ __forceinline__ void deferred(float, float, float, const H&) const {}
};

struct LabelMapper {
    static constexpr bool kDefer = false;
    CanvasXf cx;
    const uint16_t* label;
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H& h, const DeferQ&) const {
        const size_t tile_px = (size_t)cx.resx * cx.resy;
        canvas_visit(cx, x, y, [&](int t, int px, int py) {
            uint16_t lab = __ldg(label + (size_t)t * tile_px + (size_t)py * cx.resx + px);
            if (lab != kEmptyLabel) h.add((int)lab, v);
        });
    }
    template <class H>
    __device__ __forceinline__ void deferred(float, float, float, const H&) const {}
};

__device__ __forceinline__ bool index_cell(const IndexArgs& ia, float x, float y, int& cell) {
    float qx = __fdiv_rn(__fsub_rn(x, ia.lbx), ia.csx);
    float qy = __fdiv_rn(__fsub_rn(y, ia.lby), ia.csy);
    // int() truncation toward zero, then the range test of index.glsl:385
    if (!(qx > -1.0f && qx < (float)ia.res && qy > -1.0f && qy < (float)ia.res)) return false;
    cell = (int)qx + ia.res * (int)qy;
    return true;
}

template <class H>
__device__ __forceinline__ void index_probe(const IndexArgs& ia, float x, float y, float v, const H& h) {
    int cell;
    if (!index_cell(ia, x, y, cell)) return;
    const int s = __ldg(ia.cell_start + cell), e = __ldg(ia.cell_start + cell + 1);
    for (int k = s; k < e; ++k) {
        const int p = __ldg(ia.entries + k);
        const int v0 = __ldg(ia.pindex + p), n = __ldg(ia.pindex + p + 1) - v0;
        if (n > 0 && pip_f32(ia.verts + v0, n, x, y)) h.add(p, v);
    }
}

struct IndexMapper {
    static constexpr bool kDefer = false;
    IndexArgs ia;
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H& h, const DeferQ&) const {
        index_probe(ia, x, y, v, h);
    }
    template <class H>
    __device__ __forceinline__ void deferred(float, float, float, const H&) const {}
};

// Exact point-in-polygon through the classified grid: identical result to the
// fp32 crossing-number test against every candidate polygon of the query's
// grid cell (index.glsl:382-400).  The classified grid has 2^k times the query
// grid's resolution, so its fp32 cell coordinate is exactly 2^k times the
// query grid's: the right/top domain limits coincide, and the points the
// query grid admits left/below of this grid's cell 0 lie more than one cell
// outside every polygon (never inside).
template <class H>
__device__ __forceinline__ void exact_probe(const ExactIndex& ix, float x, float y, float v, const H& h) {
    float gx = __fdiv_rn(__fsub_rn(x, ix.lbx), ix.csx);
    float gy = __fdiv_rn(__fsub_rn(y, ix.lby), ix.csy);
    if (!(gx > -1.0f && gx < (float)ix.res && gy > -1.0f && gy < (float)ix.res)) return;
    const int cell = (int)gx + ix.res * (int)gy;
    const uint32_t code = __ldg(ix.code + cell);
    if (code < kCodeList) { h.add((int)code, v); return; }
    if (code == kCodeEmpty) return;
    const int s = __ldg(ix.cell_start + cell), e = __ldg(ix.cell_start + cell + 1);
    for (int k = s; k < e; ++k) {
        const int4 en = __ldg(ix.entries + k);
        if (en.y < 0) { h.add(en.x, v); continue; }
        const float4* E = ix.edges + en.w;
        bool c = false;
        for (int r = 0; r < en.y; ++r) {
            const float4 q = __ldg(E + r);
            c ^= ((q.y > y) != (q.w > y));
        }
        for (int f = 0; f < en.z; ++f) {
            const float4 q = __ldg(E + en.y + f);
            c ^= edge_toggles(q.x, q.y, q.z, q.w, x, y);
        }
        if (c) h.add(en.x, v);
    }
}

struct ExactMapper {
    static constexpr bool kDefer = false;
    ExactIndex ix;
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H& h, const DeferQ&) const {
        exact_probe(ix, x, y, v, h);
    }
    template <class H>
    __device__ __forceinline__ void deferred(float, float, float, const H&) const {}
};

struct HybridMapper {
    static constexpr bool kDefer = true;
    ExactIndex ix;
    HybridArgs ha;
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H& h, const DeferQ& q) const {
        int px, py;
        if (!hyb_rasterize(ha.h, x, y, px, py)) return;
        if (px >= ha.h.resx || py >= ha.h.resy) { q.push(x, y, v); return; }
        const size_t pix = (size_t)py * ha.h.resx + px;
        if (ha.label) {
            const uint16_t lab = __ldg(ha.label + pix);
            if (lab == kBorderLabel) q.push(x, y, v);
            else if (lab != kEmptyLabel) h.add((int)lab, v);
        } else {
            const uint32_t w = __ldg(ha.border + (size_t)py * ha.words + (px >> 5));
            if ((w >> (px & 31)) & 1u) {
                q.push(x, y, v);
            } else {
                atomicAdd(ha.canvas_c + pix, 1u);
                if (ha.canvas_s) atomicAdd(ha.canvas_s + pix, (double)v);
            }
        }
    }
    template <class H>
    __device__ __forceinline__ void deferred(float x, float y, float v, const H& h) const {
        exact_probe(ix, x, y, v, h);
    }
};

// ---------------------------------------------------------------------------
template <class M, bool AGG, bool SMEM>
__global__ void __launch_bounds__(kPointThreads)
k_points(PointArgs pa, M mp) {
    extern __shared__ double smem_d[];
    double* s_sum = smem_d;
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(smem_d + ((AGG && SMEM) ? pa.P : 0));
    float* s_q = reinterpret_cast<float*>(s_cnt + (SMEM ? pa.P : 0));
    DeferQ dq{s_q, s_q + kQueueCap, s_q + 2 * kQueueCap, reinterpret_cast<int*>(s_q + 3 * kQueueCap)};
    if (SMEM) {
        for (int b = threadIdx.x; b < pa.P; b += blockDim.x) {
            s_cnt[b] = 0u;
            if (AGG) s_sum[b] = 0.0;
        }
    }
    if (M::kDefer && threadIdx.x == 0) *dq.qn = 0;
    __syncthreads();
    Hist<AGG, SMEM> h{s_cnt, s_sum, pa.out_count, pa.out_sum};
    const DevFilter& f = pa.f;
    const uint64_t per_iter = (uint64_t)blockDim.x * 4;
    // block-uniform trip count: every thread of a block runs the same iterations
    for (uint64_t tb = (uint64_t)blockIdx.x * per_iter; tb < pa.n; tb += (uint64_t)gridDim.x * per_iter) {
        const uint64_t base = tb + (uint64_t)threadIdx.x * 4;
        float x[4], y[4], val[4] = {0.f, 0.f, 0.f, 0.f};
        uint32_t mask = 0u;
        if (base + 4 <= pa.n) {
            // column data is read once: evict-first so it does not push the
            // label map / grid out of L2
            const float4 a = __ldcs(reinterpret_cast<const float4*>(pa.xy + base));
            const float4 b = __ldcs(reinterpret_cast<const float4*>(pa.xy + base + 2));
            x[0] = a.x; y[0] = a.y; x[1] = a.z; y[1] = a.w;
            x[2] = b.x; y[2] = b.y; x[3] = b.z; y[3] = b.w;
            mask = 0xFu;
            #pragma unroll
            for (int k = 0; k < kMaxFilters; ++k) {
                if (k >= f.n) break;
                const uint4 c = __ldcs(reinterpret_cast<const uint4*>(f.col[k] + base));
                const int op = f.op[k], ty = f.typ[k], cm = (int)((f.compat_mask >> k) & 1u);
                const uint32_t fv = f.val[k];
                mask &= (pred_eval(op, ty, c.x, fv, cm) ? 1u : 0u) | (pred_eval(op, ty, c.y, fv, cm) ? 2u : 0u) |
                        (pred_eval(op, ty, c.z, fv, cm) ? 4u : 0u) | (pred_eval(op, ty, c.w, fv, cm) ? 8u : 0u);
            }
            if (AGG) {
                const uint4 c = __ldcs(reinterpret_cast<const uint4*>(f.aggr_col + base));
                val[0] = agg_value(f.aggr_typ, c.x); val[1] = agg_value(f.aggr_typ, c.y);
                val[2] = agg_value(f.aggr_typ, c.z); val[3] = agg_value(f.aggr_typ, c.w);
            }
        } else {
            #pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint64_t i = base + q;
                x[q] = 0.f; y[q] = 0.f;
                if (i >= pa.n) continue;
                const float2 p = __ldg(pa.xy + i);
                x[q] = p.x; y[q] = p.y;
                if (filter_point(f, i)) mask |= 1u << q;
                if (AGG) val[q] = agg_value(f.aggr_typ, __ldg(f.aggr_col + i));
            }
        }
        #pragma unroll
        for (int q = 0; q < 4; ++q)
            if ((mask >> q) & 1u) mp.map(x[q], y[q], val[q], h, dq);
        if (M::kDefer) {
            // drain full batches of deferred points, one point per thread
            __syncthreads();
            while (*dq.qn >= (int)blockDim.x) {
                const int s = *dq.qn - (int)blockDim.x + (int)threadIdx.x;
                mp.deferred(dq.qx[s], dq.qy[s], dq.qv[s], h);
                __syncthreads();
                if (threadIdx.x == 0) *dq.qn -= (int)blockDim.x;
                __syncthreads();
            }
        }
    }
    if (M::kDefer) {
        __syncthreads();
        const int cnt = *dq.qn;
        if ((int)threadIdx.x < cnt) mp.deferred(dq.qx[threadIdx.x], dq.qy[threadIdx.x], dq.qv[threadIdx.x], h);
    }
    if (SMEM) {
        __syncthreads();
        for (int b = threadIdx.x; b < pa.P; b += blockDim.x) {
            uint32_t c = s_cnt[b];
            if (c) atomicAdd(pa.out_count + b, (unsigned long long)c);
            if (AGG) {
                double s = s_sum[b];
                if (c) atomicAdd(pa.out_sum + b, s);
            }
        }
    }
}

// ---------------------------------------------------------------------------
static int g_max_smem_optin = -1;

static size_t hist_bytes(int P, bool agg) { return (size_t)P * (agg ? 12 : 4); }
static size_t queue_bytes(bool defer) { return defer ? (size_t)kQueueCap * 12 + 16 : 0; }

template <class M, bool AGG, bool SMEM>
static void launch_points_t(const PointArgs& pa, const M& mp, int sms, cudaStream_t st) {
    size_t smem = (SMEM ? hist_bytes(pa.P, AGG) : 0) + queue_bytes(M::kDefer);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_points<M, AGG, SMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_points<M, AGG, SMEM>, kPointThreads, smem);
    if (per_sm < 1) per_sm = 1;
    uint64_t groups = (pa.n + 3) / 4;
    uint64_t need = (groups + kPointThreads - 1) / kPointThreads;
    uint64_t blocks = (uint64_t)sms * per_sm;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    k_points<M, AGG, SMEM><<<(unsigned)blocks, kPointThreads, smem, st>>>(pa, mp);
    ++g_kernel_launches;
}

template <class M>
static void launch_points(const PointArgs& pa, const M& mp, int sms, cudaStream_t st) {
    if (g_max_smem_optin < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    const bool agg = pa.f.aggr != 0;
    const bool smem_ok = hist_bytes(pa.P, agg) + queue_bytes(M::kDefer) <= (size_t)std::max(g_max_smem_optin - 1024, 0);
    if (agg) {
        if (smem_ok) launch_points_t<M, true, true>(pa, mp, sms, st);
        else launch_points_t<M, true, false>(pa, mp, sms, st);
    } else {
        if (smem_ok) launch_points_t<M, false, true>(pa, mp, sms, st);
        else launch_points_t<M, false, false>(pa, mp, sms, st);
    }
}

void launch_raster_splat(const PointArgs& pa, const CanvasXf& cx, uint32_t* canvas_c, double* canvas_s,
                         int sms, cudaStream_t st) {
    SplatMapper m{cx, canvas_c, canvas_s};
    // the splat writes the canvas directly: no per-polygon histogram
    PointArgs p2 = pa;
    p2.P = 0;
    if (pa.f.aggr) launch_points_t<SplatMapper, true, false>(p2, m, sms, st);
    else launch_points_t<SplatMapper, false, false>(p2, m, sms, st);
}

void launch_raster_label(const PointArgs& pa, const CanvasXf& cx, const uint16_t* label, int sms,
                         cudaStream_t st) {
    LabelMapper m{cx, label};
    launch_points(pa, m, sms, st);
}

void launch_index_points(const PointArgs& pa, const IndexArgs& ia, int sms, cudaStream_t st) {
    IndexMapper m{ia};
    launch_points(pa, m, sms, st);
}

void launch_exact_points(const PointArgs& pa, const ExactIndex& ix, int sms, cudaStream_t st) {
    ExactMapper m{ix};
    launch_points(pa, m, sms, st);
}

void launch_hybrid_points(const PointArgs& pa, const ExactIndex& ix, const HybridArgs& ha, int sms,
                          cudaStream_t st) {
    HybridMapper m{ix, ha};
    launch_points(pa, m, sms, st);
}

}  // namespace rj
