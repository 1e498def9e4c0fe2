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

// ---------------------------------------------------------------------------
struct SplatMapper {
    CanvasXf cx;
    uint32_t* canvas_c;
    double* canvas_s;
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H&) const {
        const size_t tile_px = (size_t)cx.resx * cx.resy;
        canvas_visit(cx, x, y, [&](int t, int px, int py) {
            size_t pix = (size_t)t * tile_px + (size_t)py * cx.resx + px;
            atomicAdd(canvas_c + pix, 1u);
            if (canvas_s) atomicAdd(canvas_s + pix, (double)v);
        });
    }
};

struct LabelMapper {
    CanvasXf cx;
    const uint32_t* label;
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H& h) const {
        const size_t tile_px = (size_t)cx.resx * cx.resy;
        canvas_visit(cx, x, y, [&](int t, int px, int py) {
            uint32_t lab = __ldg(label + (size_t)t * tile_px + (size_t)py * cx.resx + px);
            if (lab != kEmptyLabel) h.add((int)lab, v);
        });
    }
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
    IndexArgs ia;
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H& h) const {
        index_probe(ia, x, y, v, h);
    }
};

struct HybridMapper {
    IndexArgs ia;
    HybridArgs ha;
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H& h) const {
        int px, py;
        if (!hyb_rasterize(ha.h, x, y, px, py)) return;
        bool border = true;
        if (px < ha.h.resx && py < ha.h.resy) {
            uint32_t w = __ldg(ha.border + (size_t)py * ha.words + (px >> 5));
            border = (w >> (px & 31)) & 1u;
        }
        if (border) {
            index_probe(ia, x, y, v, h);
        } else if (ha.label) {
            uint32_t lab = __ldg(ha.label + (size_t)py * ha.h.resx + px);
            if (lab != kEmptyLabel) h.add((int)lab, v);
        } else {
            size_t pix = (size_t)py * ha.h.resx + px;
            atomicAdd(ha.canvas_c + pix, 1u);
            if (ha.canvas_s) atomicAdd(ha.canvas_s + pix, (double)v);
        }
    }
};

// ---------------------------------------------------------------------------
template <class M, bool AGG, bool SMEM>
__global__ void __launch_bounds__(kPointThreads)
k_points(PointArgs pa, M mp) {
    extern __shared__ double smem_d[];
    double* s_sum = smem_d;
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(smem_d + (AGG ? pa.P : 0));
    if (SMEM) {
        for (int b = threadIdx.x; b < pa.P; b += blockDim.x) {
            s_cnt[b] = 0u;
            if (AGG) s_sum[b] = 0.0;
        }
        __syncthreads();
    }
    Hist<AGG, SMEM> h{s_cnt, s_sum, pa.out_count, pa.out_sum};
    const DevFilter& f = pa.f;
    const uint64_t ngroups = (pa.n + 3) >> 2;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ngroups; g += stride) {
        const uint64_t base = g << 2;
        float x[4], y[4], val[4] = {0.f, 0.f, 0.f, 0.f};
        uint32_t mask;
        if (base + 4 <= pa.n) {
            const float4 a = __ldg(reinterpret_cast<const float4*>(pa.xy + base));
            const float4 b = __ldg(reinterpret_cast<const float4*>(pa.xy + base + 2));
            x[0] = a.x; y[0] = a.y; x[1] = a.z; y[1] = a.w;
            x[2] = b.x; y[2] = b.y; x[3] = b.z; y[3] = b.w;
            mask = 0xFu;
            #pragma unroll
            for (int k = 0; k < kMaxFilters; ++k) {
                if (k >= f.n) break;
                const uint4 c = __ldg(reinterpret_cast<const uint4*>(f.col[k] + base));
                const int op = f.op[k], ty = f.typ[k], cm = (int)((f.compat_mask >> k) & 1u);
                const uint32_t fv = f.val[k];
                mask &= (pred_eval(op, ty, c.x, fv, cm) ? 1u : 0u) | (pred_eval(op, ty, c.y, fv, cm) ? 2u : 0u) |
                        (pred_eval(op, ty, c.z, fv, cm) ? 4u : 0u) | (pred_eval(op, ty, c.w, fv, cm) ? 8u : 0u);
            }
            if (AGG) {
                const uint4 c = __ldg(reinterpret_cast<const uint4*>(f.aggr_col + base));
                val[0] = agg_value(f.aggr_typ, c.x); val[1] = agg_value(f.aggr_typ, c.y);
                val[2] = agg_value(f.aggr_typ, c.z); val[3] = agg_value(f.aggr_typ, c.w);
            }
        } else {
            mask = 0u;
            #pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint64_t i = base + q;
                if (i >= pa.n) { x[q] = 0.f; y[q] = 0.f; continue; }
                const float2 p = __ldg(pa.xy + i);
                x[q] = p.x; y[q] = p.y;
                if (filter_point(f, i)) mask |= 1u << q;
                if (AGG) val[q] = agg_value(f.aggr_typ, __ldg(f.aggr_col + i));
            }
        }
        #pragma unroll
        for (int q = 0; q < 4; ++q)
            if ((mask >> q) & 1u) mp.map(x[q], y[q], val[q], h);
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

template <class M, bool AGG, bool SMEM>
static void launch_points_t(const PointArgs& pa, const M& mp, int sms, cudaStream_t st) {
    size_t smem = SMEM ? hist_bytes(pa.P, AGG) : 0;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_points<M, AGG, SMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 2;
    if (smem > 100 * 1024) per_sm = 1;
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
    const bool smem_ok = hist_bytes(pa.P, agg) <= (size_t)std::max(g_max_smem_optin - 1024, 0);
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

void launch_raster_label(const PointArgs& pa, const CanvasXf& cx, const uint32_t* label, int sms,
                         cudaStream_t st) {
    LabelMapper m{cx, label};
    launch_points(pa, m, sms, st);
}

void launch_index_points(const PointArgs& pa, const IndexArgs& ia, int sms, cudaStream_t st) {
    IndexMapper m{ia};
    launch_points(pa, m, sms, st);
}

void launch_hybrid_points(const PointArgs& pa, const IndexArgs& ia, const HybridArgs& ha, int sms,
                          cudaStream_t st) {
    HybridMapper m{ia, ha};
    launch_points(pa, m, sms, st);
}

}  // namespace rj
