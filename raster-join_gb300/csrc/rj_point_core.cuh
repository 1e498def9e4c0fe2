// rj_point_core.cuh -- point-side kernels (the hot path): mappers, the
// streaming kernels and their launch templates, shared by the two point-pass
// translation units (raster forms; index / exact / hybrid forms).
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
#pragma once

#include "rj_device.cuh"
#include "rj_launch.h"
#include "rj_point_map.cuh"

namespace rj {

constexpr int kPointThreads = 512;
// canvases up to this many pixels are splatted into a per-block shared copy
constexpr int kSplatPrivPixels = 8192;
// deferred-point queue: < kPointThreads left over + 4 per thread per iteration
constexpr int kQueueCap = kPointThreads * 5;

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
    static constexpr bool kTwoPhase = false;
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
__device__ __forceinline__ void exact_list(const ExactIndex& ix, int cell, float x, float y, float v, const H& h) {
    const int s = __ldg(ix.cell_start + cell), e = __ldg(ix.cell_start + cell + 1);
    unsigned ntests = 0;
    for (int k = s; k < e; ++k) {
        const int4 en = __ldg(ix.entries + k);
        if (en.y < 0) { h.add(en.x, v); continue; }
        ntests += (unsigned)(en.y + en.z);
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
    if (ix.tests && ntests) atomicAdd(ix.tests, (unsigned long long)ntests);
}

template <class H>
__device__ __forceinline__ void exact_probe(const ExactIndex& ix, float x, float y, float v, const H& h) {
    float gx = __fdiv_rn(__fsub_rn(x, ix.lbx), ix.csx);
    float gy = __fdiv_rn(__fsub_rn(y, ix.lby), ix.csy);
    if (!(gx > -1.0f && gx < (float)ix.res && gy > -1.0f && gy < (float)ix.res)) return;
    const int cell = (int)gx + ix.res * (int)gy;
    const uint32_t code = __ldg(ix.code + cell);
    if (code < kCodeList) { h.add((int)code, v); return; }
    if (code == kCodeEmpty) return;
    exact_list(ix, cell, x, y, v, h);
}

struct ExactMapper {
    static constexpr bool kDefer = false;
    static constexpr bool kTwoPhase = true;
    ExactIndex ix;
    using Key = uint2;                      // (cell code, cell)
    static constexpr uint32_t kNoneCode = kCodeEmpty;
    __device__ __forceinline__ Key lookup(float x, float y) const {
        float gx = __fdiv_rn(__fsub_rn(x, ix.lbx), ix.csx);
        float gy = __fdiv_rn(__fsub_rn(y, ix.lby), ix.csy);
        if (!(gx > -1.0f && gx < (float)ix.res && gy > -1.0f && gy < (float)ix.res)) return make_uint2(kCodeEmpty, 0u);
        const int cell = (int)gx + ix.res * (int)gy;
        return make_uint2(__ldg(ix.code + cell), (uint32_t)cell);
    }
    template <class H>
    __device__ __forceinline__ void consume(bool valid, Key k, float x, float y, float v, const H& h,
                                            const DeferQ&) const {
        h.add_warp(valid && k.x < kCodeList, (int)k.x, v);
        if (valid && k.x == kCodeList) exact_list(ix, (int)k.y, x, y, v, h);
    }
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H& h, const DeferQ&) const {
        exact_probe(ix, x, y, v, h);
    }
    template <class H>
    __device__ __forceinline__ void deferred(float, float, float, const H&) const {}
};

struct HybridMapper {
    static constexpr bool kDefer = true;
    static constexpr bool kTwoPhase = true;
    ExactIndex ix;
    HybridArgs ha;
    using Key = uint32_t;
    static constexpr Key kNone = 0xFFFFu;
    static constexpr Key kCanvas = 0x10000u;
    __device__ __forceinline__ Key lookup(float x, float y) const {
        if (!ha.label) return kCanvas;
        int px, py;
        if (!hyb_rasterize(ha.h, x, y, px, py)) return kNone;
        if (px >= ha.h.resx || py >= ha.h.resy) return kBorderLabel;
        return __ldg(ha.label + (size_t)py * ha.h.resx + px);
    }
    template <class H>
    __device__ __forceinline__ void consume(bool valid, Key k, float x, float y, float v, const H& h,
                                            const DeferQ& q) const {
        h.add_warp(valid && k < kBorderLabel, (int)k, v);
        if (valid && k == kBorderLabel) q.push(x, y, v);
        else if (valid && k == kCanvas) map(x, y, v, h, q);
    }
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
                if (ha.canvas_s) {
                    const long long fq = isfinite(v) ? fixed_value(v, ha.scale) : 0ll;
                    atomicAdd(reinterpret_cast<unsigned long long*>(ha.canvas_s + pix), (unsigned long long)fq);
                }
            }
        }
    }
    template <class H>
    __device__ __forceinline__ void deferred(float x, float y, float v, const H& h) const {
        exact_probe(ix, x, y, v, h);
    }
};

// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Streaming pipeline.  One producer warp per block copies tiles of
// kPipeTile points (the location column and every column the query reads)
// from HBM into a ring of shared-memory stages with cp.async.bulk, completing
// on an mbarrier per stage; 16 consumer warps take each tile from shared
// memory (four points per thread), release the stage at once and run the
// per-point mapping.  Every wait is bounded: on timeout the kernel records
// the error and keeps its barrier sequence, so it always terminates.
constexpr int kPipeConsumers = 512;
constexpr int kPipeThreads = kPipeConsumers + 32;
constexpr int kPipeTile = kPipeConsumers * 4;

template <class M, bool AGG, bool SMEM>
__device__ __forceinline__ void map_group(const M& mp, const Hist<AGG, SMEM>& h, const DeferQ& dq, uint32_t mask,
                                          const float* x, const float* y, const float* val) {
    if constexpr (M::kTwoPhase) {
        typename M::Key key[4];
        #pragma unroll
        for (int q = 0; q < 4; ++q)
            if ((mask >> q) & 1u) key[q] = mp.lookup(x[q], y[q]);
        #pragma unroll
        for (int q = 0; q < 4; ++q) mp.consume(((mask >> q) & 1u) != 0u, key[q], x[q], y[q], val[q], h, dq);
    } else {
        #pragma unroll
        for (int q = 0; q < 4; ++q)
            if ((mask >> q) & 1u) mp.map(x[q], y[q], val[q], h, dq);
    }
}

__device__ __forceinline__ void agg4(const DevFilter& f, uint4 c, float* val) {
    val[0] = agg_value(f.aggr_typ, c.x); val[1] = agg_value(f.aggr_typ, c.y);
    val[2] = agg_value(f.aggr_typ, c.z); val[3] = agg_value(f.aggr_typ, c.w);
}

// All predicates of column c for four values (interval form).
__device__ __forceinline__ uint32_t column_mask4(const DevFilter& f, int c, uint4 v) {
    const int t = f.ctyp[c];
    const uint32_t lo = f.lo[c], sp = f.span[c];
    return ((order_key(t, v.x) - lo <= sp) ? 1u : 0u) | ((order_key(t, v.y) - lo <= sp) ? 2u : 0u) |
           ((order_key(t, v.z) - lo <= sp) ? 4u : 0u) | ((order_key(t, v.w) - lo <= sp) ? 8u : 0u);
}

__device__ __forceinline__ uint32_t filter_mask4(const DevFilter& f, int k, uint4 c) {
    const int op = f.op[k], ty = f.typ[k], cm = (int)((f.compat_mask >> k) & 1u);
    const uint32_t fv = f.val[k];
    return (pred_eval(op, ty, c.x, fv, cm) ? 1u : 0u) | (pred_eval(op, ty, c.y, fv, cm) ? 2u : 0u) |
           (pred_eval(op, ty, c.z, fv, cm) ? 4u : 0u) | (pred_eval(op, ty, c.w, fv, cm) ? 8u : 0u);
}

template <class M, bool AGG, bool SMEM>
__global__ void __launch_bounds__(kPipeThreads, 1)
k_points_pipe(PointArgs pa, M mp, int stages) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const DevFilter& f = pa.f;
    const int ncols = f.ncol + ((AGG && f.aggr_ci < 0) ? 1 : 0);
    const uint32_t col_bytes = kPipeTile * 4;
    const uint32_t stage_bytes = kPipeTile * 8 + ncols * col_bytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);
    uint64_t* empty = full + stages;
    unsigned char* stage0 = smem + 128;
    unsigned long long* s_sum = reinterpret_cast<unsigned long long*>(stage0 + (size_t)stages * stage_bytes);
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(s_sum + ((AGG && SMEM) ? pa.P : 0));
    float* s_q = reinterpret_cast<float*>(s_cnt + (SMEM ? pa.P : 0));
    DeferQ dq{s_q, s_q + kQueueCap, s_q + 2 * kQueueCap, reinterpret_cast<int*>(s_q + 3 * kQueueCap)};
    if (tid == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, kPipeConsumers / 32);
        }
        mbar_fence_init();
        if (M::kDefer) *dq.qn = 0;
    }
    if (SMEM) {
        for (int b = tid; b < pa.P; b += blockDim.x) {
            s_cnt[b] = 0u;
            if (AGG) s_sum[b] = 0ull;
        }
    }
    __syncthreads();
    Hist<AGG, SMEM> h{s_cnt, s_sum, pa.out_count, pa.out_sum, pa.out_nonfinite, pa.f.sum_scale};
    const uint64_t ntiles = pa.n / kPipeTile;

    if (warp == kPipeConsumers / 32) {
        // ---- producer ----
        if (lane == 0) {
            const uint64_t pol = l2_evict_first_policy();
            uint32_t it = 0;
            for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
                const int s = (int)(it % stages);
                const uint32_t k = it / stages;
                if (it >= (uint32_t)stages && !mbar_wait_ns(empty + s, (k - 1) & 1u, pa.wait_ns)) atomicOr(pa.err, 1);
                unsigned char* st = stage0 + (size_t)s * stage_bytes;
                const uint64_t base = tile * kPipeTile;
                mbar_arrive_expect_tx(full + s, stage_bytes);
                bulk_g2s(st, pa.xy + base, kPipeTile * 8, full + s, pol);
                for (int c = 0; c < f.ncol; ++c)
                    bulk_g2s(st + kPipeTile * 8 + c * col_bytes, f.col[c] + base, col_bytes, full + s, pol);
                if (AGG && f.aggr_ci < 0)
                    bulk_g2s(st + kPipeTile * 8 + f.ncol * col_bytes, f.aggr_col + base, col_bytes, full + s, pol);
            }
            // no copy may still be landing when the block exits: this wait keeps
            // the fixed, generous limit whatever the phase-wait limit is
            const uint32_t first = it > (uint32_t)stages ? it - stages : 0u;
            for (uint32_t j = first; j < it; ++j)
                if (!mbar_wait(full + (j % stages), (j / stages) & 1u)) atomicOr(pa.err, 1);
        }
        return;
    }

    // ---- consumers ----
    uint32_t it = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        const int s = (int)(it % stages);
        const uint32_t k = it / stages;
        const bool ok = mbar_wait_ns(full + s, k & 1u, pa.wait_ns);
        if (!ok && lane == 0) atomicOr(pa.err, 1);
        const unsigned char* st = stage0 + (size_t)s * stage_bytes;
        float x[4], y[4], val[4] = {0.f, 0.f, 0.f, 0.f};
        uint32_t mask = 0u;
        if (ok) {
            const float4 a = reinterpret_cast<const float4*>(st)[tid * 2];
            const float4 b = reinterpret_cast<const float4*>(st)[tid * 2 + 1];
            x[0] = a.x; y[0] = a.y; x[1] = a.z; y[1] = a.w;
            x[2] = b.x; y[2] = b.y; x[3] = b.z; y[3] = b.w;
            mask = 0xFu;
            #pragma unroll
            for (int c = 0; c < kMaxFilters; ++c) {
                if (c >= f.ncol) break;
                const uint4 v = reinterpret_cast<const uint4*>(st + kPipeTile * 8 + c * col_bytes)[tid];
                if (!f.general) mask &= column_mask4(f, c, v);
                else
                    for (int kk = f.pstart[c]; kk < f.pstart[c + 1]; ++kk) mask &= filter_mask4(f, kk, v);
                if (AGG && c == f.aggr_ci) agg4(f, v, val);
            }
            if (AGG && f.aggr_ci < 0)
                agg4(f, reinterpret_cast<const uint4*>(st + kPipeTile * 8 + f.ncol * col_bytes)[tid], val);
        } else {
            x[0] = x[1] = x[2] = x[3] = y[0] = y[1] = y[2] = y[3] = 0.f;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(empty + s);     // the stage is in registers: release it
        map_group(mp, h, dq, mask, x, y, val);
        if (M::kDefer) {
            named_sync(1, kPipeConsumers);
            while (*dq.qn >= kPipeConsumers) {
                const int q = *dq.qn - kPipeConsumers + tid;
                mp.deferred(dq.qx[q], dq.qy[q], dq.qv[q], h);
                named_sync(1, kPipeConsumers);
                if (tid == 0) *dq.qn -= kPipeConsumers;
                named_sync(1, kPipeConsumers);
            }
        }
    }
    // tail points (n not a multiple of the tile) with plain loads.  The trip
    // count is uniform per warp (lanes past the end take an empty mask): the
    // mappers' warp votes need every lane of the warp.
    if (blockIdx.x == 0) {
        const uint64_t t0 = ntiles * kPipeTile;
        for (uint64_t wbase = t0 + (uint64_t)(tid - lane) * 4; wbase < pa.n; wbase += (uint64_t)kPipeConsumers * 4) {
            const uint64_t base = wbase + (uint64_t)lane * 4;
            float x[4], y[4], val[4] = {0.f, 0.f, 0.f, 0.f};
            uint32_t mask = 0u;
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
            map_group(mp, h, dq, mask, x, y, val);
        }
    }
    if (M::kDefer) {
        named_sync(1, kPipeConsumers);
        // the tail may have queued up to 4 points per thread: drain in batches
        while (*dq.qn > 0) {
            const int cnt = min(*dq.qn, kPipeConsumers);
            const int q = *dq.qn - cnt + tid;
            if (tid < cnt) mp.deferred(dq.qx[q], dq.qy[q], dq.qv[q], h);
            named_sync(1, kPipeConsumers);
            if (tid == 0) *dq.qn -= cnt;
            named_sync(1, kPipeConsumers);
        }
    }
    if (SMEM) {
        named_sync(1, kPipeConsumers);
        for (int b = tid; b < pa.P; b += kPipeConsumers) {
            uint32_t c = s_cnt[b];
            if (c) {
                if (pa.out_count32) atomicAdd(pa.out_count32 + b, c);
                else atomicAdd(pa.out_count + b, (unsigned long long)c);
            }
            if (AGG) {
                unsigned long long sv = s_sum[b];
                if (c) atomicAdd(pa.out_sum + b, sv);
            }
        }
    }
}

// Plain streaming kernel: every thread takes NG groups of four consecutive
// points per iteration (group g of a block covers a contiguous run of
// BLOCK*4 points), issues all column loads, then all per-point lookups, then
// consumes them.
template <class M, bool AGG, bool SMEM, int NG, int BLOCK>
__global__ void __launch_bounds__(BLOCK)
k_points(PointArgs pa, M mp) {
    extern __shared__ unsigned long long smem_d[];
    unsigned long long* s_sum = smem_d;
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(smem_d + ((AGG && SMEM) ? pa.P : 0));
    float* s_q = reinterpret_cast<float*>(s_cnt + (SMEM ? pa.P : 0));
    constexpr int QCAP = BLOCK * (1 + 4 * NG);
    DeferQ dq{s_q, s_q + QCAP, s_q + 2 * QCAP, reinterpret_cast<int*>(s_q + 3 * QCAP)};
    if (SMEM) {
        for (int b = threadIdx.x; b < pa.P; b += BLOCK) {
            s_cnt[b] = 0u;
            if (AGG) s_sum[b] = 0ull;
        }
    }
    if (M::kDefer && threadIdx.x == 0) *dq.qn = 0;
    __syncthreads();
    Hist<AGG, SMEM> h{s_cnt, s_sum, pa.out_count, pa.out_sum, pa.out_nonfinite, pa.f.sum_scale};
    const DevFilter& f = pa.f;
    constexpr uint64_t per_iter = (uint64_t)BLOCK * 4 * NG;
    // block-uniform trip count: every thread of a block runs the same iterations
    for (uint64_t tb = (uint64_t)blockIdx.x * per_iter; tb < pa.n; tb += (uint64_t)gridDim.x * per_iter) {
        if (pa.zones) {
            // skip rows whose zones lie apart from the query's reach (uniform)
            const uint64_t z0 = (pa.row0 + tb) >> kZoneShift;
            const uint64_t z1 = (pa.row0 + min(tb + per_iter, pa.n) - 1) >> kZoneShift;
            bool meets = false;
            for (uint64_t z = z0; z <= z1; ++z) {
                const float4 b = __ldg(pa.zones + z);
                meets |= !(b.z < pa.qbox.x || b.x > pa.qbox.z || b.w < pa.qbox.y || b.y > pa.qbox.w);
            }
            if (!meets) continue;
        }
        float x[NG][4], y[NG][4], val[NG][4];
        uint32_t mask[NG];
        if (tb + per_iter <= pa.n) {
            #pragma unroll
            for (int g = 0; g < NG; ++g) {
                const uint64_t base = tb + (uint64_t)g * BLOCK * 4 + (uint64_t)threadIdx.x * 4;
                // column data is read once: evict-first so it does not push the
                // label map / grid out of L2
                const float4 a = __ldcs(reinterpret_cast<const float4*>(pa.xy + base));
                const float4 b = __ldcs(reinterpret_cast<const float4*>(pa.xy + base + 2));
                x[g][0] = a.x; y[g][0] = a.y; x[g][1] = a.z; y[g][1] = a.w;
                x[g][2] = b.x; y[g][2] = b.y; x[g][3] = b.z; y[g][3] = b.w;
                val[g][0] = val[g][1] = val[g][2] = val[g][3] = 0.f;
                uint32_t m = 0xFu;
                #pragma unroll
                for (int c = 0; c < kMaxFilters; ++c) {
                    if (c >= f.ncol) break;
                    const uint4 v = __ldcs(reinterpret_cast<const uint4*>(f.col[c] + base));
                    if (!f.general) m &= column_mask4(f, c, v);
                    else
                        for (int k = f.pstart[c]; k < f.pstart[c + 1]; ++k) m &= filter_mask4(f, k, v);
                    if (AGG && c == f.aggr_ci) agg4(f, v, val[g]);
                }
                if (AGG && f.aggr_ci < 0) agg4(f, __ldcs(reinterpret_cast<const uint4*>(f.aggr_col + base)), val[g]);
                mask[g] = m;
            }
        } else {
            #pragma unroll
            for (int g = 0; g < NG; ++g) {
                const uint64_t base = tb + (uint64_t)g * BLOCK * 4 + (uint64_t)threadIdx.x * 4;
                mask[g] = 0u;
                #pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint64_t i = base + q;
                    x[g][q] = 0.f; y[g][q] = 0.f; val[g][q] = 0.f;
                    if (i >= pa.n) continue;
                    const float2 p = __ldg(pa.xy + i);
                    x[g][q] = p.x; y[g][q] = p.y;
                    if (filter_point(f, i)) mask[g] |= 1u << q;
                    if (AGG) val[g][q] = agg_value(f.aggr_typ, __ldg(f.aggr_col + i));
                }
            }
        }
        if constexpr (M::kTwoPhase) {
            typename M::Key key[NG][4];
            #pragma unroll
            for (int g = 0; g < NG; ++g)
                #pragma unroll
                for (int q = 0; q < 4; ++q)
                    if ((mask[g] >> q) & 1u) key[g][q] = mp.lookup(x[g][q], y[g][q]);
            #pragma unroll
            for (int g = 0; g < NG; ++g)
                #pragma unroll
                for (int q = 0; q < 4; ++q)
                    mp.consume(((mask[g] >> q) & 1u) != 0u, key[g][q], x[g][q], y[g][q], val[g][q], h, dq);
        } else {
            #pragma unroll
            for (int g = 0; g < NG; ++g)
                #pragma unroll
                for (int q = 0; q < 4; ++q)
                    if ((mask[g] >> q) & 1u) mp.map(x[g][q], y[g][q], val[g][q], h, dq);
        }
        if (M::kDefer) {
            // drain full batches of deferred points, one point per thread
            __syncthreads();
            while (*dq.qn >= BLOCK) {
                const int s = *dq.qn - BLOCK + (int)threadIdx.x;
                mp.deferred(dq.qx[s], dq.qy[s], dq.qv[s], h);
                __syncthreads();
                if (threadIdx.x == 0) *dq.qn -= BLOCK;
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
        for (int b = threadIdx.x; b < pa.P; b += BLOCK) {
            uint32_t c = s_cnt[b];
            if (c) {
                if (pa.out_count32) atomicAdd(pa.out_count32 + b, c);
                else atomicAdd(pa.out_count + b, (unsigned long long)c);
            }
            if (AGG) {
                unsigned long long sv = s_sum[b];
                if (c) atomicAdd(pa.out_sum + b, sv);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// The launch helpers below are static: each translation unit that includes
// this header launches its own kernel instances and keeps its own copy.
static int g_max_smem_optin = -1;

static size_t hist_bytes(int P, bool agg) { return (size_t)P * (agg ? 12 : 4); }
static size_t queue_bytes(bool defer, int qcap = kQueueCap) { return defer ? (size_t)qcap * 12 + 16 : 0; }

template <class M, bool AGG, bool SMEM, int NG, int BLOCK>
static void launch_plain_t(const PointArgs& pa, const M& mp, int sms, cudaStream_t st) {
    constexpr int QCAP = BLOCK * (1 + 4 * NG);
    size_t smem = (SMEM ? hist_bytes(pa.P, AGG) : 0) + queue_bytes(M::kDefer, QCAP);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_points<M, AGG, SMEM, NG, BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_points<M, AGG, SMEM, NG, BLOCK>, BLOCK, smem);
    if (per_sm < 1) per_sm = 1;
    const uint64_t per_iter = (uint64_t)BLOCK * 4 * NG;
    uint64_t need = (pa.n + per_iter - 1) / per_iter;
    uint64_t blocks = (uint64_t)sms * per_sm;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    k_points<M, AGG, SMEM, NG, BLOCK><<<(unsigned)blocks, BLOCK, smem, st>>>(pa, mp);
    ++g_kernel_launches;
}

// Point-kernel shape: 0 = plain, 4 points x 256 threads; 2 = bulk-copy
// pipeline; 3 = plain, 4 points x 512 threads.  Defaults measured on GB300
// (config-2 query, 100M points): the hybrid pass is fastest with 3 (0.833 ms
// vs 0.910 ms for 0), the raster-label and index passes with 0 (0.65 ms vs
// 0.79 ms; 2.07 ms vs 2.36 ms).  Two more plain shapes were measured and
// dropped: 8 points x 256 threads (hybrid 1.077 ms) and 4 points x 128
// threads (0.949 ms).  PointArgs::shape (rj_set_tuning RJ_TUNE_POINT_SHAPE)
// overrides the default for every mapper; every shape computes the same
// result.
template <class M>
static int point_variant(const PointArgs& pa) {
    const int v = pa.shape;
    if (v == 0 || v == 2 || v == 3) return v;
    return M::kDefer ? 3 : 0;   // the hybrid mapper defers border points to a block queue
}

template <class M, bool AGG, bool SMEM>
static void launch_points_t(const PointArgs& pa, const M& mp, int sms, cudaStream_t st) {
    if (point_variant<M>(pa) == 3) launch_plain_t<M, AGG, SMEM, 1, 512>(pa, mp, sms, st);
    else launch_plain_t<M, AGG, SMEM, 1, 256>(pa, mp, sms, st);
}

template <class M, bool AGG, bool SMEM>
static bool launch_pipe_t(const PointArgs& pa, const M& mp, int sms, cudaStream_t st) {
    const int ncols = pa.f.ncol + ((AGG && pa.f.aggr_ci < 0) ? 1 : 0);
    const size_t stage_bytes = (size_t)kPipeTile * 8 + (size_t)ncols * kPipeTile * 4;
    const size_t fixed = 128 + (SMEM ? hist_bytes(pa.P, AGG) : 0) + queue_bytes(M::kDefer);
    const size_t avail = (size_t)std::max(g_max_smem_optin - 1024, 0);
    if (fixed + 2 * stage_bytes > avail) return false;
    const int stages = (int)std::min<size_t>(4, (avail - fixed) / stage_bytes);
    const size_t smem = fixed + (size_t)stages * stage_bytes;
    if (cudaFuncSetAttribute(k_points_pipe<M, AGG, SMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    uint64_t ntiles = pa.n / kPipeTile;
    uint64_t blocks = std::min<uint64_t>((uint64_t)sms, std::max<uint64_t>(ntiles, 1));
    k_points_pipe<M, AGG, SMEM><<<(unsigned)blocks, kPipeThreads, smem, st>>>(pa, mp, stages);
    ++g_kernel_launches;
    return true;
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
    // bulk-copy pipeline for tables of at least one tile per SM (columns are 16-byte aligned)
    if (point_variant<M>(pa) == 2 && pa.err && pa.n >= (uint64_t)kPipeTile * sms && smem_ok) {
        bool launched = agg ? launch_pipe_t<M, true, true>(pa, mp, sms, st) : launch_pipe_t<M, false, true>(pa, mp, sms, st);
        if (launched) return;
    }
    if (agg) {
        if (smem_ok) launch_points_t<M, true, true>(pa, mp, sms, st);
        else launch_points_t<M, true, false>(pa, mp, sms, st);
    } else {
        if (smem_ok) launch_points_t<M, false, true>(pa, mp, sms, st);
        else launch_points_t<M, false, false>(pa, mp, sms, st);
    }
}

}  // namespace rj
