// rj_point_map.cuh -- per-point building blocks shared by the point kernels:
// per-polygon histograms (shared-memory or global, warp-aggregated), the
// canvas tile visit of a point, and the raster splat / label mappers.
#pragma once
#include "rj_device.cuh"
#include "rj_launch.h"

namespace rj {

// Sum of a 64-bit value over the lanes of `peers` (a __match_any_sync group
// inside `active`; every lane of `active` calls this), valid at the group's
// lowest lane.  Small groups (random rows): the leader pulls its peers' values
// with shuffles, as many rounds as the largest group has members.  Large
// groups (spatially clustered rows): one warp reduction per 22/22/20-bit
// piece of the value (each piece sums within 32 bits over at most 32 lanes;
// the pieces recombine modulo 2^64, the two's-complement sum); groups of one
// lane skip it.
__device__ __forceinline__ long long group_sum(unsigned active, unsigned peers, long long q) {
    const int lane = threadIdx.x & 31;
    const unsigned gsize = (unsigned)__popc(peers);
    if (__all_sync(active, gsize == 1u)) return q;          // no two lanes share a key (a vote)
    const unsigned maxg = __reduce_max_sync(active, gsize);
    if (maxg <= 4u) {
        const int leader = __ffs(peers) - 1;
        long long sum = q;
        unsigned rest = (lane == leader) ? (peers & (peers - 1u)) : 0u;
        while (__any_sync(active, rest != 0u)) {
            const int src = rest ? __ffs(rest) - 1 : lane;
            const long long o = __shfl_sync(active, q, src);
            if (rest) {
                sum += o;
                rest &= rest - 1u;
            }
        }
        return sum;
    }
    if (gsize == 1u) return q;
    const unsigned long long u = (unsigned long long)q;
    const unsigned s0 = __reduce_add_sync(peers, (unsigned)(u & 0x3FFFFFull));
    const unsigned s1 = __reduce_add_sync(peers, (unsigned)((u >> 22) & 0x3FFFFFull));
    const unsigned s2 = __reduce_add_sync(peers, (unsigned)(u >> 44));
    return (long long)((unsigned long long)s0 + ((unsigned long long)s1 << 22) + ((unsigned long long)s2 << 44));
}

// TOUCH: record the keys whose shared count leaves zero, so that a flush
// visits only them (the batched passes); the add then needs the old count
// back, so the single-query passes keep the plain, non-returning add.
template <bool AGG, bool SMEM, bool TOUCH = false>
struct Hist {
    uint32_t* s_cnt;
    unsigned long long* s_sum;
    unsigned long long* g_cnt;
    unsigned long long* g_sum;
    double* g_nonfinite;
    float scale;
    int* s_touched = nullptr;
    int* s_ntouched = nullptr;
    __device__ __forceinline__ void count(int p, unsigned c) const {
        if (TOUCH) {
            const unsigned old = atomicAdd(s_cnt + p, c);
            if (old == 0u) s_touched[atomicAdd(s_ntouched, 1)] = p;
        } else {
            atomicAdd(s_cnt + p, c);
        }
    }
    __device__ __forceinline__ long long fixq(int p, float v) const {
        if (!isfinite(v)) {
            atomicAdd(g_nonfinite + p, (double)v);
            return 0;
        }
        return fixed_value(v, scale);
    }
    __device__ __forceinline__ void add(int p, float v) const {
        if (SMEM) {
            count(p, 1u);
            if (AGG) atomicAdd(s_sum + p, (unsigned long long)fixq(p, v));
        } else {
            atomicAdd(g_cnt + p, 1ull);
            if (AGG) atomicAdd(g_sum + p, (unsigned long long)fixq(p, v));
        }
    }
    // Warp-aggregated add; every lane of the warp calls it (converged).  Lanes
    // with the same polygon form a group: the lowest lane adds the group's
    // count and its fixed-point sum with one atomic each.
    __device__ __forceinline__ void add_warp(bool valid, int p, float v) const {
        const unsigned active = __ballot_sync(0xffffffffu, valid);
        if (!valid) return;
        const int lane = threadIdx.x & 31;
        const unsigned peers = __match_any_sync(active, p);
        const int leader = __ffs(peers) - 1;
        long long sum = 0;
        if (AGG) sum = group_sum(active, peers, fixq(p, v));
        if (lane == leader) {
            const unsigned c = (unsigned)__popc(peers);
            if (SMEM) {
                count(p, c);
                if (AGG) atomicAdd(s_sum + p, (unsigned long long)sum);
            } else {
                atomicAdd(g_cnt + p, (unsigned long long)c);
                if (AGG) atomicAdd(g_sum + p, (unsigned long long)sum);
            }
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
// Additive splat of points into a canvas (point count u32 and fixed-point
// sum per pixel).  Single-tile canvases: the pixel is looked up first, lanes
// of a warp on the same pixel are merged, and the group's leader adds once;
// with `priv` the adds go to the block's shared histogram, indexed by pixel,
// which the kernel flushes into the canvas (small canvases, where global
// atomics on a few thousand pixels would serialise).  Multi-tile canvases:
// one add per tile whose window holds the point.
struct SplatMapper {
    static constexpr bool kDefer = false;
    static constexpr bool kTwoPhase = true;
    CanvasXf cx;
    uint32_t* canvas_c;
    long long* canvas_s;    // fixed-point sums (non-finite values are not representable on a canvas)
    float scale;
    double* nonfinite;
    int priv;
    using Key = uint32_t;
    static constexpr Key kNone = 0xFFFFFFFFu;
    static constexpr Key kMulti = 0xFFFFFFFEu;
    __device__ __forceinline__ Key lookup(float x, float y) const {
        if (cx.splitx != 1 || cx.splity != 1) return kMulti;
        float wx = win_coord(x, cx.col0.x, cx.col0.y, cx.col0.z);
        float wy = win_coord(y, cx.row0.x, cx.row0.y, cx.row0.z);
        if (!(wx > -1.0f && wx < (float)cx.resx + 1.0f && wy > -1.0f && wy < (float)cx.resy + 1.0f)) return kNone;
        int px = pix_of(snap_win(wx)), py = pix_of(snap_win(wy));
        if (px < 0 || px >= cx.resx || py < 0 || py >= cx.resy) return kNone;
        return (Key)py * (Key)cx.resx + (Key)px;
    }
    template <class H>
    __device__ __forceinline__ void consume(bool valid, Key k, float x, float y, float v, const H& h,
                                            const DeferQ& dq) const {
        const bool one = valid && k < kMulti;
        const unsigned active = __ballot_sync(0xffffffffu, one);
        if (one) {
            const long long q = (canvas_s && isfinite(v)) ? fixed_value(v, scale) : 0ll;
            const unsigned peers = __match_any_sync(active, k);
            const long long sum = group_sum(active, peers, q);
            if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) {
                const unsigned c = (unsigned)__popc(peers);
                if (priv) {
                    h.count((int)k, c);
                    if (canvas_s) atomicAdd(h.s_sum + k, (unsigned long long)sum);
                } else {
                    atomicAdd(canvas_c + k, c);
                    if (canvas_s) atomicAdd(reinterpret_cast<unsigned long long*>(canvas_s + k), (unsigned long long)sum);
                }
            }
        }
        if (valid && k == kMulti) map(x, y, v, h, dq);
    }
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H&, const DeferQ&) const {
        const size_t tile_px = (size_t)cx.resx * cx.resy;
        const long long q = canvas_s ? (isfinite(v) ? fixed_value(v, scale) : 0ll) : 0ll;
        canvas_visit(cx, x, y, [&](int t, int px, int py) {
            size_t pix = (size_t)t * tile_px + (size_t)py * cx.resx + px;
            atomicAdd(canvas_c + pix, 1u);
            if (canvas_s) atomicAdd(reinterpret_cast<unsigned long long*>(canvas_s + pix), (unsigned long long)q);
        });
    }
    template <class H>
    __device__ __forceinline__ void deferred(float, float, float, const H&) const {}
};

struct LabelMapper {
    static constexpr bool kDefer = false;
    static constexpr bool kTwoPhase = true;
    CanvasXf cx;
    const uint16_t* label;
    // two-phase form: lookup issues the label gather, consume uses it
    using Key = uint32_t;
    static constexpr Key kNone = 0xFFFFu;
    static constexpr Key kMulti = 0x10000u;
    __device__ __forceinline__ Key lookup(float x, float y) const {
        if (cx.splitx != 1 || cx.splity != 1) return kMulti;
        float wx = win_coord(x, cx.col0.x, cx.col0.y, cx.col0.z);
        float wy = win_coord(y, cx.row0.x, cx.row0.y, cx.row0.z);
        if (!(wx > -1.0f && wx < (float)cx.resx + 1.0f && wy > -1.0f && wy < (float)cx.resy + 1.0f)) return kNone;
        int px = pix_of(snap_win(wx)), py = pix_of(snap_win(wy));
        if (px < 0 || px >= cx.resx || py < 0 || py >= cx.resy) return kNone;
        return __ldg(label + (size_t)py * cx.resx + px);
    }
    template <class H>
    __device__ __forceinline__ void consume(bool valid, Key k, float x, float y, float v, const H& h,
                                            const DeferQ& q) const {
        h.add_warp(valid && k < kBorderLabel, (int)k, v);
        if (valid && k == kMulti) map(x, y, v, h, q);
    }
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


// Tiered canvas, label form: block code, then the pixel label of a mixed
// block's slot.
__device__ __forceinline__ uint32_t tier_label_at(const TierArgs& tr, int resx, int resy, size_t blk0, int px, int py) {
    (void)resx; (void)resy;
    const uint32_t code = __ldg(tr.code + blk0 + (size_t)(py >> 4) * tr.bw + (px >> 4));
    if (code == kTierEmpty) return kEmptyLabel;
    if (code & kTierMixed) {
        if (code == kTierMulti) return kEmptyLabel;   // never in label form (overlap takes the canvas form)
        return __ldg(tr.plabel + (size_t)(code & ~kTierMixed) * 256 + (size_t)(py & 15) * 16 + (px & 15));
    }
    return code;
}

struct TierLabelMapper {
    static constexpr bool kDefer = false;
    static constexpr bool kTwoPhase = true;
    CanvasXf cx;
    TierArgs tr;
    using Key = uint32_t;
    static constexpr Key kNone = 0xFFFFu;
    static constexpr Key kMulti = 0x10000u;
    __device__ __forceinline__ Key lookup(float x, float y) const {
        if (cx.splitx != 1 || cx.splity != 1) return kMulti;
        float wx = win_coord(x, cx.col0.x, cx.col0.y, cx.col0.z);
        float wy = win_coord(y, cx.row0.x, cx.row0.y, cx.row0.z);
        if (!(wx > -1.0f && wx < (float)cx.resx + 1.0f && wy > -1.0f && wy < (float)cx.resy + 1.0f)) return kNone;
        int px = pix_of(snap_win(wx)), py = pix_of(snap_win(wy));
        if (px < 0 || px >= cx.resx || py < 0 || py >= cx.resy) return kNone;
        return tier_label_at(tr, cx.resx, cx.resy, 0, px, py);
    }
    template <class H>
    __device__ __forceinline__ void consume(bool valid, Key k, float x, float y, float v, const H& h,
                                            const DeferQ& q) const {
        h.add_warp(valid && k < kBorderLabel, (int)k, v);
        if (valid && k == kMulti) map(x, y, v, h, q);
    }
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H& h, const DeferQ&) const {
        const size_t tile_blk = (size_t)tr.bw * tr.bh;
        canvas_visit(cx, x, y, [&](int t, int px, int py) {
            const uint32_t lab = tier_label_at(tr, cx.resx, cx.resy, (size_t)t * tile_blk, px, py);
            if (lab != kEmptyLabel) h.add((int)lab, v);
        });
    }
    template <class H>
    __device__ __forceinline__ void deferred(float, float, float, const H&) const {}
};

// Tiered canvas, canvas form: every point adds to its block's sums (merged
// per warp); points of mixed blocks also to their pixel in the block's slot.
struct TierSplatMapper {
    static constexpr bool kDefer = false;
    static constexpr bool kTwoPhase = true;
    CanvasXf cx;
    TierArgs tr;
    float scale;
    using Key = uint32_t;                               // pixel index in the tile
    static constexpr Key kNone = 0xFFFFFFFFu;
    static constexpr Key kMulti = 0xFFFFFFFEu;
    __device__ __forceinline__ Key lookup(float x, float y) const {
        if (cx.splitx != 1 || cx.splity != 1) return kMulti;
        float wx = win_coord(x, cx.col0.x, cx.col0.y, cx.col0.z);
        float wy = win_coord(y, cx.row0.x, cx.row0.y, cx.row0.z);
        if (!(wx > -1.0f && wx < (float)cx.resx + 1.0f && wy > -1.0f && wy < (float)cx.resy + 1.0f)) return kNone;
        int px = pix_of(snap_win(wx)), py = pix_of(snap_win(wy));
        if (px < 0 || px >= cx.resx || py < 0 || py >= cx.resy) return kNone;
        return (Key)py * (Key)cx.resx + (Key)px;
    }
    // A point's count (and sum) goes to the pixel slot of a mixed block, else
    // to the block's total; a block no polygon reaches keeps nothing (no
    // polygon reads it).
    __device__ static __forceinline__ bool tier_mixed(uint32_t code) {
        return (code & kTierMixed) && code < kTierMulti;
    }
    __device__ __forceinline__ void pixel_add(uint32_t code, int px, int py, long long q) const {
        const size_t at = (size_t)(code & ~kTierMixed) * 256 + (size_t)(py & 15) * 16 + (px & 15);
        atomicAdd(tr.pcnt + at, 1u);
        if (tr.psum) atomicAdd(reinterpret_cast<unsigned long long*>(tr.psum + at), (unsigned long long)q);
    }
    template <class H>
    __device__ __forceinline__ void consume(bool valid, Key k, float x, float y, float v, const H& h,
                                            const DeferQ& dq) const {
        const bool one = valid && k < kMulti;
        int px = 0, py = 0;
        uint32_t b = 0, code = kTierEmpty;
        if (one) {
            px = (int)(k % (Key)cx.resx);
            py = (int)(k / (Key)cx.resx);
            b = (uint32_t)((py >> 4) * tr.bw + (px >> 4));
            code = __ldg(tr.code + b);
        }
        const bool mixed = tier_mixed(code);
        const bool blk = !mixed && code != kTierEmpty;
        const long long q = ((mixed || blk) && tr.bsum && isfinite(v)) ? fixed_value(v, scale) : 0ll;
        const unsigned active = __ballot_sync(0xffffffffu, blk);
        if (blk) {
            const unsigned peers = __match_any_sync(active, b);
            const long long sum = group_sum(active, peers, q);
            if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) {
                atomicAdd(tr.bcnt + b, (unsigned)__popc(peers));
                if (tr.bsum) atomicAdd(reinterpret_cast<unsigned long long*>(tr.bsum + b), (unsigned long long)sum);
            }
        }
        if (mixed) pixel_add(code, px, py, q);
        if (valid && k == kMulti) map(x, y, v, h, dq);
    }
    template <class H>
    __device__ __forceinline__ void map(float x, float y, float v, const H&, const DeferQ&) const {
        const size_t tile_blk = (size_t)tr.bw * tr.bh;
        const long long q = (tr.bsum && isfinite(v)) ? fixed_value(v, scale) : 0ll;
        canvas_visit(cx, x, y, [&](int t, int px, int py) {
            const size_t b = (size_t)t * tile_blk + (size_t)(py >> 4) * tr.bw + (px >> 4);
            const uint32_t code = __ldg(tr.code + b);
            if (tier_mixed(code)) {
                pixel_add(code, px, py, q);
            } else if (code != kTierEmpty) {
                atomicAdd(tr.bcnt + b, 1u);
                if (tr.bsum) atomicAdd(reinterpret_cast<unsigned long long*>(tr.bsum + b), (unsigned long long)q);
            }
        });
    }
    template <class H>
    __device__ __forceinline__ void deferred(float, float, float, const H&) const {}
};

}  // namespace rj
