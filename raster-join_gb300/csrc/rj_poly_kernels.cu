// rj_poly_kernels.cu -- polygon-side kernels.
//
//  * k_transform_vertices : world -> per-tile window coordinates (float and
//    1/256-pixel fixed point), the vertex stage of polygon.vert:9-13.
//  * k_poly_pass<MODE>    : edge-function coverage of pixel centres, one warp
//    per (tile, polygon), rows processed in bands whose edges are staged in
//    shared memory.  MODE_REDUCE sums canvas counts/sums of covered pixels
//    into the polygon (polygon.frag:12-27), MODE_LABEL writes a polygon label
//    per covered pixel, MODE_BOUNDS additionally runs the error-bound outline
//    pass (line-bound.frag:243-286).
//  * grid index build     : index-size.glsl + create-index.glsl as a CSR grid.
//  * hybrid border mask   : outline pass of HybridJoin::drawOutline
//    (HybridJoin.cpp:197-268) as a conservative supercover + dilation.
#include <climits>
#include <cstdio>

#include "rj_device.cuh"
#include "rj_launch.h"

namespace rj {

thread_local int g_kernel_launches = 0;

// ---------------------------------------------------------------------------
__global__ void k_transform_vertices(const float2* __restrict__ verts, int V,
                                     const float4* __restrict__ colxf,  // per tile column: (sx, tx, hx, -)
                                     const float4* __restrict__ rowxf,  // per tile row:    (sy, ty, hy, -)
                                     int splitx, int T,
                                     int2* __restrict__ wv, float2* __restrict__ wf) {
    size_t total = (size_t)T * V;
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
        int t = (int)(g / V);
        int v = (int)(g - (size_t)t * V);
        int cx = t % splitx, cy = t / splitx;
        float4 cxf = __ldg(colxf + cx), ryf = __ldg(rowxf + cy);
        float2 p = __ldg(verts + v);
        float wx = win_coord(p.x, cxf.x, cxf.y, cxf.z);
        float wy = win_coord(p.y, ryf.x, ryf.y, ryf.z);
        wv[g] = make_int2(snap_win(wx), snap_win(wy));
        if (wf) wf[g] = make_float2(wx, wy);
    }
}

// ---------------------------------------------------------------------------
// Cohen-Sutherland clip of an edge against one pixel and the area fraction on
// one side, computeFraction line-bound.frag:51-211, in fp32 window units.
__device__ __forceinline__ int cs_outcode(float x, float y, float xmin, float ymin, float xmax, float ymax) {
    int code = 0;
    if (x < xmin) code |= 1;
    else if (x > xmax) code |= 2;
    if (y < ymin) code |= 4;
    else if (y > ymax) code |= 8;
    return code;
}

__device__ __forceinline__ float tri_area(float ax, float ay, float bx, float by, float cx, float cy) {
    // abs(0.5 * length(cross(b - a, c - a))) with z = 0
    float ix = __fsub_rn(bx, ax), iy = __fsub_rn(by, ay);
    float jx = __fsub_rn(cx, ax), jy = __fsub_rn(cy, ay);
    float cz = __fsub_rn(__fmul_rn(ix, jy), __fmul_rn(iy, jx));
    return fabsf(__fmul_rn(0.5f, cz));
}

__device__ bool compute_fraction(float x0, float y0, float x1, float y1,
                                 float xmin, float ymin, float xmax, float ymax, float& frac) {
    int oc0 = cs_outcode(x0, y0, xmin, ymin, xmax, ymax);
    int oc1 = cs_outcode(x1, y1, xmin, ymin, xmax, ymax);
    bool accept = false;
    frac = 0.0f;
    for (int it = 0; it < 16; ++it) {   // the reference loops until accept/reject
        if ((oc0 | oc1) == 0) { accept = true; break; }
        if ((oc0 & oc1) != 0) break;
        float x = 0.0f, y = 0.0f;
        int out = (oc0 != 0) ? oc0 : oc1;
        if (out & 8) {
            x = __fadd_rn(x0, __fdiv_rn(__fmul_rn(__fsub_rn(x1, x0), __fsub_rn(ymax, y0)), __fsub_rn(y1, y0)));
            y = ymax;
        } else if (out & 4) {
            x = __fadd_rn(x0, __fdiv_rn(__fmul_rn(__fsub_rn(x1, x0), __fsub_rn(ymin, y0)), __fsub_rn(y1, y0)));
            y = ymin;
        } else if (out & 2) {
            y = __fadd_rn(y0, __fdiv_rn(__fmul_rn(__fsub_rn(y1, y0), __fsub_rn(xmax, x0)), __fsub_rn(x1, x0)));
            x = xmax;
        } else if (out & 1) {
            y = __fadd_rn(y0, __fdiv_rn(__fmul_rn(__fsub_rn(y1, y0), __fsub_rn(xmin, x0)), __fsub_rn(x1, x0)));
            x = xmin;
        }
        if (out == oc0) { x0 = x; y0 = y; oc0 = cs_outcode(x0, y0, xmin, ymin, xmax, ymax); }
        else            { x1 = x; y1 = y; oc1 = cs_outcode(x1, y1, xmin, ymin, xmax, ymax); }
    }
    if (!accept) return false;
    if (x0 > x1) { float t = x0; x0 = x1; x1 = t; t = y0; y0 = y1; y1 = t; }
    float v1x = 0, v1y = 0, v2x = 0, v2y = 0, v3x = 0, v3y = 0, v4x = 0, v4y = 0;
    bool tri = false, compute = true;
    if (x0 == xmin) {
        if (x1 == xmax) {                      // horizontal cut
            v1x = xmin; v1y = ymin; v2x = xmax; v2y = ymin; v3x = x1; v3y = y1; v4x = x0; v4y = y0;
        } else if (y1 == ymax) {
            v1x = xmin; v1y = ymax; v2x = x0; v2y = y0; v3x = x1; v3y = y1; tri = true;
        } else if (y1 == ymin) {
            v1x = xmin; v1y = ymin; v2x = x0; v2y = y0; v3x = x1; v3y = y1; tri = true;
        } else {
            compute = false;
        }
    } else if (x1 == xmax) {
        if (y0 == ymax) {
            v1x = xmax; v1y = ymax; v2x = x0; v2y = y0; v3x = x1; v3y = y1; tri = true;
        } else if (y0 == ymin) {
            v1x = xmax; v1y = ymin; v2x = x1; v2y = y1; v3x = x0; v3y = y0; tri = true;
        } else {
            compute = false;
        }
    } else if (y0 == ymin && y1 == ymax) {     // vertical cut
        v1x = xmin; v1y = ymin; v2x = xmin; v2y = ymax; v3x = x1; v3y = y1; v4x = x0; v4y = y0;
    } else if (y1 == ymin && y0 == ymax) {     // vertical cut
        v1x = xmin; v1y = ymin; v2x = xmin; v2y = ymax; v3x = x0; v3y = y0; v4x = x1; v4y = y1;
    } else {
        compute = false;
    }
    frac = 0.5f;
    if (compute) {
        float area = tri_area(v1x, v1y, v2x, v2y, v3x, v3y);
        if (!tri) area = __fadd_rn(area, tri_area(v1x, v1y, v3x, v3y, v4x, v4y));
        frac = __fdiv_rn(area, __fmul_rn(__fsub_rn(ymax, ymin), __fsub_rn(xmax, xmin)));
    }
    return true;
}

// ---------------------------------------------------------------------------
constexpr int kPolyWarps = 8;
constexpr int kBand = 16;          // pixel rows per work item
constexpr int kBandCap = 256;      // staged edges per warp
constexpr int kCrossCap = 512;     // crossings per row per warp (sorted into spans)
// dynamic shared memory of k_poly_pass: per warp the staged edges, their
// indices and one row's crossings
constexpr size_t kPolySmem = (size_t)kPolyWarps * (kBandCap * (sizeof(int4) + sizeof(int)) + kCrossCap * sizeof(int));

// Ascending sort of buf[0, m) by one warp (bitonic network in shared memory,
// m padded to a power of two with INT_MAX).
__device__ __forceinline__ void warp_sort_ints(int* buf, int m, int lane) {
    int mp = 2;
    while (mp < m) mp <<= 1;
    for (int i = m + lane; i < mp; i += 32) buf[i] = INT_MAX;
    __syncwarp();
    for (int k = 2; k <= mp; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < mp; i += 32) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const int x = buf[i], y = buf[ixj];
                    const bool up = (i & k) == 0;
                    if ((x > y) == up) {
                        buf[i] = y;
                        buf[ixj] = x;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// Per (tile, polygon): pixel column range that can be covered, rows to visit
// and rows whose centre line the polygon can cross; number of row bands.
template <int MODE>
__global__ void k_poly_info(PolyPassArgs a) {
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int TP = a.T * a.P;
    for (int item = wid; item < TP; item += nw) {
        const int t = item / a.P, p = item - t * a.P;
        const int v0 = __ldg(a.pindex + p);
        const int n = __ldg(a.pindex + p + 1) - v0;
        const int2* pv = a.wv + (size_t)t * a.V + v0;
        int xmin = INT_MAX, xmax = INT_MIN, ymin = INT_MAX, ymax = INT_MIN;
        for (int k = lane; k < n; k += 32) {
            int2 q = pv[k];
            xmin = min(xmin, q.x); xmax = max(xmax, q.x);
            ymin = min(ymin, q.y); ymax = max(ymax, q.y);
        }
        xmin = warp_min(xmin); xmax = warp_max(xmax);
        ymin = warp_min(ymin); ymax = warp_max(ymax);
        if (lane != 0) continue;
        int nbands = 0;
        int4 ia = make_int4(0, -1, 0, -1);
        int2 ib = make_int2(0, -1);
        if (n >= 2) {
            // rows whose centre can be crossed: ymin < Cy <= ymax
            int j_lo = (int)floordiv64((int64_t)ymin - kSub / 2, kSub) + 1;
            int j_hi = (int)floordiv64((int64_t)ymax - kSub / 2, kSub);
            // pixels that can be inside: ceil((xmin-128)/256) .. ceil((xmax-128)/256)-1
            int i_lo = (int)floordiv64((int64_t)xmin - kSub / 2 + kSub - 1, kSub);
            int i_hi = (int)floordiv64((int64_t)xmax - kSub / 2 + kSub - 1, kSub) - 1;
            int r_lo = j_lo, r_hi = j_hi;
            const bool outline = MODE == MODE_BOUNDS || (MODE == MODE_TIER_CLASSIFY && a.outline_rows);
            if (outline) {
                // rows whose pixel rectangle an edge may touch
                r_lo = min(r_lo, (int)floordiv64((int64_t)ymin, kSub) - 1);
                r_hi = max(r_hi, (int)floordiv64((int64_t)ymax, kSub) + 1);
            }
            r_lo = max(r_lo, 0);
            r_hi = min(r_hi, a.resy - 1);
            if (MODE >= MODE_TIER_CLASSIFY) r_lo &= ~15;   // bands on block rows
            i_lo = max(i_lo, 0);
            i_hi = min(i_hi, a.resx - 1);
            if (r_lo <= r_hi && (outline || i_lo <= i_hi)) {
                nbands = (r_hi - r_lo + kBand) / kBand;
                ia = make_int4(i_lo, i_hi, r_lo, r_hi);
                ib = make_int2(j_lo, j_hi);
            }
        }
        a.info_a[item] = ia;
        a.info_b[item] = ib;
        a.nbands[item] = nbands;
    }
}

// One warp per (tile, polygon, band of kBand rows): the band's edges are
// staged in shared memory, each row's centre-line crossings are computed
// exactly, and every pixel of the row is inside iff an odd number of
// crossings lies to its right.
template <int MODE>
__global__ void __launch_bounds__(kPolyWarps * 32)
k_poly_pass(PolyPassArgs a) {
    extern __shared__ int4 s_poly[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int TP = a.T * a.P;
    const int total = a.band_start[TP];
    int4* my_edge = s_poly + (size_t)warp * kBandCap;
    int* my_eidx = reinterpret_cast<int*>(s_poly + (size_t)kPolyWarps * kBandCap) + (size_t)warp * kBandCap;
    int* my_cross = reinterpret_cast<int*>(s_poly + (size_t)kPolyWarps * kBandCap) + (size_t)kPolyWarps * kBandCap +
                    (size_t)warp * kCrossCap;

    for (;;) {
        int item = 0;
        if (lane == 0) item = (int)atomicAdd(a.work_ctr, 1u);
        item = __shfl_sync(FULL, item, 0);
        if (item >= total) break;
        const int tp = warp_find_owner(a.band_start, TP, item, lane);
        const int t = tp / a.P, p = tp - t * a.P;
        const int band = item - a.band_start[tp];
        const int4 ia = a.info_a[tp];
        const int2 ib = a.info_b[tp];
        const int i_lo = ia.x, i_hi = ia.y, j_lo = ib.x, j_hi = ib.y;
        const int jb = ia.z + band * kBand;
        const int je = min(jb + kBand - 1, ia.w);
        const int v0 = __ldg(a.pindex + p);
        const int n = __ldg(a.pindex + p + 1) - v0;
        const int2* pv = a.wv + (size_t)t * a.V + v0;
        const float2* pf = a.wf ? a.wf + (size_t)t * a.V + v0 : nullptr;
        const size_t tile_off = (size_t)t * a.resx * a.resy;

        unsigned long long acc_c = 0;
        long long acc_s = 0;
        long long b_fn = 0, b_fp = 0, b_fn1 = 0, b_fp1 = 0;

        // fixed-point y window of the band (one pixel of margin each side)
        const int64_t band_lo = (int64_t)jb * kSub - kSub;
        const int64_t band_hi = (int64_t)(je + 1) * kSub + kSub;
        int nb = 0;
        for (int k0 = 0; k0 < n; k0 += 32) {
            int k = k0 + lane;
            bool take = false;
            int4 e = make_int4(0, 0, 0, 0);
            if (k < n) {
                int2 A = pv[k];
                int2 B = pv[(k + 1 == n) ? 0 : k + 1];
                int lo = min(A.y, B.y), hi = max(A.y, B.y);
                take = (hi >= band_lo) && (lo <= band_hi);
                e = make_int4(A.x, A.y, B.x, B.y);
            }
            unsigned m = __ballot_sync(FULL, take);
            int pos = nb + __popc(m & ((1u << lane) - 1u));
            if (take && pos < kBandCap) { my_edge[pos] = e; my_eidx[pos] = k; }
            nb += __popc(m);
        }
        const bool overflow = nb > kBandCap;
        __syncwarp();

        for (int j = jb; j <= je; ++j) {
            const int32_t cy = j * kSub + kSub / 2;
            // crossings of this row's centre line: from the staged edges, or
            // from all edges of the polygon when the band held too many
            int m = 0;
            const int ne = overflow ? n : nb;
            for (int e0 = 0; e0 < ne; e0 += 32) {
                const int e = e0 + lane;
                bool c = false;
                int L = 0;
                if (e < ne) {
                    int4 q;
                    if (!overflow) {
                        q = my_edge[e];
                    } else {
                        const int2 A = pv[e];
                        const int2 B = pv[(e + 1 == n) ? 0 : e + 1];
                        q = make_int4(A.x, A.y, B.x, B.y);
                    }
                    if (cross_row(q.y, q.w, cy)) { c = true; L = cross_L(q.x, q.y, q.z, q.w, cy); }
                }
                const unsigned bm = __ballot_sync(FULL, c);
                const int pos = m + __popc(bm & ((1u << lane) - 1u));
                if (c && pos < kCrossCap) my_cross[pos] = L;
                m += __popc(bm);
            }
            const bool cover_slow = m > kCrossCap;
            __syncwarp();
            const bool centre_row = (j >= j_lo && j <= j_hi);
            if (centre_row && m > 0) {
                // pixel i is covered when an odd number of crossings lie at or
                // left of it: with the crossings sorted, [c0, c1), [c2, c3), ...
                auto visit = [&](int i) {
                    if (MODE == MODE_BOUNDS && a.tier_code) return;   // counts: the tier reduction
                    const size_t pix = tile_off + (size_t)j * a.resx + i;
                    if (a.border) {
                        uint32_t w = __ldg(a.border + ((size_t)j * a.border_words + (i >> 5)));
                        if ((w >> (i & 31)) & 1u) return;
                    }
                    if (MODE == MODE_LABEL) {
                        a.label[pix] = (uint16_t)p;   // overlaps detected by counting, see k_label_finish
                        ++acc_c;
                    } else {
                        acc_c += __ldg(a.canvas_c + pix);
                        if (a.canvas_s) acc_s += __ldg(a.canvas_s + pix);
                    }
                };
                if (!cover_slow) {
                    warp_sort_ints(my_cross, m, lane);   // the outline's inside test searches them too
                    if (!(MODE == MODE_BOUNDS && a.tier_code))
                    for (int s2 = 0; s2 + 1 < m; s2 += 2) {
                        const int L = max(my_cross[s2], i_lo), R = min(my_cross[s2 + 1], i_hi + 1);
                        for (int i = L + lane; i < R; i += 32) visit(i);
                    }
                } else {
                    for (int i = i_lo + lane; i <= i_hi; i += 32) {
                        bool inside = false;
                        for (int k = 0; k < n; ++k) {
                            int2 A = pv[k];
                            int2 B = pv[(k + 1 == n) ? 0 : k + 1];
                            if (cross_row(A.y, B.y, cy)) inside ^= (i < cross_L(A.x, A.y, B.x, B.y, cy));
                        }
                        if (inside) visit(i);
                    }
                }
            }
            if (MODE == MODE_BOUNDS) {
                // Outline pass: every edge of the polygon touching this pixel
                // row, every pixel of the row the edge clips.  The (edge,
                // pixel) pairs of 32 edges at a time are spread over the
                // lanes, so a long edge does not leave the others idle.
                const float ylo = (float)j, yhi = (float)(j + 1);
                for (int e0 = 0; e0 < ne; e0 += 32) {
                    const int e = e0 + lane;
                    int k = 0, ia0 = 0, cnt = 0;
                    if (e < ne) {
                        k = overflow ? e : my_eidx[e];
                        const float2 P0 = pf[k];
                        const float2 P1 = pf[(k + 1 == n) ? 0 : k + 1];
                        const float eylo = fminf(P0.y, P1.y), eyhi = fmaxf(P0.y, P1.y);
                        if (!(eyhi < ylo - 0.01f || eylo > yhi + 0.01f)) {
                            // x range of the edge inside the slab (conservative, +-1 px)
                            float xa, xb;
                            if (P0.y == P1.y) {
                                xa = fminf(P0.x, P1.x); xb = fmaxf(P0.x, P1.x);
                            } else {
                                float ta = (ylo - P0.y) / (P1.y - P0.y);
                                float tb = (yhi - P0.y) / (P1.y - P0.y);
                                ta = fminf(fmaxf(ta, 0.0f), 1.0f);
                                tb = fminf(fmaxf(tb, 0.0f), 1.0f);
                                float x_a = P0.x + (P1.x - P0.x) * ta;
                                float x_b = P0.x + (P1.x - P0.x) * tb;
                                xa = fminf(x_a, x_b); xb = fmaxf(x_a, x_b);
                            }
                            ia0 = max((int)floorf(xa) - 1, 0);
                            const int ib0 = min((int)floorf(xb) + 1, a.resx - 1);
                            cnt = max(ib0 - ia0 + 1, 0);
                        }
                    }
                    int incl = cnt;
                    #pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int v = __shfl_up_sync(FULL, incl, o);
                        if (lane >= o) incl += v;
                    }
                    const int npairs = __shfl_sync(FULL, incl, 31);
                    for (int base = 0; base < npairs; base += 32) {
                        const int idx = base + lane;
                        int lo = 0, hi = 31;   // the lane whose edge holds pair idx
                        #pragma unroll
                        for (int st = 0; st < 5; ++st) {
                            const int mid = (lo + hi) >> 1;
                            if (__shfl_sync(FULL, incl, mid) > idx) hi = mid; else lo = mid + 1;
                        }
                        const int ke = __shfl_sync(FULL, k, lo);
                        const int i = __shfl_sync(FULL, ia0, lo) + idx -
                                      (__shfl_sync(FULL, incl, lo) - __shfl_sync(FULL, cnt, lo));
                        if (idx >= npairs) continue;
                        const float2 P0 = pf[ke];
                        const float2 P1 = pf[(ke + 1 == n) ? 0 : ke + 1];
                        uint32_t val;
                        if (a.tier_code) {
                            // the pixel's count in its mixed block's slot
                            const size_t b = (size_t)t * a.tier_bw * a.tier_bh + (size_t)(j >> 4) * a.tier_bw + (i >> 4);
                            const uint32_t code = __ldg(a.tier_code + b);
                            if (!(code & kTierMixed) || code >= kTierMulti) {
                                atomicOr(a.err, 4);   // never: such blocks are made mixed
                                continue;
                            }
                            val = __ldg(a.tier_pcnt + (size_t)(code & ~kTierMixed) * 256 + (size_t)(j & 15) * 16 + (i & 15));
                        } else {
                            val = __ldg(a.canvas_c + tile_off + (size_t)j * a.resx + i);
                        }
                        if (val == 0) continue;
                        if (a.line_filter) {
                            // varying interpolation along the line (projection of
                            // the pixel centre), kept within 0.5 px: line-bound.frag:221
                            float cxp = (float)i + 0.5f, cyp = (float)j + 0.5f;
                            float dx = __fsub_rn(P1.x, P0.x), dy = __fsub_rn(P1.y, P0.y);
                            float l2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
                            if (!(l2 > 0.0f)) continue;
                            float tt = __fdiv_rn(__fadd_rn(__fmul_rn(__fsub_rn(cxp, P0.x), dx),
                                                          __fmul_rn(__fsub_rn(cyp, P0.y), dy)), l2);
                            float qx = __fadd_rn(P0.x, __fmul_rn(tt, dx));
                            float qy = __fadd_rn(P0.y, __fmul_rn(tt, dy));
                            if (fabsf(__fsub_rn(qx, cxp)) >= 0.5f || fabsf(__fsub_rn(qy, cyp)) >= 0.5f) continue;
                        }
                        float frac;
                        if (!compute_fraction(P0.x, P0.y, P1.x, P1.y, (float)i, ylo, (float)(i + 1), yhi, frac)) continue;
                        // inside test of the pixel centre: the same coverage rule
                        // (an odd number of the row's crossings right of i; the
                        // crossings are sorted, so a binary search counts them)
                        bool inside = false;
                        if (!cover_slow && centre_row) {
                            int clo = 0, chi = m;   // first crossing right of i
                            while (clo < chi) {
                                const int mid = (clo + chi) >> 1;
                                if (my_cross[mid] <= i) clo = mid + 1; else chi = mid;
                            }
                            inside = ((m - clo) & 1) != 0;
                        } else if (centre_row) {
                            for (int kk = 0; kk < n; ++kk) {
                                int2 A = pv[kk];
                                int2 B = pv[(kk + 1 == n) ? 0 : kk + 1];
                                if (cross_row(A.y, B.y, cy)) inside ^= (i < cross_L(A.x, A.y, B.x, B.y, cy));
                            }
                        }
                        if (frac > 0.5f) frac = __fsub_rn(1.0f, frac);
                        int toAdd = (int)ceilf(__fmul_rn(frac, (float)val));
                        if (inside) { b_fp += toAdd; b_fp1 += val; }
                        else        { b_fn += toAdd; b_fn1 += val; }
                    }
                }
            }
            __syncwarp();
        }
        if (MODE == MODE_LABEL) {
            acc_c = warp_sum_u64(acc_c);
            if (lane == 0 && acc_c) atomicAdd(a.covered, acc_c);
        } else {
            acc_c = warp_sum_u64(acc_c);
            if (a.canvas_s) acc_s = (long long)warp_sum_u64((unsigned long long)acc_s);
            if (lane == 0 && acc_c) atomicAdd(a.out_count + p, acc_c);
            if (lane == 0 && a.canvas_s && acc_s != 0) atomicAdd(a.out_sum + p, (unsigned long long)acc_s);
        }
        if (MODE == MODE_BOUNDS) {
            b_fn = (long long)warp_sum_u64((unsigned long long)b_fn);
            b_fp = (long long)warp_sum_u64((unsigned long long)b_fp);
            b_fn1 = (long long)warp_sum_u64((unsigned long long)b_fn1);
            b_fp1 = (long long)warp_sum_u64((unsigned long long)b_fp1);
            if (lane == 0) {
                if (b_fn) atomicAdd((unsigned long long*)(a.out_bounds + p), (unsigned long long)b_fn);
                if (b_fp) atomicAdd((unsigned long long*)(a.out_bounds + a.P + p), (unsigned long long)b_fp);
                if (b_fn1) atomicAdd((unsigned long long*)(a.out_bounds + 2 * a.P + p), (unsigned long long)b_fn1);
                if (b_fp1) atomicAdd((unsigned long long*)(a.out_bounds + 3 * a.P + p), (unsigned long long)b_fp1);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Grid index (GLFunction::createPolyIndex GLFunction.cpp:65-156).  One warp
// per polygon: MBR in fp32, cell range as index-size.glsl:50-68 with the
// upper bound clamped to res (default) or res-1 (compat, create-index.glsl:56-61).
__device__ __forceinline__ void poly_cells(const float2* __restrict__ verts, const int* __restrict__ pindex,
                                           const GridArgs& g, int p, int lane,
                                           int& stx, int& sty, int& enx, int& eny) {
    const int v0 = __ldg(pindex + p), n = __ldg(pindex + p + 1) - v0;
    float lbx = INFINITY, lby = INFINITY, rtx = -INFINITY, rty = -INFINITY;
    for (int k = lane; k < n; k += 32) {
        float2 q = __ldg(verts + v0 + k);
        lbx = fminf(lbx, q.x); rtx = fmaxf(rtx, q.x);
        lby = fminf(lby, q.y); rty = fmaxf(rty, q.y);
    }
    lbx = warp_minf(lbx); rtx = warp_maxf(rtx);
    lby = warp_minf(lby); rty = warp_maxf(rty);
    stx = __float2int_rz(__fdiv_rn(__fsub_rn(lbx, g.lbx), g.csx));
    sty = __float2int_rz(__fdiv_rn(__fsub_rn(lby, g.lby), g.csy));
    enx = __float2int_rz(__fdiv_rn(__fsub_rn(rtx, g.lbx), g.csx)) + 1;
    eny = __float2int_rz(__fdiv_rn(__fsub_rn(rty, g.lby), g.csy)) + 1;
    const int cap = g.compat_clamp ? g.res - 1 : g.res;
    if (enx >= cap) enx = cap;
    if (eny >= cap) eny = cap;
    if (stx < 0) stx = 0;
    if (sty < 0) sty = 0;
    if (n == 0) { enx = stx; eny = sty; }
}

__global__ void k_grid_count(GridArgs g) {
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int p = wid; p < g.P; p += nw) {
        int stx, sty, enx, eny;
        poly_cells(g.verts, g.pindex, g, p, lane, stx, sty, enx, eny);
        const int w = enx - stx, h = eny - sty;
        if (w <= 0 || h <= 0) continue;
        for (int c = lane; c < w * h; c += 32) {
            int x = stx + c % w, y = sty + c / w;
            atomicAdd(g.cell_count + (size_t)y * g.res + x, 1);
        }
    }
}

__global__ void k_grid_fill(GridArgs g) {
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int p = wid; p < g.P; p += nw) {
        int stx, sty, enx, eny;
        poly_cells(g.verts, g.pindex, g, p, lane, stx, sty, enx, eny);
        const int w = enx - stx, h = eny - sty;
        if (w <= 0 || h <= 0) continue;
        for (int c = lane; c < w * h; c += 32) {
            int x = stx + c % w, y = sty + c / w;
            size_t cell = (size_t)y * g.res + x;
            int pos = g.cell_start[cell] + atomicAdd(g.cursor + cell, 1);
            g.entries[pos] = p;
            if (g.pair_cell) g.pair_cell[pos] = (int)cell;
        }
    }
}

// Deterministic order inside each cell: ascending polygon id.
__global__ void k_grid_sort(const int* __restrict__ cell_start, int* __restrict__ entries, int ncells) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
        int s = cell_start[c], e = cell_start[c + 1];
        for (int i = s + 1; i < e; ++i) {
            int v = entries[i], j = i - 1;
            while (j >= s && entries[j] > v) { entries[j + 1] = entries[j]; --j; }
            entries[j + 1] = v;
        }
    }
}

// ---------------------------------------------------------------------------
// Classified grid.  For the pair (cell c, polygon p) let R be the cell grown
// by `margin` (>= the fp32 error of the crossing test, of the point-to-cell
// assignment and of the relative coordinates used here).  If no edge of p
// meets R, every point assigned to c has the same crossing-number result as
// the cell centre: the pair is FULL or OUT.  Otherwise only edges whose
// y-extent meets R's rows can toggle a point of c; of those, edges entirely
// left of R never toggle and edges entirely right of R toggle exactly when
// they straddle the point's y.
// Level 1 classifies the candidate pairs on the coarse (query) grid; FULL and
// OUT results hold for every fine cell inside, EDGE pairs are refined into
// their scale x scale fine cells and classified again (level 2), keeping the
// edge lists of the fine EDGE pairs.
struct CellRect {
    float cx, cy;      // centre
    float hw, hh;      // half extents grown by the margin
};

__device__ __forceinline__ int pair_poly(const ClsArgs& a, int k) {
    int lo = 0, hi = a.P - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(a.pair_off + mid) <= k) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// rectangle of fine cells [gx, gx+n) x [gy, gy+n) of the fine grid
__device__ __forceinline__ CellRect cells_rect(const ClsArgs& a, int gx, int gy, int n) {
    float x0 = a.lbx + (float)gx * a.csx, x1 = a.lbx + (float)(gx + n) * a.csx;
    float y0 = a.lby + (float)gy * a.csy, y1 = a.lby + (float)(gy + n) * a.csy;
    // cell 0 also receives points with (p - lb)/cs in (-1, 0): int() truncates
    if (gx == 0) x0 = a.lbx - a.csx;
    if (gy == 0) y0 = a.lby - a.csy;
    CellRect r;
    r.cx = 0.5f * (x0 + x1);
    r.cy = 0.5f * (y0 + y1);
    r.hw = 0.5f * (x1 - x0) + a.margin;
    r.hh = 0.5f * (y1 - y0) + a.margin;
    return r;
}

// Does the segment a-b meet the box [-hw,hw] x [-hh,hh]?  (Liang-Barsky)
__device__ __forceinline__ bool seg_meets_box(float ax, float ay, float bx, float by, float hw, float hh) {
    if (fmaxf(ax, bx) < -hw || fminf(ax, bx) > hw || fmaxf(ay, by) < -hh || fminf(ay, by) > hh) return false;
    float t0 = 0.0f, t1 = 1.0f;
    const float dx = bx - ax, dy = by - ay;
    const float p[4] = {-dx, dx, -dy, dy};
    const float q[4] = {ax + hw, hw - ax, ay + hh, hh - ay};
    #pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (p[i] == 0.0f) {
            if (q[i] < 0.0f) return false;
        } else {
            float r = q[i] / p[i];
            if (p[i] < 0.0f) t0 = fmaxf(t0, r);
            else t1 = fminf(t1, r);
            if (t0 > t1) return false;
        }
    }
    return true;
}

// per edge of the pair: bit0 meets R, bit1 kept (may toggle), bit2 straddle-only
__device__ __forceinline__ int edge_class(const CellRect& r, float2 vi, float2 vj) {
    const float ax = vi.x - r.cx, ay = vi.y - r.cy;
    const float bx = vj.x - r.cx, by = vj.y - r.cy;
    int c = seg_meets_box(ax, ay, bx, by, r.hw, r.hh) ? 1 : 0;
    const bool band = !(fmaxf(ay, by) < -r.hh || fminf(ay, by) > r.hh) && !(fmaxf(ax, bx) < -r.hw);
    if (band) {
        c |= 2;
        if (fminf(ax, bx) > r.hw) c |= 4;
    }
    return c;
}

__global__ void k_cls_classify(ClsArgs a) {
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const unsigned FULL = 0xffffffffu;
    const int npairs = a.level == 1 ? a.npairs : *a.plist_n;
    for (int k = wid; k < npairs; k += nw) {
        int p, gx, gy, n;
        if (a.level == 1) {
            p = pair_poly(a, k);
            const int4 r = __ldg(a.prange + p);
            const int w = r.y - r.x, l = k - __ldg(a.pair_off + p);
            gx = (r.x + l % w) * a.scale;
            gy = (r.z + l / w) * a.scale;
            n = a.scale;
        } else {
            const int2 q = a.plist[k];
            p = q.x;
            gx = q.y % a.res;
            gy = q.y / a.res;
            n = 1;
        }
        const int v0 = __ldg(a.pindex + p), nv = __ldg(a.pindex + p + 1) - v0;
        const CellRect r = cells_rect(a, gx, gy, n);
        int meets = 0, nr = 0, nf = 0;
        bool inside = false;
        for (int e0 = 0; e0 < nv; e0 += 32) {
            int e = e0 + lane;
            int c = 0;
            bool tog = false;
            if (e < nv) {
                float2 vi = __ldg(a.verts + v0 + e);
                float2 vj = __ldg(a.verts + v0 + (e == 0 ? nv - 1 : e - 1));
                c = edge_class(r, vi, vj);
                tog = edge_toggles(vi.x, vi.y, vj.x, vj.y, r.cx, r.cy);
            }
            meets += __popc(__ballot_sync(FULL, c & 1));
            nr += __popc(__ballot_sync(FULL, (c & 6) == 6));
            nf += __popc(__ballot_sync(FULL, (c & 6) == 2));
            inside ^= (__popc(__ballot_sync(FULL, tog)) & 1) != 0;
        }
        const int kind = meets ? 0 : (inside ? -1 : -2);
        if (a.level == 1) {
            if (lane == 0) a.info[k] = make_int4(p, kind, 0, gy * a.res + gx);
            if (kind == -1) {
                for (int s = lane; s < n * n; s += 32)
                    atomicAdd(a.cell_kept + (gy + s / n) * a.res + gx + s % n, 1);
            } else if (kind == 0) {
                int base = 0;
                if (lane == 0) base = atomicAdd(a.plist_n, n * n);
                base = __shfl_sync(FULL, base, 0);
                for (int s = lane; s < n * n; s += 32)
                    a.plist[base + s] = make_int2(p, (gy + s / n) * a.res + gx + s % n);
            }
        } else if (lane == 0) {
            const int cell = gy * a.res + gx;
            a.info[k] = (kind == 0) ? make_int4(p, nr, nf, cell) : make_int4(p, kind, 0, cell);
            a.ecount[k] = (kind == 0) ? nr + nf : 0;
            if (kind != -2) atomicAdd(a.cell_kept + cell, 1);
        }
    }
}

// Kept pairs into the cell-major list (order inside a cell is immaterial).
// Level 1: FULL coarse pairs expand to their fine cells.  Level 2: kept pairs.
__global__ void k_cls_emit(ClsArgs a) {
    const int npairs = a.level == 1 ? a.npairs : *a.plist_n;
    const int nn = a.scale * a.scale;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < npairs; k += gridDim.x * blockDim.x) {
        int4 in = a.info[k];
        if (a.level == 1) {
            if (in.y != -1) continue;
            const int gx = in.w % a.res, gy = in.w / a.res;
            for (int s = 0; s < nn; ++s) {
                const int cell = (gy + s / a.scale) * a.res + gx + s % a.scale;
                const int pos = a.cell_start[cell] + atomicAdd(a.cursor + cell, 1);
                a.entries[pos] = make_int4(in.x, -1, 0, 0);
            }
        } else {
            if (in.y == -2) continue;
            const int cell = in.w;
            const int pos = a.cell_start[cell] + atomicAdd(a.cursor + cell, 1);
            in.w = (in.y >= 0) ? a.eoff[k] : 0;
            if (in.y < 0) in.z = 0;
            a.entries[pos] = in;
        }
    }
}

// Level 2: edge lists of fine EDGE pairs (straddle-only edges first).
__global__ void k_cls_fill_edges(ClsArgs a) {
    const int lane = threadIdx.x & 31;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const unsigned FULL = 0xffffffffu;
    const int npairs = *a.plist_n;
    for (int k = wid; k < npairs; k += nw) {
        if (a.ecount[k] == 0) continue;
        const int4 in = a.info[k];
        const int p = in.x, cell = in.w, nr = in.y;
        const int v0 = __ldg(a.pindex + p), nv = __ldg(a.pindex + p + 1) - v0;
        const CellRect r = cells_rect(a, cell % a.res, cell / a.res, 1);
        float4* out = a.edges + a.eoff[k];
        int wr = 0, wf = nr;
        for (int e0 = 0; e0 < nv; e0 += 32) {
            int e = e0 + lane;
            int c = 0;
            float2 vi = make_float2(0.f, 0.f), vj = vi;
            if (e < nv) {
                vi = __ldg(a.verts + v0 + e);
                vj = __ldg(a.verts + v0 + (e == 0 ? nv - 1 : e - 1));
                c = edge_class(r, vi, vj);
            }
            const bool is_r = (c & 6) == 6, is_f = (c & 6) == 2;
            const unsigned mr = __ballot_sync(FULL, is_r), mf = __ballot_sync(FULL, is_f);
            const unsigned below = (1u << lane) - 1u;
            if (is_r) out[wr + __popc(mr & below)] = make_float4(vi.x, vi.y, vj.x, vj.y);
            if (is_f) out[wf + __popc(mf & below)] = make_float4(vi.x, vi.y, vj.x, vj.y);
            wr += __popc(mr);
            wf += __popc(mf);
        }
    }
}

// Count labelled pixels (a polygon set overlaps iff fewer pixels carry a
// label than polygon coverages were written) and fuse the dilated border mask
// of the hybrid canvas into the label map.
__global__ void k_label_finish(uint16_t* __restrict__ label, const uint32_t* __restrict__ mask, int resx, int resy,
                               int ntiles, int words, unsigned long long* __restrict__ nonempty) {
    // one thread per 32-pixel run of a row (the width of one mask word)
    const int runs = (resx + 31) / 32;
    const size_t total = (size_t)runs * resy * ntiles;
    unsigned long long cnt = 0;
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
        const int w = (int)(g % runs);
        const size_t row = g / runs;                  // tile * resy + j
        const int j = (int)(row % resy);
        uint16_t* l = label + row * resx + (size_t)w * 32;
        const int n = min(32, resx - w * 32);
        const uint32_t m = mask ? __ldg(mask + (size_t)j * words + w) : 0u;
        for (int i = 0; i < n; ++i) {
            const uint16_t v = l[i];
            cnt += (v != kEmptyLabel);
            if ((m >> i) & 1u) l[i] = kBorderLabel;
        }
    }
    cnt = warp_sum_u64(cnt);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(nonempty, cnt);
}

// Per classified cell: the polygon id when the cell lies inside exactly one
// polygon and needs no test, else kCodeEmpty / kCodeList.
__global__ void k_cls_codes(const int* __restrict__ cell_start, const int4* __restrict__ entries,
                            uint32_t* __restrict__ code, int ncells) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
        const int s = cell_start[c], e = cell_start[c + 1];
        uint32_t v;
        if (e == s) v = kCodeEmpty;
        else if (e == s + 1 && entries[s].y == -1) v = (uint32_t)entries[s].x;
        else v = kCodeList;
        code[c] = v;
    }
}

// ---------------------------------------------------------------------------
// Exclusive scan of int counts (n <= 16M) into out[0..n]; out[n] = total.
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ int block_exclusive_scan(int v, int* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
    #pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = (lane < (blockDim.x >> 5)) ? s_warp[lane] : 0;
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    int base = warp ? s_warp[warp - 1] : 0;
    int r = base + x - v;
    __syncthreads();
    return r;
}

__global__ void k_scan_tiles(const int* in, int* out, int n, int* __restrict__ tile_sums) {
    __shared__ int s_warp[32];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
    int v[kScanItems];
    int local = 0;
    #pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        size_t i = base + k;
        v[k] = (i < (size_t)n) ? in[i] : 0;
        local += v[k];
    }
    int ex = block_exclusive_scan(local, s_warp);
    #pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        size_t i = base + k;
        if (i < (size_t)n) out[i] = ex;
        ex += v[k];
    }
    if (threadIdx.x == blockDim.x - 1) tile_sums[blockIdx.x] = ex;
}

__global__ void k_scan_sums(int* __restrict__ tile_sums, int ntiles, int* __restrict__ total_out) {
    // single block: exclusive scan of tile sums (ntiles <= 4096)
    __shared__ int s_warp[32];
    int v[kScanItems];
    int local = 0;
    #pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int i = threadIdx.x * kScanItems + k;
        v[k] = (i < ntiles) ? tile_sums[i] : 0;
        local += v[k];
    }
    int ex = block_exclusive_scan(local, s_warp);
    #pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int i = threadIdx.x * kScanItems + k;
        if (i < ntiles) tile_sums[i] = ex;
        ex += v[k];
    }
    if (threadIdx.x == blockDim.x - 1) *total_out = ex;
}

__global__ void k_scan_add(int* __restrict__ out, int n, const int* __restrict__ tile_sums) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (size_t)n) out[i] += tile_sums[i / kScanTile];
}

// ---------------------------------------------------------------------------
// Hybrid border mask.  Window coordinates follow hybrid.glsl rasterize()
// without the range test; every pixel whose rectangle, grown by `margin`
// pixels, meets an edge is marked (a conservative superset of the outline
// fragments of line-simple.frag).
__device__ __forceinline__ void hyb_win(const HybXf& h, float x, float y, float& u, float& v) {
    u = __fmul_rn(__fmul_rn(__fadd_rn(__fdiv_rn(__fsub_rn(x, h.ox), h.dx), 1.0f), 0.5f), (float)h.resx);
    v = __fmul_rn(__fmul_rn(__fadd_rn(__fdiv_rn(__fsub_rn(y, h.oy), h.dy), 1.0f), 0.5f), (float)h.resy);
}

__global__ void k_outline_mask(const float2* __restrict__ verts, const int* __restrict__ pindex, int P,
                               const int* __restrict__ edge_poly, int V, HybXf h, float margin,
                               uint32_t* __restrict__ mask, int words) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < V; k += gridDim.x * blockDim.x) {
        const int p = edge_poly[k];
        const int v0 = pindex[p], n = pindex[p + 1] - v0;
        const int kn = (k + 1 == v0 + n) ? v0 : k + 1;
        float2 A = verts[k], B = verts[kn];
        float ax, ay, bx, by;
        hyb_win(h, A.x, A.y, ax, ay);
        hyb_win(h, B.x, B.y, bx, by);
        float ylo = fminf(ay, by) - margin, yhi = fmaxf(ay, by) + margin;
        int jlo = max((int)floorf(ylo), 0), jhi = min((int)floorf(yhi), h.resy - 1);
        for (int j = jlo; j <= jhi; ++j) {
            // x extent of the segment within the slab [j - margin, j + 1 + margin]
            float sy0 = (float)j - margin, sy1 = (float)(j + 1) + margin;
            float xa, xb;
            if (ay == by) { xa = fminf(ax, bx); xb = fmaxf(ax, bx); }
            else {
                float ta = (sy0 - ay) / (by - ay), tb = (sy1 - ay) / (by - ay);
                ta = fminf(fmaxf(ta, 0.0f), 1.0f); tb = fminf(fmaxf(tb, 0.0f), 1.0f);
                float x0 = ax + (bx - ax) * ta, x1 = ax + (bx - ax) * tb;
                xa = fminf(x0, x1); xb = fmaxf(x0, x1);
            }
            int ilo = max((int)floorf(xa - margin), 0), ihi = min((int)floorf(xb + margin), h.resx - 1);
            for (int i = ilo; i <= ihi; ++i)
                atomicOr(mask + (size_t)j * words + (i >> 5), 1u << (i & 31));
        }
    }
}

// Dilation by `radius` pixels (isBorder's 3x3 neighbourhood for radius 1,
// hybrid.glsl:174-185).
__global__ void k_dilate_mask(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                              int resx, int resy, int words, int radius) {
    size_t total = (size_t)resy * words;
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
        int j = (int)(g / words), w = (int)(g % words);
        uint32_t acc = 0;
        for (int dj = -radius; dj <= radius; ++dj) {
            int jj = j + dj;
            if (jj < 0 || jj >= resy) continue;
            const uint32_t* row = in + (size_t)jj * words;
            uint32_t c = row[w];
            uint32_t l = (w > 0) ? row[w - 1] : 0u;
            uint32_t r = (w + 1 < words) ? row[w + 1] : 0u;
            uint32_t hacc = c;
            for (int s = 1; s <= radius; ++s) {
                // bit i of out gets bits i-s and i+s of the input row
                hacc |= (c << s) | (l >> (32 - s));
                hacc |= (c >> s) | (r << (32 - s));
            }
            acc |= hacc;
        }
        out[g] = acc;
    }
}

// ---------------------------------------------------------------------------
// launchers
void launch_transform_vertices(const float2* verts, int V, const float4* colxf, const float4* rowxf,
                               int splitx, int T, int2* wv, float2* wf, int sms, cudaStream_t st) {
    size_t total = (size_t)T * V;
    int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)sms * 8);
    if (blocks < 1) blocks = 1;
    k_transform_vertices<<<blocks, 256, 0, st>>>(verts, V, colxf, rowxf, splitx, T, wv, wf);
    ++g_kernel_launches;
}

void launch_poly_info(int mode, const PolyPassArgs& a, int sms, cudaStream_t st) {
    int items = a.T * a.P;
    int blocks = std::min((items * 32 + 255) / 256, sms * 8);
    if (blocks < 1) blocks = 1;
    ++g_kernel_launches;
    if (mode == MODE_BOUNDS) k_poly_info<MODE_BOUNDS><<<blocks, 256, 0, st>>>(a);
    else if (mode >= MODE_TIER_CLASSIFY) k_poly_info<MODE_TIER_CLASSIFY><<<blocks, 256, 0, st>>>(a);
    else k_poly_info<MODE_REDUCE><<<blocks, 256, 0, st>>>(a);
}

template <int MODE>
static void launch_poly_pass_t(const PolyPassArgs& a, int sms, cudaStream_t st) {
    static bool attr_set = false;   // per template instance
    if (!attr_set) {
        cudaFuncSetAttribute(k_poly_pass<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPolySmem);
        attr_set = true;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_poly_pass<MODE>, kPolyWarps * 32, kPolySmem);
    const int blocks = sms * std::max(per_sm, 1);
    k_poly_pass<MODE><<<blocks, kPolyWarps * 32, kPolySmem, st>>>(a);
}

void launch_poly_pass(int mode, const PolyPassArgs& a, int sms, cudaStream_t st) {
    ++g_kernel_launches;
    switch (mode) {
        case MODE_REDUCE: launch_poly_pass_t<MODE_REDUCE>(a, sms, st); break;
        case MODE_LABEL: launch_poly_pass_t<MODE_LABEL>(a, sms, st); break;
        default: launch_poly_pass_t<MODE_BOUNDS>(a, sms, st); break;
    }
}

void launch_grid_count(const GridArgs& g, int sms, cudaStream_t st) {
    int blocks = std::min((g.P * 32 + 255) / 256, sms * 8);
    if (blocks < 1) blocks = 1;
    k_grid_count<<<blocks, 256, 0, st>>>(g);
    ++g_kernel_launches;
}
void launch_grid_fill(const GridArgs& g, int sms, cudaStream_t st) {
    int blocks = std::min((g.P * 32 + 255) / 256, sms * 8);
    if (blocks < 1) blocks = 1;
    k_grid_fill<<<blocks, 256, 0, st>>>(g);
    ++g_kernel_launches;
}
void launch_grid_sort(const int* cell_start, int* entries, int ncells, int sms, cudaStream_t st) {
    int blocks = std::min((ncells + 255) / 256, sms * 8);
    if (blocks < 1) blocks = 1;
    k_grid_sort<<<blocks, 256, 0, st>>>(cell_start, entries, ncells);
    ++g_kernel_launches;
}

// Scratch ints for launch_exclusive_scan: one level of tile sums per 4096x.
int scan_tmp_ints(int n) {
    int total = 0;
    int m = n;
    do {
        int ntiles = (m + kScanTile - 1) / kScanTile;
        if (ntiles < 1) ntiles = 1;
        total += ntiles + 1;
        m = ntiles;
    } while (m > kScanTile);
    return total + 1;
}

bool launch_exclusive_scan(const int* in, int* out, int n, int* tmp, cudaStream_t st) {
    int ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles < 1) ntiles = 1;
    k_scan_tiles<<<ntiles, kScanThreads, 0, st>>>(in, out, n, tmp);
    if (ntiles <= kScanTile) {
        k_scan_sums<<<1, kScanThreads, 0, st>>>(tmp, ntiles, out + n);
        g_kernel_launches += 2;
    } else {
        // scan the tile sums recursively (in place through a second buffer level)
        int* sums = tmp;
        int* next = tmp + ntiles + 1;
        if (!launch_exclusive_scan(sums, sums, ntiles, next, st)) return false;
        // out[n] = total of all tiles = scanned sums[ntiles]
        cudaMemcpyAsync(out + n, sums + ntiles, sizeof(int), cudaMemcpyDeviceToDevice, st);
        g_kernel_launches += 1;
    }
    k_scan_add<<<(n + 255) / 256, 256, 0, st>>>(out, n, tmp);
    g_kernel_launches += 1;
    return true;
}

void launch_cls_classify(const ClsArgs& c, int sms, cudaStream_t st) {
    // level 2 reads its pair count on the device; c.npairs is then an upper bound
    int blocks = (int)std::min<long long>(((long long)c.npairs * 32 + 255) / 256, (long long)sms * 32);
    if (blocks < 1) blocks = 1;
    ++g_kernel_launches;
    k_cls_classify<<<blocks, 256, 0, st>>>(c);
}
void launch_cls_emit(const ClsArgs& c, int sms, cudaStream_t st) {
    int blocks = std::min((c.npairs + 255) / 256, sms * 16);
    if (blocks < 1) blocks = 1;
    ++g_kernel_launches;
    k_cls_emit<<<blocks, 256, 0, st>>>(c);
}
void launch_cls_fill_edges(const ClsArgs& c, int sms, cudaStream_t st) {
    int blocks = (int)std::min<long long>(((long long)c.npairs * 32 + 255) / 256, (long long)sms * 32);
    if (blocks < 1) blocks = 1;
    ++g_kernel_launches;
    k_cls_fill_edges<<<blocks, 256, 0, st>>>(c);
}
void launch_label_finish(uint16_t* label, const uint32_t* mask, int resx, int resy, int ntiles, int words,
                         unsigned long long* nonempty, int sms, cudaStream_t st) {
    size_t total = (size_t)((resx + 31) / 32) * resy * ntiles;
    int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)sms * 16);
    if (blocks < 1) blocks = 1;
    ++g_kernel_launches;
    k_label_finish<<<blocks, 256, 0, st>>>(label, mask, resx, resy, ntiles, words, nonempty);
}
void launch_cls_codes(const int* cell_start, const int4* entries, uint32_t* code, int ncells, int sms,
                      cudaStream_t st) {
    int blocks = std::min((ncells + 255) / 256, sms * 16);
    if (blocks < 1) blocks = 1;
    ++g_kernel_launches;
    k_cls_codes<<<blocks, 256, 0, st>>>(cell_start, entries, code, ncells);
}

void launch_outline_mask(const float2* verts, const int* pindex, int P, const int* edge_poly, int V,
                         const HybXf& h, float margin, uint32_t* mask, int words, int sms, cudaStream_t st) {
    int blocks = std::min((V + 255) / 256, sms * 8);
    if (blocks < 1) blocks = 1;
    k_outline_mask<<<blocks, 256, 0, st>>>(verts, pindex, P, edge_poly, V, h, margin, mask, words);
    ++g_kernel_launches;
}
void launch_dilate_mask(const uint32_t* in, uint32_t* out, int resx, int resy, int words, int radius,
                        int sms, cudaStream_t st) {
    size_t total = (size_t)resy * words;
    int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)sms * 16);
    if (blocks < 1) blocks = 1;
    k_dilate_mask<<<blocks, 256, 0, st>>>(in, out, resx, resy, words, radius);
    ++g_kernel_launches;
}

}  // namespace rj
