// rj_tier_lean.cu -- lean point pass of the raster join over a tiered canvas
// (16 x 16-pixel blocks: one entry per full block, per-pixel data in the
// slots of mixed blocks; rj_tier_kernels.cu), on one or several canvas tiles.
// The counterpart of the generic pass's TierLabelMapper / TierSplatMapper
// (rj_point_map.cuh) with the lean passes' structure: coalesced point-pair
// loads, interval-form filters, the exact snapped pixel (rj_lean.cuh), no
// warp grouping.
//
// Tiles: per axis the tile is guessed with one multiplication; when the
// pixel in the guessed tile lies at least one pixel inside it, no other tile's
// window can hold the point and that is the only hit.  Otherwise (within a
// pixel of a seam, or a guess off by one) the guessed tile and both
// neighbours are tried exactly, as the generic mapping does: near a seam a
// point can fall in two tiles' windows and counts in both (every tile is
// rendered with all points, RasterJoin.cpp:224-231).
//
//   LABEL: the block code (full polygon, empty, or mixed | slot) and, for a
//          mixed block, the pixel's label give the polygon; one count (and
//          the fixed-point value) into the block's shared histogram.
//   splat: one count (and sum) per point with plain global atomics: into
//          the pixel slot of a mixed block, else into the block's total (an
//          empty block keeps nothing); the polygon pass reduces them.
#include "rj_lean.cuh"

namespace rj {

namespace {

constexpr int kLeanMaxSplit = 64;   // tiles per axis held in shared memory

template <int NCOL>
__device__ __forceinline__ bool tl_pass(const LeanCols& lc, const uint32_t (&v)[NCOL > 0 ? NCOL : 1]) {
    bool ok = true;
    #pragma unroll
    for (int c = 0; c < NCOL; ++c) {
        const uint32_t key = v[c] ^ (((uint32_t)((int32_t)v[c] >> 31) & lc.fm[c]) ^ lc.xm[c]);
        ok &= (key - lc.lo[c]) <= lc.span[c];
    }
    return ok;
}

// Tiles of one axis whose window holds coordinate v, with the pixel in each
// (t[k], p[k]); returns how many (0..3).  xf[c] = (s, t, 256 h) of tile c.
__device__ __forceinline__ int tl_axis(float v, const float3* xf, int split, float lb, float inv_td, int res,
                                       int (&t)[3], int (&p)[3]) {
    if (split == 1) {
        const int q = snapped_pixel(v, xf[0].x, xf[0].y, xf[0].z);
        t[0] = 0;
        p[0] = q;
        return (unsigned)q < (unsigned)res ? 1 : 0;
    }
    const float g = (v - lb) * inv_td;
    if (!(g > -2.0f && g < (float)split + 1.0f)) return 0;   // NaN, infinities, far outside
    const int c0 = (int)floorf(g);
    if (c0 >= 0 && c0 < split) {
        const int q = snapped_pixel(v, xf[c0].x, xf[c0].y, xf[c0].z);
        if (q >= 1 && q <= res - 2) {
            t[0] = c0;
            p[0] = q;
            return 1;
        }
    }
    int n = 0;
    #pragma unroll
    for (int d = -1; d <= 1; ++d) {
        const int c = c0 + d;
        if (c < 0 || c >= split) continue;
        const int q = snapped_pixel(v, xf[c].x, xf[c].y, xf[c].z);
        if ((unsigned)q < (unsigned)res) {
            t[n] = c;
            p[n] = q;
            ++n;
        }
    }
    return n;
}

template <bool AGG>
__device__ __forceinline__ void tl_hist_add(uint32_t* h_cnt, uint32_t P, const LeanCols& lc, uint32_t l, float v) {
    atomicAdd(h_cnt + l, 1u);
    if (AGG) {
        if (isfinite(v)) {
            const unsigned long long q = (unsigned long long)fixed_value(v, lc.scale);
            const uint32_t qlo = (uint32_t)q;
            const uint32_t old = atomicAdd(h_cnt + P + l, qlo);
            atomicAdd(h_cnt + 2 * P + l, (uint32_t)(q >> 32) + ((old + qlo < old) ? 1u : 0u));
        } else {
            atomicAdd(lc.nonfinite + l, (double)v);
        }
    }
}

// One point at pixel (px, py) of tile t.
template <bool AGG, bool LABEL>
__device__ __forceinline__ void tl_visit(const TierLeanArgs& a, uint32_t* h_cnt, const LeanCols& lc, int t, int px,
                                         int py, float v) {
    const size_t b = (size_t)t * a.tr.bw * a.tr.bh + (size_t)(py >> 4) * a.tr.bw + (px >> 4);
    const uint32_t code = __ldg(a.tr.code + b);
    const size_t at = (size_t)(code & ~kTierMixed) * 256 + (size_t)(py & 15) * 16 + (px & 15);
    if (LABEL) {
        uint32_t lab;
        if (code == kTierEmpty || code == kTierMulti) lab = kEmptyLabel;   // (multi: never in label form)
        else if (code & kTierMixed) lab = __ldg(a.tr.plabel + at);
        else lab = code;
        if (lab < (uint32_t)a.P) tl_hist_add<AGG>(h_cnt, (uint32_t)a.P, lc, lab, v);
    } else {
        // the pixel slot of a mixed block, else the block total (an empty
        // block keeps nothing: no polygon reads it)
        const bool fin = AGG && isfinite(v);
        const unsigned long long q = fin ? (unsigned long long)fixed_value(v, lc.scale) : 0ull;
        if ((code & kTierMixed) && code < kTierMulti) {
            atomicAdd(a.tr.pcnt + at, 1u);
            if (fin) atomicAdd(reinterpret_cast<unsigned long long*>(a.tr.psum + at), q);
        } else if (code != kTierEmpty) {
            atomicAdd(a.tr.bcnt + b, 1u);
            if (fin) atomicAdd(reinterpret_cast<unsigned long long*>(a.tr.bsum + b), q);
        }
    }
}

template <bool AGG, bool LABEL>
__device__ __forceinline__ void tl_point(const TierLeanArgs& a, const float3* sx, const float3* sy, uint32_t* h_cnt,
                                         const LeanCols& lc, float x, float y, float v) {
    int tx[3], px[3], ty[3], py[3];
    const int nx = tl_axis(x, sx, a.splitx, a.lbx, a.inv_tdx, a.resx, tx, px);
    if (nx == 0) return;
    const int ny = tl_axis(y, sy, a.splity, a.lby, a.inv_tdy, a.resy, ty, py);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
            tl_visit<AGG, LABEL>(a, h_cnt, lc, ty[j] * a.splitx + tx[i], px[i], py[j], v);
}

template <int BLOCK, int NV, int NCOL, bool AGG, bool LABEL>
__global__ void __launch_bounds__(BLOCK) k_tier_lean(TierLeanArgs a, LeanCols lc) {
    extern __shared__ uint32_t s_words[];
    constexpr int HW = AGG ? 3 : 1;
    float3* sx = reinterpret_cast<float3*>(s_words);
    float3* sy = sx + kLeanMaxSplit;
    uint32_t* s_hist = reinterpret_cast<uint32_t*>(sy + kLeanMaxSplit);   // LABEL: HW x P
    for (int i = threadIdx.x; i < a.splitx; i += BLOCK) {
        const float4 c = __ldg(a.colxf + i);
        sx[i] = make_float3(c.x, c.y, __fmul_rn(c.z, (float)kSub));
    }
    for (int i = threadIdx.x; i < a.splity; i += BLOCK) {
        const float4 r = __ldg(a.rowxf + i);
        sy[i] = make_float3(r.x, r.y, __fmul_rn(r.z, (float)kSub));
    }
    if (LABEL)
        for (int i = threadIdx.x; i < HW * a.P; i += BLOCK) s_hist[i] = 0u;
    __syncthreads();
    const uint2* aggr2 = lc.aggr_col;

    const uint64_t npairs = a.n >> 1;
    constexpr uint64_t kPerIter = (uint64_t)BLOCK * NV;
    const uint64_t warp_ofs = (uint64_t)(threadIdx.x >> 5) * 32 * NV;
    const uint64_t lane_ofs = warp_ofs + (threadIdx.x & 31);
    for (uint64_t base = (uint64_t)blockIdx.x * kPerIter; base < npairs; base += (uint64_t)gridDim.x * kPerIter) {
        if (a.zones) {
            const uint64_t r0 = a.zrow0 + 2 * (base + warp_ofs);
            const uint64_t r1 = a.zrow0 + min(2 * (base + warp_ofs + 32 * NV), a.n) - 1;
            const int lane = threadIdx.x & 31;
            bool meets = false;
            if (r0 <= r1 && (uint64_t)lane <= (r1 >> kZoneShift) - (r0 >> kZoneShift)) {
                const float4 bb = __ldg(a.zones + (r0 >> kZoneShift) + lane);
                meets = !(bb.z < a.qbox.x || bb.x > a.qbox.z || bb.w < a.qbox.y || bb.y > a.qbox.w);
            }
            if (!__any_sync(0xffffffffu, meets)) continue;
        }
        float4 p[NV];
        uint2 cv[NCOL > 0 ? NCOL : 1][NV];
        uint2 av[NV];
        #pragma unroll
        for (int k = 0; k < NV; ++k) {
            const uint64_t i = base + lane_ofs + (uint64_t)k * 32;
            const bool live = i < npairs;
            p[k] = live ? __ldcs(a.xy + i) : make_float4(NAN, NAN, NAN, NAN);
            #pragma unroll
            for (int c = 0; c < NCOL; ++c) cv[c][k] = live ? __ldcs(lc.col[c] + i) : make_uint2(0u, 0u);
            if (AGG) av[k] = (live && lc.aggr_ci < 0) ? __ldcs(aggr2 + i) : make_uint2(0u, 0u);
        }
        #pragma unroll
        for (int j = 0; j < 2 * NV; ++j) {
            const int k = j >> 1;
            const bool hi = (j & 1) != 0;
            uint32_t v[NCOL > 0 ? NCOL : 1];
            #pragma unroll
            for (int c = 0; c < NCOL; ++c) v[c] = hi ? cv[c][k].y : cv[c][k].x;
            if (!tl_pass<NCOL>(lc, v)) continue;
            float val = 0.f;
            if (AGG) {
                uint32_t raw = hi ? av[k].y : av[k].x;
                #pragma unroll
                for (int cc = 0; cc < NCOL; ++cc)
                    if (cc == lc.aggr_ci) raw = v[cc];
                val = agg_value(lc.aggr_typ, raw);
            }
            tl_point<AGG, LABEL>(a, sx, sy, s_hist, lc, hi ? p[k].z : p[k].x, hi ? p[k].w : p[k].y, val);
        }
    }
    // the last point of an odd-sized table
    if ((a.n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const uint64_t i = a.n - 1;
        const float2 q = __ldg(reinterpret_cast<const float2*>(a.xy) + i);
        uint32_t v[NCOL > 0 ? NCOL : 1];
        #pragma unroll
        for (int c = 0; c < NCOL; ++c) v[c] = __ldg(reinterpret_cast<const uint32_t*>(lc.col[c]) + i);
        if (tl_pass<NCOL>(lc, v)) {
            float fv = 0.f;
            if (AGG) {
                uint32_t raw = lc.aggr_ci < 0 ? __ldg(reinterpret_cast<const uint32_t*>(aggr2) + i) : 0u;
                #pragma unroll
                for (int cc = 0; cc < NCOL; ++cc)
                    if (cc == lc.aggr_ci) raw = v[cc];
                fv = agg_value(lc.aggr_typ, raw);
            }
            tl_point<AGG, LABEL>(a, sx, sy, s_hist, lc, q.x, q.y, fv);
        }
    }
    if (LABEL) {
        __syncthreads();
        for (int b = threadIdx.x; b < a.P; b += BLOCK) {
            const uint32_t cnt = s_hist[b];
            if (cnt) {
                atomicAdd(a.out_count + b, (unsigned long long)cnt);
                if (AGG)
                    atomicAdd(lc.out_sum + b, ((unsigned long long)s_hist[2 * a.P + b] << 32) + s_hist[a.P + b]);
            }
        }
    }
}

using TierLeanKernel = void (*)(TierLeanArgs, LeanCols);

struct TlShape {
    int block;
    int nv;
};
constexpr TlShape kTlShapes[] = {{512, 2}, {256, 4}, {1024, 2}};
constexpr int kNumTlShapes = (int)(sizeof(kTlShapes) / sizeof(kTlShapes[0]));

template <int NCOL, bool AGG, bool LABEL>
TierLeanKernel pick_tl(int shape) {
    switch (shape) {
        case 0: return k_tier_lean<512, 2, NCOL, AGG, LABEL>;
        case 1: return k_tier_lean<256, 4, NCOL, AGG, LABEL>;
        default: return k_tier_lean<1024, 2, NCOL, AGG, LABEL>;
    }
}

template <bool AGG, bool LABEL>
TierLeanKernel pick_tl_ncol(int ncol, int shape) {
    switch (ncol) {
        case 0: return pick_tl<0, AGG, LABEL>(shape);
        case 1: return pick_tl<1, AGG, LABEL>(shape);
        case 2: return pick_tl<2, AGG, LABEL>(shape);
        case 3: return pick_tl<3, AGG, LABEL>(shape);
        case 4: return pick_tl<4, AGG, LABEL>(shape);
        default: return nullptr;
    }
}

int g_tl_optin = -1;

}  // namespace

int tier_lean_shapes() { return kNumTlShapes; }

size_t tier_lean_smem(bool label, int P, bool agg) {
    return 2 * kLeanMaxSplit * sizeof(float3) + (label ? (size_t)P * (agg ? 3 : 1) * 4 : 0);
}

bool launch_tier_lean(int shape, bool label, const TierLeanArgs& a, const LeanCols& lc, int sms, cudaStream_t st) {
    if (shape < 0 || shape >= kNumTlShapes || lc.ncol < 0 || lc.ncol > 4) return false;
    if (a.splitx < 1 || a.splity < 1 || a.splitx > kLeanMaxSplit || a.splity > kLeanMaxSplit) return false;
    const bool agg = lc.aggr != 0;
    if (!label && agg && (!a.tr.bsum || !a.tr.psum)) return false;
    TierLeanKernel k = label ? (agg ? pick_tl_ncol<true, true>(lc.ncol, shape) : pick_tl_ncol<false, true>(lc.ncol, shape))
                             : (agg ? pick_tl_ncol<true, false>(lc.ncol, shape) : pick_tl_ncol<false, false>(lc.ncol, shape));
    if (!k) return false;
    if (g_tl_optin < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_tl_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    const size_t smem = tier_lean_smem(label, a.P, agg);
    if (smem > (size_t)g_tl_optin || smem > 200 * 1024) return false;
    if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const int block = kTlShapes[shape].block;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        return false;
    }
    const uint64_t per_iter = (uint64_t)block * kTlShapes[shape].nv;
    const uint64_t need = ((a.n >> 1) + per_iter - 1) / per_iter;
    uint64_t blocks = std::min<uint64_t>((uint64_t)sms * per_sm, std::max<uint64_t>(need, 1));
    // shared counts are 32-bit: a block must see fewer than 2^31 points, twice
    // over for points on a seam (up to four hits each)
    while (blocks < (uint64_t)sms * per_sm && a.n / blocks >= (1ull << 29)) ++blocks;
    if (label && a.n / blocks >= (1ull << 29)) return false;
    k<<<(unsigned)blocks, block, smem, st>>>(a, lc);
    ++g_kernel_launches;
    return true;
}

}  // namespace rj
