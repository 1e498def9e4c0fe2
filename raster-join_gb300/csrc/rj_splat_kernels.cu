// rj_splat_kernels.cu -- lean point pass of the raster join onto a point
// canvas (points.vert:138-159 with its additive blending into the count and
// sum textures, RasterJoin.cpp:215-236), used where the label map does not
// apply: polygon sets whose coverage overlaps on the canvas, and the
// error-bounds join (whose polygon pass reads per-pixel counts).
//
// Per point: the interval-form predicates, the exact snapped pixel of the
// single canvas tile (rj_lean.cuh), then one count (and, with an aggregate,
// the int64 fixed-point value; a non-finite value adds nothing to a canvas
// sum, as in the generic splat) into the pixel:
//   * SMEM: the whole canvas held per block in shared memory (count, and the
//     sum as two 32-bit words with carry), in warp-group copies when room
//     allows, flushed once per block with one global atomic per touched
//     pixel;
//   * global: one atomic per point straight into the canvas in global memory
//     (L2 atomics; no warp grouping, whose match instructions limited the
//     generic splat).
// Loads are the lean passes' coalesced pairs (x, y as one float4, each
// 4-byte column as one uint2 per lane).
#include "rj_lean.cuh"

namespace rj {

namespace {

template <int NCOL>
__device__ __forceinline__ bool splat_pass(const LeanCols& lc, const uint32_t (&v)[NCOL > 0 ? NCOL : 1]) {
    bool ok = true;
    #pragma unroll
    for (int c = 0; c < NCOL; ++c) {
        const uint32_t key = v[c] ^ (((uint32_t)((int32_t)v[c] >> 31) & lc.fm[c]) ^ lc.xm[c]);
        ok &= (key - lc.lo[c]) <= lc.span[c];
    }
    return ok;
}

// Adds one point to pixel k of the canvas (shared copy or global canvas).
template <bool AGG, bool SMEM>
__device__ __forceinline__ void splat_add(const SplatLeanArgs& a, uint32_t* s_can, uint32_t npix, const LeanCols& lc,
                                          uint32_t k, float v) {
    if (SMEM) {
        atomicAdd(s_can + k, 1u);
        if (AGG && isfinite(v)) {
            const unsigned long long q = (unsigned long long)fixed_value(v, lc.scale);
            const uint32_t qlo = (uint32_t)q;
            const uint32_t old = atomicAdd(s_can + npix + k, qlo);
            atomicAdd(s_can + 2 * npix + k, (uint32_t)(q >> 32) + ((old + qlo < old) ? 1u : 0u));
        }
    } else {
        atomicAdd(a.canvas_c + k, 1u);
        if (AGG && isfinite(v)) atomicAdd(a.canvas_s + k, (unsigned long long)fixed_value(v, lc.scale));
    }
}

template <int BLOCK, int NV, int NCOL, bool AGG, bool SMEM>
__global__ void __launch_bounds__(BLOCK) k_splat_lean(SplatLeanArgs a, LeanCols lc) {
    extern __shared__ uint32_t s_words[];
    constexpr int HW = AGG ? 3 : 1;                   // count | sum low word | sum high word
    const uint32_t npix = (uint32_t)a.resx * (uint32_t)a.resy;
    uint32_t* s_can = s_words;
    if (SMEM) {
        for (uint32_t i = threadIdx.x; i < (uint32_t)lc.copies * HW * npix; i += BLOCK) s_words[i] = 0u;
        __syncthreads();
        s_can = s_words + ((threadIdx.x >> 5) & (lc.copies - 1)) * HW * npix;
    }
    const TileXf2 xf{a.col0.x, a.col0.y, __fmul_rn(a.col0.z, (float)kSub),
                     a.row0.x, a.row0.y, __fmul_rn(a.row0.z, (float)kSub)};
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
                const float4 b = __ldg(a.zones + (r0 >> kZoneShift) + lane);
                meets = !(b.z < a.qbox.x || b.x > a.qbox.z || b.w < a.qbox.y || b.y > a.qbox.w);
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
            const float x = hi ? p[k].z : p[k].x;
            const float y = hi ? p[k].w : p[k].y;
            const int px = snapped_pixel(x, xf.sx, xf.tx, xf.Hx);
            const int py = snapped_pixel(y, xf.sy, xf.ty, xf.Hy);
            if ((unsigned)px < (unsigned)a.resx && (unsigned)py < (unsigned)a.resy && splat_pass<NCOL>(lc, v)) {
                float val = 0.f;
                if (AGG) {
                    uint32_t raw = hi ? av[k].y : av[k].x;
                    #pragma unroll
                    for (int cc = 0; cc < NCOL; ++cc)
                        if (cc == lc.aggr_ci) raw = v[cc];
                    val = agg_value(lc.aggr_typ, raw);
                }
                splat_add<AGG, SMEM>(a, s_can, npix, lc, (uint32_t)py * (uint32_t)a.resx + (uint32_t)px, val);
            }
        }
    }
    // the last point of an odd-sized table
    if ((a.n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const uint64_t i = a.n - 1;
        const float2 q = __ldg(reinterpret_cast<const float2*>(a.xy) + i);
        uint32_t v[NCOL > 0 ? NCOL : 1];
        #pragma unroll
        for (int c = 0; c < NCOL; ++c) v[c] = __ldg(reinterpret_cast<const uint32_t*>(lc.col[c]) + i);
        const int px = snapped_pixel(q.x, xf.sx, xf.tx, xf.Hx);
        const int py = snapped_pixel(q.y, xf.sy, xf.ty, xf.Hy);
        if ((unsigned)px < (unsigned)a.resx && (unsigned)py < (unsigned)a.resy && splat_pass<NCOL>(lc, v)) {
            float fv = 0.f;
            if (AGG) {
                uint32_t raw = lc.aggr_ci < 0 ? __ldg(reinterpret_cast<const uint32_t*>(aggr2) + i) : 0u;
                #pragma unroll
                for (int cc = 0; cc < NCOL; ++cc)
                    if (cc == lc.aggr_ci) raw = v[cc];
                fv = agg_value(lc.aggr_typ, raw);
            }
            splat_add<AGG, SMEM>(a, s_can, npix, lc, (uint32_t)py * (uint32_t)a.resx + (uint32_t)px, fv);
        }
    }
    if (SMEM) {
        __syncthreads();
        for (uint32_t b = threadIdx.x; b < npix; b += BLOCK) {
            uint32_t cnt = 0;
            unsigned long long sum = 0;
            #pragma unroll 1
            for (int w = 0; w < lc.copies; ++w) {
                const uint32_t* h = s_words + (uint32_t)w * HW * npix;
                cnt += h[b];
                if (AGG) sum += ((unsigned long long)h[2 * npix + b] << 32) + h[npix + b];
            }
            if (cnt) {
                atomicAdd(a.canvas_c + b, cnt);
                if (AGG && sum) atomicAdd(a.canvas_s + b, sum);
            }
        }
    }
}

using SplatKernel = void (*)(SplatLeanArgs, LeanCols);

struct SplatShape {
    int block;
    int nv;
    bool smem;
};
constexpr SplatShape kSplatShapes[] = {{512, 2, true}, {256, 4, true}, {1024, 2, true},
                                       {512, 2, false}, {256, 4, false}, {1024, 2, false}};
constexpr int kNumSplatShapes = (int)(sizeof(kSplatShapes) / sizeof(kSplatShapes[0]));

template <int NCOL, bool AGG>
SplatKernel pick_splat(int shape) {
    switch (shape) {
        case 0: return k_splat_lean<512, 2, NCOL, AGG, true>;
        case 1: return k_splat_lean<256, 4, NCOL, AGG, true>;
        case 2: return k_splat_lean<1024, 2, NCOL, AGG, true>;
        case 3: return k_splat_lean<512, 2, NCOL, AGG, false>;
        case 4: return k_splat_lean<256, 4, NCOL, AGG, false>;
        default: return k_splat_lean<1024, 2, NCOL, AGG, false>;
    }
}

template <bool AGG>
SplatKernel pick_splat_ncol(int ncol, int shape) {
    switch (ncol) {
        case 0: return pick_splat<0, AGG>(shape);
        case 1: return pick_splat<1, AGG>(shape);
        case 2: return pick_splat<2, AGG>(shape);
        case 3: return pick_splat<3, AGG>(shape);
        case 4: return pick_splat<4, AGG>(shape);
        default: return nullptr;
    }
}

int g_splat_optin = -1;

// canvas copies in shared memory: a power of two up to the warps of the
// block, within 64 KB (a single copy may take up to 200 KB)
int splat_copies(int shape, size_t npix, bool agg) {
    const size_t per = npix * (agg ? 3 : 1) * 4;
    if (per > 200 * 1024) return 0;
    const int warps = kSplatShapes[shape].block / 32;
    int copies = 1;
    while (copies * 2 <= warps && per * copies * 2 <= 64 * 1024) copies *= 2;
    return copies;
}

}  // namespace

int splat_lean_shapes() { return kNumSplatShapes; }

size_t splat_lean_smem(int shape, size_t npix, bool agg) {
    if (shape < 0 || shape >= kNumSplatShapes) return 0;
    if (!kSplatShapes[shape].smem) return 1;   // runs with no shared memory
    const int copies = splat_copies(shape, npix, agg);
    return copies ? (size_t)copies * npix * (agg ? 3 : 1) * 4 : 0;
}

bool launch_splat_lean(int shape, const SplatLeanArgs& a, const LeanCols& lc_in, int sms, cudaStream_t st) {
    if (shape < 0 || shape >= kNumSplatShapes || lc_in.ncol < 0 || lc_in.ncol > 4) return false;
    const bool agg = lc_in.aggr != 0;
    if (agg && !a.canvas_s) return false;
    SplatKernel k = agg ? pick_splat_ncol<true>(lc_in.ncol, shape) : pick_splat_ncol<false>(lc_in.ncol, shape);
    if (!k) return false;
    if (g_splat_optin < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_splat_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    const size_t npix = (size_t)a.resx * a.resy;
    if (npix == 0 || npix > 0xFFFFFFFFull) return false;
    LeanCols lc = lc_in;
    size_t smem = 0;
    if (kSplatShapes[shape].smem) {
        lc.copies = splat_copies(shape, npix, agg);
        if (!lc.copies) return false;
        smem = (size_t)lc.copies * npix * (agg ? 3 : 1) * 4;
        if (smem > (size_t)g_splat_optin) return false;
        if (smem > 48 * 1024 &&
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
    } else {
        lc.copies = 1;
    }
    const int block = kSplatShapes[shape].block;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        return false;
    }
    const uint64_t per_iter = (uint64_t)block * kSplatShapes[shape].nv;
    const uint64_t need = ((a.n >> 1) + per_iter - 1) / per_iter;
    uint64_t blocks = std::min<uint64_t>((uint64_t)sms * per_sm, std::max<uint64_t>(need, 1));
    // shared counts are 32-bit: a block must see fewer than 2^31 points
    while (blocks < (uint64_t)sms * per_sm && a.n / blocks >= (1ull << 31)) ++blocks;
    if (kSplatShapes[shape].smem && a.n / blocks >= (1ull << 31)) return false;
    k<<<(unsigned)blocks, block, smem, st>>>(a, lc);
    ++g_kernel_launches;
    return true;
}

}  // namespace rj
