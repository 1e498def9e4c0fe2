// rj_hybrid_lean.cu -- lean point pass of the hybrid join (hybrid.glsl:224-300,
// HybridJoin::glJoin HybridJoin.cpp:87-195) over the hybrid canvas's polygon
// label map, and of the index join (index.glsl:186-248) over the classified
// grid's cell labels, with interval-form filters on up to four columns and
// an optional summed aggregate.
//
// Per point: the predicates, the hybrid canvas pixel (rasterize,
// hybrid.glsl:187-200), then the pixel's label through the block-code map in
// shared memory (the label map in L2 only for blocks whose pixels differ).
// A labelled pixel is inside exactly one polygon and away from every
// outline: the point goes to that polygon's histogram (plain shared-memory
// atomics, count and two-word fixed-point sum as in rj_lean_kernels.cu).  A
// pixel marked border (within the fp32 error radius of an outline, isBorder
// hybrid.glsl:174-185) sends the point to the exact test through the
// classified grid: such points are appended to a block-wide queue with one
// atomic per warp (ballot + prefix, no divergent per-lane appends) and run
// in full blocks, one point per thread, when the queue holds a block's worth.
#include "rj_lean.cuh"
#include "rj_point_core.cuh"

namespace rj {

namespace {

// Hist-like adapter for exact_probe: adds to the block's histogram copy.
template <bool AGG>
struct LeanHist {
    uint32_t* cnt;
    uint32_t* lo;
    uint32_t* hi;
    const LeanCols* lc;
    __device__ __forceinline__ void add(int p, float v) const {
        atomicAdd(cnt + p, 1u);
        if (AGG) {
            if (isfinite(v)) {
                const unsigned long long q = (unsigned long long)fixed_value(v, lc->scale);
                const uint32_t qlo = (uint32_t)q;
                const uint32_t old = atomicAdd(lo + p, qlo);
                atomicAdd(hi + p, (uint32_t)(q >> 32) + ((old + qlo < old) ? 1u : 0u));
            } else {
                atomicAdd(lc->nonfinite + p, (double)v);
            }
        }
    }
};

template <int NCOL>
__device__ __forceinline__ bool hyb_pass(const LeanCols& lc, const uint32_t (&v)[NCOL > 0 ? NCOL : 1]) {
    bool ok = true;
    #pragma unroll
    for (int c = 0; c < NCOL; ++c) {
        const uint32_t key = v[c] ^ (((uint32_t)((int32_t)v[c] >> 31) & lc.fm[c]) ^ lc.xm[c]);
        ok &= (key - lc.lo[c]) <= lc.span[c];
    }
    return ok;
}

// kind of a point: 0 none, 1 labelled (label in *lab), 2 border (exact test).
//
// Hybrid canvas (mode 0): a labelled pixel lies in one polygon with no edge
// within the border radius (at least one pixel) of it, so every location
// within that slack of the pixel is inside the same polygon under the exact
// test.  The pixel therefore only has to be found to far better than a pixel,
// not bit for bit: one FMA per axis (error ~1e-4 px on a 4096-pixel canvas)
// instead of hybrid.glsl's two divisions.  Within 2 pixels of the canvas rim
// the exact rasterize decides, so the canvas bounds (half-open [-1, 1),
// hybrid.glsl:187-200) and NaN are handled exactly as before.
// Classified grid (mode 1): the cell of the exact test itself (index.glsl:
// 382-385, fp32 division, int() truncation), as the ExactMapper computes it.
__device__ __forceinline__ int hyb_classify(const HybLeanArgs& a, const uint16_t* sc, float x, float y, uint32_t& lab) {
    int px, py, resx;
    if (a.mode == 0) {
        resx = a.h.resx;
        const float fx = fmaf(x, a.fast.x, a.fast.y), fy = fmaf(y, a.fast.z, a.fast.w);
        if (fx >= 2.0f && fx < (float)(a.h.resx - 2) && fy >= 2.0f && fy < (float)(a.h.resy - 2)) {
            px = (int)fx;
            py = (int)fy;
        } else {
            if (!hyb_rasterize(a.h, x, y, px, py)) return 0;
            if (px >= a.h.resx || py >= a.h.resy) return 2;
        }
    } else {
        resx = a.ix.res;
        const float gx = __fdiv_rn(__fsub_rn(x, a.ix.lbx), a.ix.csx);
        const float gy = __fdiv_rn(__fsub_rn(y, a.ix.lby), a.ix.csy);
        if (!(gx > -1.0f && gx < (float)a.ix.res && gy > -1.0f && gy < (float)a.ix.res)) return 0;
        px = (int)gx;
        py = (int)gy;
    }
    uint32_t c = sc[(py >> a.bs) * a.nbx + (px >> a.bs)];
    if (c == kCodeMixed) c = __ldg(a.label + (size_t)py * resx + px);
    if (c == kBorderLabel) return 2;
    lab = c;
    return c < (uint32_t)a.P ? 1 : 0;
}

}  // namespace

// A classified point: a labelled one into the histogram, a border one into
// the block's queue (one reservation per warp: ballot + prefix; every lane of
// the warp calls this).
template <bool AGG>
__device__ __forceinline__ void hyb_take(const LeanHist<AGG>& hist, int* qn, float* qx, float* qy, float* qv,
                                         int lane, int kind, uint32_t lab, float x, float y, float val) {
    if (kind == 1) hist.add((int)lab, val);
    const unsigned m = __ballot_sync(0xffffffffu, kind == 2);
    if (m) {
        int at = 0;
        if (lane == 0) at = atomicAdd(qn, __popc(m));
        at = __shfl_sync(0xffffffffu, at, 0);
        if (kind == 2) {
            const int s = at + __popc(m & ((1u << lane) - 1u));
            qx[s] = x;
            qy[s] = y;
            qv[s] = val;
        }
    }
}

// COMPACT: the points that pass the filters are first packed per warp into
// shared memory (ballot + prefix), then classified and counted 32 at a time,
// so that the pixel, label and histogram work runs on full warps even when
// the filters drop most points.
template <int BLOCK, int NV, int NCOL, bool AGG, bool COMPACT>
__device__ __forceinline__ void hybrid_lean_body(const HybLeanArgs& a, const LeanCols& lc) {
    extern __shared__ uint32_t s_words[];
    constexpr int HW = AGG ? 3 : 1;
    constexpr int QCAP = BLOCK * (1 + 2 * NV);        // < BLOCK left over + every point of one iteration
    constexpr int WCAP = 32 * 2 * NV;                 // one warp's points of one iteration
    uint32_t* s_code = s_words;
    uint32_t* s_hist = s_code + a.code_words;          // lc.copies x HW x P
    float* qx = reinterpret_cast<float*>(s_hist + lc.copies * HW * a.P);
    float* qy = qx + QCAP;
    float* qv = qy + QCAP;
    int* qn = reinterpret_cast<int*>(qv + QCAP);
    // per-warp staging of the points that pass the filters (COMPACT)
    float* wx = reinterpret_cast<float*>(qn + 4) + (threadIdx.x >> 5) * WCAP * (AGG ? 3 : 2);
    float* wy = wx + WCAP;
    float* wv = wy + WCAP;
    {
        const uint32_t* g = reinterpret_cast<const uint32_t*>(a.codes);
        for (int i = threadIdx.x; i < a.code_words; i += BLOCK) s_code[i] = __ldg(g + i);
        for (int i = threadIdx.x; i < lc.copies * HW * a.P; i += BLOCK) s_hist[i] = 0u;
        if (threadIdx.x == 0) *qn = 0;
    }
    __syncthreads();
    const uint16_t* sc = reinterpret_cast<const uint16_t*>(s_code);
    uint32_t* h_cnt = s_hist + ((threadIdx.x >> 5) & (lc.copies - 1)) * HW * a.P;
    const LeanHist<AGG> hist{h_cnt, h_cnt + a.P, h_cnt + 2 * a.P, &lc};
    const int lane = threadIdx.x & 31;

    const uint64_t npairs = a.n >> 1;
    constexpr uint64_t kPerIter = (uint64_t)BLOCK * NV;
    const uint64_t warp_ofs = (uint64_t)(threadIdx.x >> 5) * 32 * NV;
    const uint64_t lane_ofs = warp_ofs + lane;
    // block-uniform trip count (the queue drain below has block barriers)
    for (uint64_t base = (uint64_t)blockIdx.x * kPerIter; base < npairs; base += (uint64_t)gridDim.x * kPerIter) {
        bool skip = false;
        if (a.zones) {
            const uint64_t r0 = a.zrow0 + 2 * (base + warp_ofs);
            const uint64_t r1 = a.zrow0 + min(2 * (base + warp_ofs + 32 * NV), a.n) - 1;
            bool meets = false;
            if (r0 <= r1 && (uint64_t)lane <= (r1 >> kZoneShift) - (r0 >> kZoneShift)) {
                const float4 b = __ldg(a.zones + (r0 >> kZoneShift) + lane);
                meets = !(b.z < a.qbox.x || b.x > a.qbox.z || b.w < a.qbox.y || b.y > a.qbox.w);
            }
            skip = !__any_sync(0xffffffffu, meets);
        }
        if (!skip) {
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
                if (AGG) av[k] = (live && lc.aggr_ci < 0) ? __ldcs(lc.aggr_col + i) : make_uint2(0u, 0u);
            }
            int nst = 0;                               // staged points of this warp (COMPACT)
            #pragma unroll
            for (int j = 0; j < 2 * NV; ++j) {
                const int k = j >> 1;
                const bool hi = (j & 1) != 0;
                uint32_t v[NCOL > 0 ? NCOL : 1];
                #pragma unroll
                for (int c = 0; c < NCOL; ++c) v[c] = hi ? cv[c][k].y : cv[c][k].x;
                const float x = hi ? p[k].z : p[k].x;
                const float y = hi ? p[k].w : p[k].y;
                float val = 0.f;
                if (AGG) {
                    uint32_t raw = hi ? av[k].y : av[k].x;
                    #pragma unroll
                    for (int cc = 0; cc < NCOL; ++cc)
                        if (cc == lc.aggr_ci) raw = v[cc];
                    val = agg_value(lc.aggr_typ, raw);
                }
                if (COMPACT) {
                    const bool ok = hyb_pass<NCOL>(lc, v);
                    const unsigned m = __ballot_sync(0xffffffffu, ok);
                    if (ok) {
                        const int s = nst + __popc(m & ((1u << lane) - 1u));
                        wx[s] = x;
                        wy[s] = y;
                        if (AGG) wv[s] = val;
                    }
                    nst += __popc(m);
                } else {
                    uint32_t lab = 0;
                    const int kind = hyb_pass<NCOL>(lc, v) ? hyb_classify(a, sc, x, y, lab) : 0;
                    hyb_take<AGG>(hist, qn, qx, qy, qv, lane, kind, lab, x, y, val);
                }
            }
            if (COMPACT) {
                __syncwarp();
                for (int kb = 0; kb < nst; kb += 32) {
                    const int k = kb + lane;
                    const bool live = k < nst;
                    const float x = live ? wx[k] : 0.f, y = live ? wy[k] : 0.f;
                    const float val = (AGG && live) ? wv[k] : 0.f;
                    uint32_t lab = 0;
                    const int kind = live ? hyb_classify(a, sc, x, y, lab) : 0;
                    hyb_take<AGG>(hist, qn, qx, qy, qv, lane, kind, lab, x, y, val);
                }
                __syncwarp();
            }
        }
        // drain full blocks of queued points, one point per thread
        __syncthreads();
        while (*qn >= BLOCK) {
            const int s = *qn - BLOCK + (int)threadIdx.x;
            exact_probe(a.ix, qx[s], qy[s], qv[s], hist);
            __syncthreads();
            if (threadIdx.x == 0) *qn -= BLOCK;
            __syncthreads();
        }
    }
    // the last point of an odd-sized table
    if ((a.n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const uint64_t i = a.n - 1;
        const float2 q = __ldg(reinterpret_cast<const float2*>(a.xy) + i);
        uint32_t v[NCOL > 0 ? NCOL : 1];
        #pragma unroll
        for (int c = 0; c < NCOL; ++c) v[c] = __ldg(reinterpret_cast<const uint32_t*>(lc.col[c]) + i);
        float val = 0.f;
        if (AGG) {
            uint32_t raw = lc.aggr_ci < 0 ? __ldg(reinterpret_cast<const uint32_t*>(lc.aggr_col) + i) : 0u;
            #pragma unroll
            for (int cc = 0; cc < NCOL; ++cc)
                if (cc == lc.aggr_ci) raw = v[cc];
            val = agg_value(lc.aggr_typ, raw);
        }
        uint32_t lab = 0;
        const int kind = hyb_pass<NCOL>(lc, v) ? hyb_classify(a, sc, q.x, q.y, lab) : 0;
        if (kind == 1) hist.add((int)lab, val);
        if (kind == 2) exact_probe(a.ix, q.x, q.y, val, hist);
    }
    __syncthreads();
    {
        const int cnt = *qn;
        if ((int)threadIdx.x < cnt) exact_probe(a.ix, qx[threadIdx.x], qy[threadIdx.x], qv[threadIdx.x], hist);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < a.P; b += BLOCK) {
        uint32_t cnt = 0;
        unsigned long long sum = 0;
        #pragma unroll 1
        for (int w = 0; w < lc.copies; ++w) {
            const uint32_t* h = s_hist + w * HW * a.P;
            cnt += h[b];
            if (AGG) sum += ((unsigned long long)h[2 * a.P + b] << 32) + h[a.P + b];
        }
        if (cnt) {
            atomicAdd(a.out_count + b, (unsigned long long)cnt);
            if (AGG) atomicAdd(lc.out_sum + b, sum);
        }
    }
}

template <int BLOCK, int NV, int NCOL, bool AGG, bool COMPACT>
__global__ void __launch_bounds__(BLOCK) k_hybrid_lean(HybLeanArgs a, LeanCols lc) {
    hybrid_lean_body<BLOCK, NV, NCOL, AGG, COMPACT>(a, lc);
}

// The same pass with a register budget of two blocks per SM (64 registers at
// 512 threads): no spills, fewer resident warps.  The tuner decides.
template <int BLOCK, int NV, int NCOL, bool AGG, bool COMPACT>
__global__ void __launch_bounds__(BLOCK, 2) k_hybrid_lean_r2(HybLeanArgs a, LeanCols lc) {
    hybrid_lean_body<BLOCK, NV, NCOL, AGG, COMPACT>(a, lc);
}

// 16-bit cell labels of the classified grid for the lean pass (mode 1).
__global__ void k_cell_labels(const uint32_t* __restrict__ code, int ncells, uint16_t* __restrict__ label) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
        const uint32_t v = __ldg(code + c);
        label[c] = v < kCodeList ? (uint16_t)v : (v == kCodeEmpty ? kEmptyLabel : kBorderLabel);
    }
}

void launch_cell_labels(const uint32_t* code, int ncells, uint16_t* label, int sms, cudaStream_t st) {
    const int blocks = std::max(1, std::min((ncells + 255) / 256, sms * 8));
    k_cell_labels<<<blocks, 256, 0, st>>>(code, ncells, label);
    ++g_kernel_launches;
}

// ---------------------------------------------------------------------------
namespace {

using HybKernel = void (*)(HybLeanArgs, LeanCols);

struct HybShape {
    int block;
    int nv;
    bool compact;
};
// 3 and 6: the register budget of two blocks per SM
constexpr HybShape kHybShapes[] = {{512, 2, false}, {1024, 2, false}, {256, 4, false}, {512, 2, false},
                                   {512, 2, true},  {256, 4, true},   {512, 2, true},  {1024, 2, true},
                                   {512, 1, true}};
constexpr int kNumHybShapes = (int)(sizeof(kHybShapes) / sizeof(kHybShapes[0]));

template <int NCOL, bool AGG>
HybKernel pick_hyb(int shape) {
    switch (shape) {
        case 0: return k_hybrid_lean<512, 2, NCOL, AGG, false>;
        case 1: return k_hybrid_lean<1024, 2, NCOL, AGG, false>;
        case 2: return k_hybrid_lean<256, 4, NCOL, AGG, false>;
        case 3: return k_hybrid_lean_r2<512, 2, NCOL, AGG, false>;
        case 4: return k_hybrid_lean<512, 2, NCOL, AGG, true>;
        case 5: return k_hybrid_lean<256, 4, NCOL, AGG, true>;
        case 6: return k_hybrid_lean_r2<512, 2, NCOL, AGG, true>;
        case 7: return k_hybrid_lean<1024, 2, NCOL, AGG, true>;
        default: return k_hybrid_lean<512, 1, NCOL, AGG, true>;
    }
}

template <bool AGG>
HybKernel pick_hyb_ncol(int ncol, int shape) {
    switch (ncol) {
        case 0: return pick_hyb<0, AGG>(shape);
        case 1: return pick_hyb<1, AGG>(shape);
        case 2: return pick_hyb<2, AGG>(shape);
        case 3: return pick_hyb<3, AGG>(shape);
        case 4: return pick_hyb<4, AGG>(shape);
        default: return nullptr;
    }
}

int g_hyb_optin = -1;

int hyb_copies(int shape, int P, bool agg) {
    const int warps = kHybShapes[shape].block / 32;
    int copies = 1;
    const size_t per = (size_t)P * (agg ? 3 : 1) * 4;
    while (copies * 2 <= warps && per * copies * 2 <= 48 * 1024) copies *= 2;
    return copies;
}

}  // namespace

int hybrid_lean_shapes() { return kNumHybShapes; }

size_t hybrid_lean_smem(int shape, int code_words, int P, bool agg) {
    if (shape < 0 || shape >= kNumHybShapes) return 0;
    const HybShape& s = kHybShapes[shape];
    const size_t qcap = (size_t)s.block * (1 + 2 * s.nv);
    const size_t stage = s.compact ? (size_t)s.block * 2 * s.nv * (agg ? 3 : 2) * 4 : 0;   // per-warp staging
    return (size_t)code_words * 4 + (size_t)hyb_copies(shape, P, agg) * P * (agg ? 3 : 1) * 4 + qcap * 12 + 16 + stage;
}

bool launch_hybrid_lean(int shape, const HybLeanArgs& a, const LeanCols& lc_in, int sms, cudaStream_t st) {
    if (shape < 0 || shape >= kNumHybShapes || lc_in.ncol < 0 || lc_in.ncol > 4) return false;
    const bool agg = lc_in.aggr != 0;
    HybKernel k = agg ? pick_hyb_ncol<true>(lc_in.ncol, shape) : pick_hyb_ncol<false>(lc_in.ncol, shape);
    if (!k) return false;
    if (g_hyb_optin < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_hyb_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    LeanCols lc = lc_in;
    lc.copies = hyb_copies(shape, a.P, agg);
    const size_t smem = hybrid_lean_smem(shape, a.code_words, a.P, agg);
    if (smem > (size_t)g_hyb_optin) return false;
    if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const int block = kHybShapes[shape].block;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        return false;
    }
    const uint64_t per_iter = (uint64_t)block * kHybShapes[shape].nv;
    const uint64_t need = ((a.n >> 1) + per_iter - 1) / per_iter;
    uint64_t blocks = std::min<uint64_t>((uint64_t)sms * per_sm, std::max<uint64_t>(need, 1));
    while (blocks < (uint64_t)sms * per_sm && a.n / blocks >= (1ull << 31)) ++blocks;
    if (a.n / blocks >= (1ull << 31)) return false;
    k<<<(unsigned)blocks, block, smem, st>>>(a, lc);
    ++g_kernel_launches;
    return true;
}

}  // namespace rj
