// rj_lean_kernels.cu -- lean point pass of the raster join over a polygon
// label map (one canvas tile, polygons that do not overlap) with attribute
// filters and/or a summed aggregate: the label-map counterpart of
// points.vert:138-159 (typed predicates, floatVal) feeding the per-polygon
// sums of polygon.frag:12-27.
//
// Same structure as the plain count pass (rj_count_kernels.cu): the block-code
// map of the label canvas in shared memory, plain shared-memory atomics into
// per-warp-group histogram copies, fully coalesced loads (each lane two
// consecutive points: x, y as one float4, each 4-byte column as one uint2).
// The predicates are the interval form the host compiles them to: per column
// the query holds exactly when order_key(value) - lo <= span (unsigned); the
// order key of a float, int or uint column is value ^ ((sign & fm) ^ xm),
// branch-free.  Sums are the runtime's exact int64 fixed-point values,
// accumulated in shared memory as two 32-bit words (low word with carry into
// the high word: the pair is the sum modulo 2^64, order-independent) so that
// every shared atomic stays a native 32-bit one; non-finite values go to the
// fp64 side sum in global memory.
#include "rj_lean.cuh"

namespace rj {

template <int NCOL>
__device__ __forceinline__ bool lean_pass(const LeanCols& lc, const uint32_t (&v)[NCOL > 0 ? NCOL : 1]) {
    bool ok = true;
    #pragma unroll
    for (int c = 0; c < NCOL; ++c) {
        const uint32_t key = v[c] ^ (((uint32_t)((int32_t)v[c] >> 31) & lc.fm[c]) ^ lc.xm[c]);
        ok &= (key - lc.lo[c]) <= lc.span[c];
    }
    return ok;
}

// Adds one point of polygon l to the block's histogram copy.
template <bool AGG>
__device__ __forceinline__ void lean_add(uint32_t* h_cnt, uint32_t* h_lo, uint32_t* h_hi, const LeanCols& lc,
                                         uint32_t l, float v) {
    atomicAdd(h_cnt + l, 1u);
    if (AGG) {
        if (isfinite(v)) {
            const unsigned long long q = (unsigned long long)fixed_value(v, lc.scale);
            const uint32_t qlo = (uint32_t)q;
            const uint32_t old = atomicAdd(h_lo + l, qlo);
            atomicAdd(h_hi + l, (uint32_t)(q >> 32) + ((old + qlo < old) ? 1u : 0u));
        } else {
            atomicAdd(lc.nonfinite + l, (double)v);
        }
    }
}

template <int BLOCK, int NV, int NCOL, bool AGG>
__global__ void __launch_bounds__(BLOCK) k_label_lean(LabelCountArgs a, LeanCols lc) {
    extern __shared__ uint32_t s_words[];
    constexpr int HW = AGG ? 3 : 1;                   // count | sum low word | sum high word
    uint32_t* s_code = s_words;
    uint32_t* s_hist = s_words + a.code_words;        // lc.copies x HW x P
    {
        const uint32_t* g = reinterpret_cast<const uint32_t*>(a.codes);
        for (int i = threadIdx.x; i < a.code_words; i += BLOCK) s_code[i] = __ldg(g + i);
        for (int i = threadIdx.x; i < lc.copies * HW * a.P; i += BLOCK) s_hist[i] = 0u;
    }
    __syncthreads();
    const uint16_t* sc = reinterpret_cast<const uint16_t*>(s_code);
    const uint32_t P = (uint32_t)a.P;
    uint32_t* h_cnt = s_hist + ((threadIdx.x >> 5) & (lc.copies - 1)) * HW * a.P;
    uint32_t* h_lo = h_cnt + a.P;
    uint32_t* h_hi = h_cnt + 2 * a.P;
    const TileXf2 xf = tile_xf2(a);
    const uint2* aggr2 = lc.aggr_col;

    const uint64_t npairs = a.n >> 1;
    constexpr uint64_t kPerIter = (uint64_t)BLOCK * NV;
    const uint64_t warp_ofs = (uint64_t)(threadIdx.x >> 5) * 32 * NV;
    const uint64_t lane_ofs = warp_ofs + (threadIdx.x & 31);
    // block-uniform trip count; no barrier inside, so a warp may skip an iteration
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
        uint32_t lab[2 * NV];
        float val[2 * NV];
        #pragma unroll
        for (int j = 0; j < 2 * NV; ++j) {
            const int k = j >> 1;
            const bool hi = (j & 1) != 0;
            uint32_t v[NCOL > 0 ? NCOL : 1];
            #pragma unroll
            for (int c = 0; c < NCOL; ++c) v[c] = hi ? cv[c][k].y : cv[c][k].x;
            const float x = hi ? p[k].z : p[k].x;
            const float y = hi ? p[k].w : p[k].y;
            int px, py;
            const bool in = count_pixel(a, xf, x, y, px, py) && lean_pass<NCOL>(lc, v);
            px = in ? px : 0;
            py = in ? py : 0;
            uint32_t c = in ? (uint32_t)sc[(py >> a.bs) * a.nbx + (px >> a.bs)] : (uint32_t)kEmptyLabel;
            if (c == kCodeMixed) c = __ldg(a.label + (size_t)py * a.resx + px);
            lab[j] = c;
            val[j] = 0.f;
            if (AGG) {
                uint32_t raw = hi ? av[k].y : av[k].x;
                #pragma unroll
                for (int cc = 0; cc < NCOL; ++cc)
                    if (cc == lc.aggr_ci) raw = v[cc];
                val[j] = agg_value(lc.aggr_typ, raw);
            }
        }
        #pragma unroll
        for (int j = 0; j < 2 * NV; ++j)
            if (lab[j] < P) lean_add<AGG>(h_cnt, h_lo, h_hi, lc, lab[j], val[j]);
    }
    // the last point of an odd-sized table
    if ((a.n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const uint64_t i = a.n - 1;
        const float2 q = __ldg(reinterpret_cast<const float2*>(a.xy) + i);
        uint32_t v[NCOL > 0 ? NCOL : 1];
        #pragma unroll
        for (int c = 0; c < NCOL; ++c) v[c] = __ldg(reinterpret_cast<const uint32_t*>(lc.col[c]) + i);
        int px, py;
        if (count_pixel(a, xf, q.x, q.y, px, py) && lean_pass<NCOL>(lc, v)) {
            const uint32_t l = __ldg(a.label + (size_t)py * a.resx + px);
            if (l < P) {
                float fv = 0.f;
                if (AGG) {
                    uint32_t raw = lc.aggr_ci < 0 ? __ldg(reinterpret_cast<const uint32_t*>(aggr2) + i) : 0u;
                    #pragma unroll
                    for (int cc = 0; cc < NCOL; ++cc)
                        if (cc == lc.aggr_ci) raw = v[cc];
                    fv = agg_value(lc.aggr_typ, raw);
                }
                lean_add<AGG>(h_cnt, h_lo, h_hi, lc, l, fv);
            }
        }
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

// ---------------------------------------------------------------------------
namespace {

using LeanKernel = void (*)(LabelCountArgs, LeanCols);

struct LeanShape {
    int block;
    int nv;
};
constexpr LeanShape kLeanShapes[] = {{1024, 2}, {512, 4}, {512, 2}, {256, 4}};
constexpr int kNumLeanShapes = (int)(sizeof(kLeanShapes) / sizeof(kLeanShapes[0]));

template <int NCOL, bool AGG>
LeanKernel pick_kernel(int shape) {
    switch (shape) {
        case 0: return k_label_lean<1024, 2, NCOL, AGG>;
        case 1: return k_label_lean<512, 4, NCOL, AGG>;
        case 2: return k_label_lean<512, 2, NCOL, AGG>;
        default: return k_label_lean<256, 4, NCOL, AGG>;
    }
}

template <bool AGG>
LeanKernel pick_ncol(int ncol, int shape) {
    switch (ncol) {
        case 0: return pick_kernel<0, AGG>(shape);
        case 1: return pick_kernel<1, AGG>(shape);
        case 2: return pick_kernel<2, AGG>(shape);
        case 3: return pick_kernel<3, AGG>(shape);
        case 4: return pick_kernel<4, AGG>(shape);
        default: return nullptr;
    }
}

int g_lean_optin = -1;

}  // namespace

int label_lean_shapes() { return kNumLeanShapes; }
int label_lean_max_cols() { return 4; }

// histogram copies: a power of two up to the warps of the block, within 64 KB
int label_lean_copies(int shape, int P, bool agg) {
    if (shape < 0 || shape >= kNumLeanShapes) return 0;
    const int warps = kLeanShapes[shape].block / 32;
    int copies = 1;
    const size_t per = (size_t)P * (agg ? 3 : 1) * 4;
    while (copies * 2 <= warps && per * copies * 2 <= 64 * 1024) copies *= 2;
    return copies;
}

size_t label_lean_smem(int shape, int code_words, int P, bool agg) {
    const int copies = label_lean_copies(shape, P, agg);
    if (!copies) return 0;
    return (size_t)code_words * 4 + (size_t)copies * P * (agg ? 3 : 1) * 4;
}

bool launch_label_lean(int shape, const LabelCountArgs& a, const LeanCols& lc_in, int sms, cudaStream_t st) {
    if (shape < 0 || shape >= kNumLeanShapes || lc_in.ncol < 0 || lc_in.ncol > 4) return false;
    const bool agg = lc_in.aggr != 0;
    LeanKernel k = agg ? pick_ncol<true>(lc_in.ncol, shape) : pick_ncol<false>(lc_in.ncol, shape);
    if (!k) return false;
    if (g_lean_optin < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_lean_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    LeanCols lc = lc_in;
    lc.copies = label_lean_copies(shape, a.P, agg);
    const size_t smem = label_lean_smem(shape, a.code_words, a.P, agg);
    if (smem > (size_t)g_lean_optin) return false;
    if (smem > 48 * 1024 && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const int block = kLeanShapes[shape].block;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        return false;
    }
    const uint64_t per_iter = (uint64_t)block * kLeanShapes[shape].nv;
    const uint64_t need = ((a.n >> 1) + per_iter - 1) / per_iter;
    uint64_t blocks = std::min<uint64_t>((uint64_t)sms * per_sm, std::max<uint64_t>(need, 1));
    // shared counts are 32-bit: a block must see fewer than 2^31 points
    while (blocks < (uint64_t)sms * per_sm && a.n / blocks >= (1ull << 31)) ++blocks;
    if (a.n / blocks >= (1ull << 31)) return false;
    k<<<(unsigned)blocks, block, smem, st>>>(a, lc);
    ++g_kernel_launches;
    return true;
}

}  // namespace rj
