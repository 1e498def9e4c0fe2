// rj_device.cuh -- device-side building blocks shared by every join kernel.
//
// All floating-point arithmetic that decides a result (pixel of a point,
// crossing-number point-in-polygon) uses explicitly rounded intrinsics so
// that no multiply-add is contracted: the CPU oracle evaluates the same
// expressions operation by operation and must agree bit for bit.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "../../include/rj.h"

namespace rj {

constexpr int kMaxFilters = RJ_MAX_CONSTRAINTS + 2;   // + time range (2 predicates)
constexpr uint16_t kEmptyLabel = 0xFFFFu;     // pixel covered by no polygon
constexpr uint16_t kBorderLabel = 0xFFFEu;    // hybrid: pixel near an outline
constexpr int kMaxLabelPolys = 0xFFFD;        // polygon ids that fit a 16-bit label
constexpr uint32_t kCodeEmpty = 0xFFFFFFFFu;  // classified cell without polygons
constexpr uint32_t kCodeList = 0x80000000u;   // classified cell: consult the entry list
constexpr int kSubpixelBits = 8;                      // GL_SUBPIXEL_BITS on NVIDIA
constexpr int kSub = 1 << kSubpixelBits;              // 256 fixed-point units per pixel
constexpr float kWinClamp = 1048576.0f;               // |window coord| clamp (2^20 px)

// ---------------------------------------------------------------------------
// Filter + aggregate description (GLFunction::setupPoints GLFunction.cpp:199-344
// gathers constraint columns; points.vert:138-159 evaluates them).
struct DevFilter {
    int ncol;                                // distinct columns the predicates read
    const uint32_t* col[kMaxFilters];
    // Interval form (general == 0): the predicates of column c hold exactly
    // when order_key(ctyp[c], value) - lo[c] <= span[c] (unsigned).
    int general;
    int ctyp[kMaxFilters];
    uint32_t lo[kMaxFilters], span[kMaxFilters];
    // General form: predicates of column c: [pstart[c], pstart[c+1])
    int pstart[kMaxFilters + 1];
    int n;                                   // predicates (constraints + time range)
    int op[kMaxFilters];                     // rj_constraint_type
    int typ[kMaxFilters];                    // rj_attribute_type of the column
    uint32_t val[kMaxFilters];               // comparison value (bit pattern)
    uint32_t compat_mask;                    // bit k: predicate k uses RJ_FLAG_COMPAT_FLOAT_EQ
    int aggr;                                // 0: count only, else sum of aggr_col
    int aggr_typ;
    int aggr_ci;                             // index of aggr_col in col[], or -1
    const uint32_t* aggr_col;
    float sum_scale;                         // 2^(s-32): values are summed as int64 round(v * 2^s)
};

// Fixed-point value of an aggregate: round(v * 2^s) as int64, from only
// 32-bit conversions (t = v * 2^(s-32) = hi + r with hi = floor(t), r in
// [0,1); r * 2^32 needs rounding only when |t| < 1).  |v| * 2^s < 2^63 by the
// choice of s; non-finite values are summed separately in fp64.
__device__ __forceinline__ long long fixed_value(float v, float scale) {
    const float t = __fmul_rn(v, scale);
    const float hi = floorf(t);
    const float r = __fsub_rn(t, hi);
    const unsigned lo = __float2uint_rn(__fmul_rn(r, 4294967296.0f));
    return (long long)(((unsigned long long)(long long)(int)hi << 32) + (unsigned long long)lo);
}

// aLessThan / aGreaterThan / aEqual, points.vert:24-85: Uint and Int compare
// the reinterpreted bits, Float compares as fp32; Location (or anything else)
// yields true.
__host__ __device__ __forceinline__ bool pred_less(int typ, uint32_t a, uint32_t f) {
    switch (typ) {
        case RJ_UINT: return a < f;
        case RJ_INT: return (int32_t)a < (int32_t)f;
        case RJ_FLOAT: {
            float af, ff;
            memcpy(&af, &a, 4); memcpy(&ff, &f, 4);
            return af < ff;
        }
        default: return true;
    }
}
__host__ __device__ __forceinline__ bool pred_greater(int typ, uint32_t a, uint32_t f) {
    switch (typ) {
        case RJ_UINT: return a > f;
        case RJ_INT: return (int32_t)a > (int32_t)f;
        case RJ_FLOAT: {
            float af, ff;
            memcpy(&af, &a, 4); memcpy(&ff, &f, 4);
            return af > ff;
        }
        default: return true;
    }
}
__host__ __device__ __forceinline__ bool pred_equal(int typ, uint32_t a, uint32_t f) {
    switch (typ) {
        case RJ_UINT: return a == f;
        case RJ_INT: return (int32_t)a == (int32_t)f;
        case RJ_FLOAT: {
            float af, ff;
            memcpy(&af, &a, 4); memcpy(&ff, &f, 4);
            return af == ff;
        }
        default: return true;
    }
}
// validFilter, points.vert:87-114.  LTE/GTE add an equality test that the
// reference writes as a float comparison of the raw bits
// (`filterVal == attributes[aid-1]`, points.vert:99,107); by default the
// equality is typed, RJ_FLAG_COMPAT_FLOAT_EQ selects the float comparison.
__host__ __device__ __forceinline__ bool pred_eval(int op, int typ, uint32_t a, uint32_t f, int compat) {
    bool eq_ext = false;
    if (op == RJ_LTE || op == RJ_GTE) {
        if (compat) {
            float af, ff;
            memcpy(&af, &a, 4); memcpy(&ff, &f, 4);
            eq_ext = (ff == af);
        } else {
            eq_ext = pred_equal(typ, a, f);
        }
    }
    switch (op) {
        case RJ_EQ: return pred_equal(typ, a, f);
        case RJ_LT: return pred_less(typ, a, f);
        case RJ_LTE: return pred_less(typ, a, f) || eq_ext;
        case RJ_GT: return pred_greater(typ, a, f);
        case RJ_GTE: return pred_greater(typ, a, f) || eq_ext;
        default: return false;
    }
}

// floatVal, points.vert:116-136: the aggregate value as fp32.
__host__ __device__ __forceinline__ float agg_value(int typ, uint32_t a) {
    switch (typ) {
        case RJ_UINT: return (float)a;
        case RJ_INT: return (float)(int32_t)a;
        case RJ_FLOAT: { float af; memcpy(&af, &a, 4); return af; }
        default: return 0.0f;
    }
}

// Order-preserving map of a 4-byte value to uint32: unsigned compare of the
// keys equals the typed compare of the values (floats: -NaN < -inf < ... <
// -0 < +0 < ... < +inf < +NaN; the intervals exclude the NaNs).
__host__ __device__ __forceinline__ uint32_t order_key(int typ, uint32_t a) {
    if (typ == RJ_INT) return a ^ 0x80000000u;
    if (typ == RJ_FLOAT) return (a & 0x80000000u) ? ~a : (a | 0x80000000u);
    return a;
}

__device__ __forceinline__ bool filter_point(const DevFilter& f, uint64_t i) {
    #pragma unroll 1
    for (int c = 0; c < f.ncol; ++c) {
        const uint32_t a = __ldg(f.col[c] + i);
        if (!f.general) {
            if (order_key(f.ctyp[c], a) - f.lo[c] > f.span[c]) return false;
            continue;
        }
        for (int k = f.pstart[c]; k < f.pstart[c + 1]; ++k)
            if (!pred_eval(f.op[k], f.typ[k], a, f.val[k], (int)((f.compat_mask >> k) & 1u))) return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// Raster canvas geometry (RasterJoin::updateBuffers RasterJoin.cpp:51-78, tile
// loop :224-231, getMVP Utils.h:36-46).  One tile's model-view-projection is a
// scale and a translation held in fp32 (QMatrix4x4); the viewport maps NDC to
// window pixels.
struct TileXf {
    float sx, tx, sy, ty;     // ndc = s*world + t
    float hx, hy;             // res/2 per axis
};

// world -> window coordinate along one axis: ndc = fl(fl(s*v) + t);
// window = fl(fl(h*ndc) + h)  (GL viewport transform, origin 0).
__host__ __device__ __forceinline__ float win_coord(float v, float s, float t, float h) {
#ifdef __CUDA_ARCH__
    float ndc = __fadd_rn(__fmul_rn(s, v), t);
    return __fadd_rn(__fmul_rn(h, ndc), h);
#else
    volatile float p = s * v;
    volatile float ndc = p + t;
    volatile float q = h * ndc;
    return q + h;
#endif
}

// Snap a window coordinate to the 1/256-pixel lattice, round to nearest even.
__host__ __device__ __forceinline__ int32_t snap_win(float w) {
    w = fminf(fmaxf(w, -kWinClamp), kWinClamp);
#ifdef __CUDA_ARCH__
    return __float2int_rn(__fmul_rn(w, (float)kSub));
#else
    return (int32_t)lrintf(w * (float)kSub);
#endif
}

__host__ __device__ __forceinline__ int64_t floordiv64(int64_t a, int64_t b) {
    // b > 0
    int64_t q = a / b;
    if ((a % b != 0) && (a < 0)) --q;
    return q;
}

// Pixel column of a snapped point coordinate: floor(X/256).
__host__ __device__ __forceinline__ int32_t pix_of(int32_t X) {
    return X >> kSubpixelBits;   // arithmetic shift == floor division by 256
}

// Exact edge-function crossing for the pixel-centre fill rule.  Vertices are
// fixed-point window coordinates.  Row centre Cy (fixed point).  The edge
// (A,B) crosses the row iff (A.y >= Cy) != (B.y >= Cy) (top-closed, as GL's
// top-left rule).  It then toggles every pixel i whose centre lies strictly
// left of the exact intersection x; those are the pixels i < L with
// L = ceil((x_int - 128)/256).  Returns L (may be <0 or >res; caller clamps).
__host__ __device__ __forceinline__ int32_t cross_L(int32_t ax, int32_t ay, int32_t bx, int32_t by, int32_t cy) {
    int64_t dy = (int64_t)by - ay;
    int64_t num = ((int64_t)ax - (kSub / 2)) * dy + ((int64_t)bx - ax) * ((int64_t)cy - ay);
    int64_t den = dy * kSub;
    if (den < 0) { num = -num; den = -den; }
    // ceil(num/den)
    int64_t q = floordiv64(num, den);
    if (q * den != num) ++q;
    if (q > (int64_t)0x3fffffff) q = 0x3fffffff;
    if (q < -(int64_t)0x3fffffff) q = -0x3fffffff;
    return (int32_t)q;
}
__host__ __device__ __forceinline__ bool cross_row(int32_t ay, int32_t by, int32_t cy) {
    return (ay >= cy) != (by >= cy);
}

// ---------------------------------------------------------------------------
// Crossing-number point-in-polygon, index.glsl:47-67 / GridIndexF.cpp:383-402,
// evaluated in fp32 with the reference's expression order
// (vj.x - vi.x) * (testy - vi.y) / (vj.y - vi.y) + vi.x.
//
// The comparison needs the exactly rounded crossing xi only when tx lies
// close to it.  A fast quotient (__fdividef, within 2 ulp while |den| is in
// [2^-126, 2^126]) gives xa with |xi - xa| <= 2^-21 (|q| + |vix|); when tx is
// farther than twice that from xa the answer is the same as the exact one,
// else the exact division decides.  Results are identical to the always
// exact form; most tests skip the IEEE division.
__device__ __forceinline__ bool edge_toggles(float vix, float viy, float vjx, float vjy, float tx, float ty) {
    if ((viy > ty) != (vjy > ty)) {
        const float num = __fmul_rn(__fsub_rn(vjx, vix), __fsub_rn(ty, viy));
        const float den = __fsub_rn(vjy, viy);
        const float ad = fabsf(den);
        if (ad > 1e-30f && ad < 1e30f) {
            const float qa = __fdividef(num, den);
            const float xa = qa + vix;
            const float tol = (fabsf(qa) + fabsf(vix)) * 1e-6f;
            if (tx < xa - tol) return true;
            if (tx > xa + tol) return false;
        }
        const float xi = __fadd_rn(__fdiv_rn(num, den), vix);
        return tx < xi;
    }
    return false;
}

__device__ __forceinline__ bool pip_f32(const float2* __restrict__ v, int n, float tx, float ty) {
    bool c = false;
    float2 vj = __ldg(v + (n - 1));
    for (int i = 0; i < n; ++i) {
        float2 vi = __ldg(v + i);
        if (edge_toggles(vi.x, vi.y, vj.x, vj.y, tx, ty)) c = !c;
        vj = vi;
    }
    return c;
}

// Grid cell of a point, index.glsl:382-385: int() truncates toward zero.
__device__ __forceinline__ int grid_cell_1d(float p, float lb, float cs) {
    return __float2int_rz(__fdiv_rn(__fsub_rn(p, lb), cs));
}

// ---------------------------------------------------------------------------
// Hybrid canvas pixel of a point, hybrid.glsl:187-200 (rasterize): half-open
// [-1,1) in normalised coordinates, fp32 throughout.
struct HybXf {
    float ox, oy;      // origin = (rightTop + leftBottom)/2
    float dx, dy;      // diff = (rightTop - leftBottom)/2
    int resx, resy;    // fboRes
};
__device__ __forceinline__ bool hyb_rasterize(const HybXf& h, float x, float y, int& px, int& py) {
    float u = __fdiv_rn(__fsub_rn(x, h.ox), h.dx);
    float v = __fdiv_rn(__fsub_rn(y, h.oy), h.dy);
    // outside [-1,1) -- and NaN, which lies in no polygon (the exact test's
    // grid cell rejects it)
    if (!(u >= -1.0f && u < 1.0f && v >= -1.0f && v < 1.0f)) return false;
    u = __fmul_rn(__fadd_rn(u, 1.0f), 0.5f);
    v = __fmul_rn(__fadd_rn(v, 1.0f), 0.5f);
    px = __float2int_rz(__fmul_rn(u, (float)h.resx));
    py = __float2int_rz(__fmul_rn(v, (float)h.resy));
    return true;
}

// ---------------------------------------------------------------------------
// Warp helpers
__device__ __forceinline__ int warp_min(int v) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_max(int v) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_minf(float v) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_maxf(float v) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// The work item's owner: the last index tp in [0, n) with start[tp] <= item,
// for a nondecreasing start[] with start[0] == 0 <= item.  Called by the whole
// warp: each round the 32 lanes probe evenly spaced entries and the range
// shrinks to the gap between the last probe at or below item and the next,
// so a search over n entries takes ceil(log32 n) dependent loads instead of
// log2 n.
__device__ __forceinline__ int warp_find_owner(const int* __restrict__ start, int n, int item, int lane) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int step = (hi - lo + 32) >> 5;   // ceil((hi - lo + 1) / 32)
        const int pos = min(lo + lane * step, hi);
        const unsigned le = __ballot_sync(0xffffffffu, __ldg(start + pos) <= item);
        const int last = 31 - __clz(le);          // lane 0 probes lo: le != 0
        const int plast = min(lo + last * step, hi);
        const int pnext = last < 31 ? min(lo + (last + 1) * step, hi) : hi + 1;
        lo = plast;
        hi = (pnext > plast) ? min(pnext - 1, hi) : hi;
    }
    return lo;
}
__device__ __forceinline__ double warp_sum_f64(double v) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace rj

// ---------------------------------------------------------------------------
// Bulk-copy pipeline primitives (mbarrier + cp.async.bulk, sm_90+ PTX).
namespace rj {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// One try on the phase of the given parity; a thread whose phase is not
// complete may be suspended up to about hint_ns before the try returns false.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity, uint32_t hint_ns) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Wait for the phase of the given parity to complete, bounded in wall time:
// false once limit_ns nanoseconds have passed (the caller records an error
// and stops).  The bound is time, not tries: a try may suspend the thread.
constexpr uint64_t kWaitLimitNs = 1000000000ull;   // 1 s
__device__ __forceinline__ bool mbar_wait_ns(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity, 1000u)) return true;
    const uint64_t t0 = global_ns();
    do {
        if (mbar_try_wait(bar, parity, 2000u)) return true;
    } while (global_ns() - t0 < limit_ns);
    return false;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    return mbar_wait_ns(bar, parity, kWaitLimitNs);
}
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
// global -> shared bulk copy completing on an mbarrier (16-byte aligned, size % 16 == 0)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar, uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}
__device__ __forceinline__ void named_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

}  // namespace rj
