// rj_point_kernels.cu -- point passes of the raster joins (label, splat and
// tiered canvas forms), the zone map and the column statistics.  The kernels
// and mappers are in rj_point_core.cuh.
#include "rj_point_core.cuh"

namespace rj {

void launch_raster_splat(const PointArgs& pa, const CanvasXf& cx, uint32_t* canvas_c, long long* canvas_s,
                         int sms, cudaStream_t st) {
    const size_t npix = (size_t)cx.resx * cx.resy;
    PointArgs p2 = pa;
    if (cx.splitx == 1 && cx.splity == 1 && npix <= (size_t)kSplatPrivPixels) {
        // small canvas: per-block private canvas in shared memory, flushed once
        SplatMapper m{cx, canvas_c, canvas_s, pa.f.sum_scale, pa.out_nonfinite, 1};
        p2.P = (int)npix;
        p2.out_count = nullptr;
        p2.out_count32 = canvas_c;
        p2.out_sum = reinterpret_cast<unsigned long long*>(canvas_s);
        if (pa.f.aggr) launch_points_t<SplatMapper, true, true>(p2, m, sms, st);
        else launch_points_t<SplatMapper, false, true>(p2, m, sms, st);
        return;
    }
    // the splat writes the canvas directly: no per-polygon histogram
    SplatMapper m{cx, canvas_c, canvas_s, pa.f.sum_scale, pa.out_nonfinite, 0};
    p2.P = 0;
    if (pa.f.aggr) launch_points_t<SplatMapper, true, false>(p2, m, sms, st);
    else launch_points_t<SplatMapper, false, false>(p2, m, sms, st);
}

// Zone map: one warp per kZoneRows rows; NaN coordinates drop out.
__global__ void k_zone_boxes(const float2* __restrict__ xy, uint64_t n, float4* __restrict__ zones) {
    const uint64_t nz = (n + (1ull << kZoneShift) - 1) >> kZoneShift;
    const int lane = threadIdx.x & 31;
    for (uint64_t z = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; z < nz;
         z += ((uint64_t)gridDim.x * blockDim.x) >> 5) {
        float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
        const uint64_t a = z << kZoneShift, b = (n < a + (1ull << kZoneShift)) ? n : a + (1ull << kZoneShift);
        for (uint64_t i = a + lane; i < b; i += 32) {
            const float2 p = __ldcs(xy + i);
            x0 = fminf(x0, p.x); x1 = fmaxf(x1, p.x);
            y0 = fminf(y0, p.y); y1 = fmaxf(y1, p.y);
        }
        x0 = warp_minf(x0); x1 = warp_maxf(x1);
        y0 = warp_minf(y0); y1 = warp_maxf(y1);
        if (lane == 0) zones[z] = make_float4(x0, y0, x1, y1);
    }
}

void launch_zone_boxes(const float2* xy, uint64_t n, float4* zones, int sms, cudaStream_t st) {
    const uint64_t nz = (n + (1ull << kZoneShift) - 1) >> kZoneShift;
    uint64_t blocks = std::min<uint64_t>((nz * 32 + 255) / 256, (uint64_t)sms * 16);
    if (blocks < 1) blocks = 1;
    k_zone_boxes<<<(unsigned)blocks, 256, 0, st>>>(xy, n, zones);
    ++g_kernel_launches;
}

__global__ void k_col_absmax(const uint32_t* __restrict__ col, int typ, uint64_t n, unsigned* __restrict__ out_bits) {
    unsigned m = 0u;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float v = fabsf(agg_value(typ, __ldcs(col + i)));
        if (isfinite(v)) m = max(m, __float_as_uint(v));   // non-negative floats order as their bits
    }
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out_bits, m);
}

void launch_col_absmax(const uint32_t* col, int typ, uint64_t n, unsigned* out_bits, int sms, cudaStream_t st) {
    uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8);
    if (blocks < 1) blocks = 1;
    k_col_absmax<<<(unsigned)blocks, 256, 0, st>>>(col, typ, n, out_bits);
    ++g_kernel_launches;
}

// The bounded wait of the bulk-copy pipeline on its own: an mbarrier that
// nothing arrives on, so the wait can only run out.  Host-side failure
// handling (RJ_E_TIMEOUT, a context that stays usable) is tested with it
// without copies in flight.
__global__ void k_wait_selftest(int* err, uint64_t limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait_ns(&bar, 0u, limit_ns)) atomicOr(err, 1);
    __syncthreads();
}

void launch_wait_selftest(int* err, uint64_t limit_ns, cudaStream_t st) {
    k_wait_selftest<<<1, 32, 0, st>>>(err, limit_ns);
    ++g_kernel_launches;
}

__global__ void k_write_xf(XfArgs a, int n, float4* dst) {
    if ((int)threadIdx.x < n) dst[threadIdx.x] = a.v[threadIdx.x];
}

void launch_write_xf(const XfArgs& a, int n, float4* dst, cudaStream_t st) {
    k_write_xf<<<1, kXfArgs, 0, st>>>(a, n, dst);
    ++g_kernel_launches;
}

void launch_raster_label(const PointArgs& pa, const CanvasXf& cx, const uint16_t* label, int sms,
                         cudaStream_t st) {
    LabelMapper m{cx, label};
    launch_points(pa, m, sms, st);
}

void launch_tier_label_points(const PointArgs& pa, const CanvasXf& cx, const TierArgs& tr, int sms, cudaStream_t st) {
    TierLabelMapper m{cx, tr};
    launch_points(pa, m, sms, st);
}

void launch_tier_splat_points(const PointArgs& pa, const CanvasXf& cx, const TierArgs& tr, int sms, cudaStream_t st) {
    TierSplatMapper m{cx, tr, pa.f.sum_scale};
    PointArgs p2 = pa;
    p2.P = 0;   // no per-polygon histogram: the canvas takes the points
    if (pa.f.aggr) launch_points_t<TierSplatMapper, true, false>(p2, m, sms, st);
    else launch_points_t<TierSplatMapper, false, false>(p2, m, sms, st);
}

}  // namespace rj
