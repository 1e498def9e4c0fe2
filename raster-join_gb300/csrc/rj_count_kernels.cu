// rj_count_kernels.cu -- lean point pass of the raster join for the common
// case of the benchmark and of the reference's own experiments: a plain
// count over one canvas tile whose polygons do not overlap (the label form),
// with no attribute filter.
//
// The reference renders every point into an fp32 framebuffer and then every
// polygon's triangles over it (RasterJoin.cpp:91-194, points.vert:138-159,
// polygon.frag:12-27).  With a per-pixel polygon label the polygon pass
// disappears: a point's polygon is the label of its pixel.  What limits that
// pass on GB300 is not DRAM but the per-point work around the label lookup:
//   * the label gather: one random 32-byte L2 sector per point (the 16-bit
//     label map of a 4000 x 4000 canvas is 32 MB); at one request per point
//     the L2 request rate, not HBM, bounds the pass;
//   * the per-polygon histogram: warp grouping with __match_any_sync runs on
//     a narrow pipe and saturates it long before HBM does.
// This kernel therefore
//   * keeps a block-code map of the canvas in shared memory: per block of
//     2^bs x 2^bs pixels the label every pixel of the block shares, or
//     kCodeMixed when an edge passes through it.  Only points in mixed
//     blocks read the label map in L2 (about 15 % of the points at 16 x 16
//     blocks for 260 Voronoi cells at 10 m);
//   * counts with plain shared-memory atomic increments (no warp grouping),
//     optionally into one histogram copy per warp;
//   * streams the location column with fully coalesced 128-bit evict-first
//     loads (each lane two points per load), several loads in flight per
//     thread before the first is used.
// The pixel of a point is the generic pass's (per-tile MVP in fp32, snap to
// 1/256 px, floor), computed with two exact rewrites that save operations
// (rj_lean.cuh), so the counts are identical.
#include "rj_lean.cuh"

namespace rj {

// Block codes from a label map: one warp per block.
__global__ void k_block_codes(const uint16_t* __restrict__ label, int resx, int resy, int bs, int nbx, int nby,
                              uint16_t* __restrict__ codes) {
    const int lane = threadIdx.x & 31;
    const int B = 1 << bs;
    const int nb = nbx * nby;
    for (int b = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); b < nb;
         b += (int)((gridDim.x * blockDim.x) >> 5)) {
        const int bx = b % nbx, by = b / nbx;
        const int x0 = bx << bs, y0 = by << bs;
        const int w = min(x0 + B, resx) - x0, h = min(y0 + B, resy) - y0;
        const uint16_t first = __ldg(label + (size_t)y0 * resx + x0);
        bool same = true;
        for (int i = lane; i < w * h; i += 32) {
            const int yy = y0 + i / w, xx = x0 + i % w;
            same &= (__ldg(label + (size_t)yy * resx + xx) == first);
        }
        same = __all_sync(0xffffffffu, same);
        if (lane == 0) codes[b] = same ? first : kCodeMixed;
    }
}

void launch_block_codes(const uint16_t* label, int resx, int resy, int bs, int nbx, int nby, uint16_t* codes,
                        int sms, cudaStream_t st) {
    const long long warps = (long long)nbx * nby;
    long long blocks = (warps * 32 + 255) / 256;
    blocks = std::max(1LL, std::min(blocks, (long long)sms * 16));
    k_block_codes<<<(unsigned)blocks, 256, 0, st>>>(label, resx, resy, bs, nbx, nby, codes);
    ++g_kernel_launches;
}

template <int BLOCK, int NV, bool CODES, bool WARP_HIST>
__global__ void __launch_bounds__(BLOCK) k_label_count(LabelCountArgs a) {
    extern __shared__ uint32_t s_words[];
    uint32_t* s_code = s_words;                                  // a.code_words (CODES)
    uint32_t* s_hist = s_words + (CODES ? a.code_words : 0);     // P per copy
    constexpr int kCopies = WARP_HIST ? BLOCK / 32 : 1;
    if (CODES) {
        const uint32_t* g = reinterpret_cast<const uint32_t*>(a.codes);
        for (int i = threadIdx.x; i < a.code_words; i += BLOCK) s_code[i] = __ldg(g + i);
    }
    for (int i = threadIdx.x; i < a.P * kCopies; i += BLOCK) s_hist[i] = 0u;
    __syncthreads();
    const uint16_t* sc = reinterpret_cast<const uint16_t*>(s_code);
    uint32_t* hist = s_hist + (WARP_HIST ? (threadIdx.x >> 5) * a.P : 0);
    const uint32_t P = (uint32_t)a.P;
    const TileXf2 xf = tile_xf2(a);

    const uint64_t npairs = a.n >> 1;
    constexpr uint64_t kPerIter = (uint64_t)BLOCK * NV;
    const uint64_t warp_ofs = (uint64_t)(threadIdx.x >> 5) * 32 * NV;
    const uint64_t lane_ofs = warp_ofs + (threadIdx.x & 31);
    // block-uniform trip count; no barrier inside, so a warp may skip an iteration
    for (uint64_t base = (uint64_t)blockIdx.x * kPerIter; base < npairs; base += (uint64_t)gridDim.x * kPerIter) {
        if (a.zones) {
            // the warp's 64*NV rows lie in at most two zones of 1024 rows:
            // skip them when no zone's bounds reach the canvas
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
        #pragma unroll
        for (int k = 0; k < NV; ++k) {
            const uint64_t i = base + lane_ofs + (uint64_t)k * 32;
            p[k] = (i < npairs) ? __ldcs(a.xy + i) : make_float4(NAN, NAN, NAN, NAN);
        }
        uint32_t lab[2 * NV];
        #pragma unroll
        for (int k = 0; k < 2 * NV; ++k) {
            const float x = (k & 1) ? p[k >> 1].z : p[k >> 1].x;
            const float y = (k & 1) ? p[k >> 1].w : p[k >> 1].y;
            int px, py;
            const bool in = count_pixel(a, xf, x, y, px, py);
            px = in ? px : 0;
            py = in ? py : 0;
            uint32_t c;
            if (CODES) {
                c = in ? (uint32_t)sc[(py >> a.bs) * a.nbx + (px >> a.bs)] : (uint32_t)kEmptyLabel;
                if (c == kCodeMixed) c = __ldg(a.label + (size_t)py * a.resx + px);
            } else {
                c = in ? (uint32_t)__ldg(a.label + (size_t)py * a.resx + px) : (uint32_t)kEmptyLabel;
            }
            lab[k] = c;
        }
        #pragma unroll
        for (int k = 0; k < 2 * NV; ++k)
            if (lab[k] < P) atomicAdd(hist + lab[k], 1u);
    }
    // the last point of an odd-sized table
    if ((a.n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const float2 q = __ldg(reinterpret_cast<const float2*>(a.xy) + (a.n - 1));
        int px, py;
        if (count_pixel(a, xf, q.x, q.y, px, py)) {
            const uint32_t c = __ldg(a.label + (size_t)py * a.resx + px);
            if (c < P) atomicAdd(hist + c, 1u);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < a.P; b += BLOCK) {
        uint32_t c = 0;
        #pragma unroll 1
        for (int w = 0; w < kCopies; ++w) c += s_hist[w * a.P + b];
        if (c) atomicAdd(a.out_count + b, (unsigned long long)c);
    }
}

// ---------------------------------------------------------------------------
// Shapes.  Every shape computes the same counts; the autotuner of the host
// runtime times them on the query at hand and keeps the fastest.
namespace {

struct CountShape {
    void (*kernel)(LabelCountArgs);
    int block;
    bool codes;
    bool warp_hist;
};

template <int BLOCK, int NV, bool CODES, bool WH>
constexpr CountShape shape() {
    return CountShape{k_label_count<BLOCK, NV, CODES, WH>, BLOCK, CODES, WH};
}

const CountShape kShapes[] = {
    shape<512, 4, true, false>(),  shape<512, 4, true, true>(),   shape<1024, 4, true, false>(),
    shape<1024, 2, true, false>(), shape<512, 8, true, false>(),  shape<1024, 4, true, true>(),
    shape<512, 4, false, false>(), shape<256, 4, true, false>(),  shape<1024, 8, true, true>(),
    shape<512, 8, true, true>(),   shape<1024, 2, true, true>(),
};
constexpr int kNumShapes = (int)(sizeof(kShapes) / sizeof(kShapes[0]));

int g_optin = -1;

}  // namespace

int label_count_shapes() { return kNumShapes; }

size_t label_count_smem(int shape, int code_words, int P) {
    if (shape < 0 || shape >= kNumShapes) return 0;
    const CountShape& s = kShapes[shape];
    const size_t copies = s.warp_hist ? (size_t)s.block / 32 : 1;
    return (s.codes ? (size_t)code_words * 4 : 0) + (size_t)P * copies * 4;
}

// false: the shape cannot run this query (shared memory); nothing launched
bool launch_label_count(int shape, const LabelCountArgs& a, int sms, cudaStream_t st) {
    if (shape < 0 || shape >= kNumShapes) return false;
    const CountShape& s = kShapes[shape];
    if (g_optin < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    }
    const size_t smem = label_count_smem(shape, a.code_words, a.P);
    if (smem > (size_t)g_optin) return false;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(s.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, s.kernel, s.block, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        return false;
    }
    const uint64_t per_iter = (uint64_t)s.block * 4;   // pairs per block iteration (lower bound over shapes)
    uint64_t need = ((a.n >> 1) + per_iter - 1) / per_iter;
    uint64_t blocks = std::min<uint64_t>((uint64_t)sms * per_sm, std::max<uint64_t>(need, 1));
    // shared counts are 32-bit: a block must see fewer than 2^32 points
    while (blocks < (uint64_t)sms * per_sm && a.n / blocks >= (1ull << 31)) ++blocks;
    if (a.n / blocks >= (1ull << 31)) return false;
    s.kernel<<<(unsigned)blocks, s.block, smem, st>>>(a);
    ++g_kernel_launches;
    return true;
}

}  // namespace rj
