// rj_tier_kernels.cu -- tiered canvas for fine resolutions.
//
// A raster canvas of 10^8-10^9 pixels is mostly the interiors of polygons.
// The tiered canvas keeps it as 16 x 16-pixel blocks:
//   * a block every pixel centre of which lies inside one polygon ("full")
//     is one entry: the polygon id (label form) or one count / sum (canvas
//     form);
//   * a block no polygon reaches is empty;
//   * only "mixed" blocks (crossed by an edge, or full for one polygon and
//     touched by another) keep per-pixel data, in a compact slot of 256
//     pixels.
// Coverage is the same pixel-centre rule as the flat canvas (exact integer
// crossings of the row centre lines, spans between sorted crossings), so
// every result is identical; the work becomes proportional to polygon
// perimeters and mixed blocks instead of polygon areas.
//
// One warp per (tile, polygon, band of 16 rows); bands are aligned to block
// rows.  Per band the warp builds two pixel bitmaps over the polygon's
// column range: I = pixels covered on all 16 rows, U = pixels covered on any
// row.  A block column with all 16 bits of I set is full for the polygon;
// one with bits of U set but not full is mixed.
#include "rj_device.cuh"
#include "rj_launch.h"
#include "rj_point_map.cuh"

namespace rj {

namespace {

constexpr int kTW = 8;            // warps per block
constexpr int kTBand = 16;        // rows per work item (one block row)
constexpr int kTEdgeCap = 256;    // staged edges per warp
constexpr int kTCrossCap = 512;   // crossings per row per warp
constexpr int kTWords = 256;      // bitmap words per warp: 8192 pixel columns
constexpr size_t kTierSmem =
    (size_t)kTW * (kTEdgeCap * sizeof(int4) + kTCrossCap * sizeof(int) + 2 * kTWords * sizeof(uint32_t));

__device__ __forceinline__ int x1_of(int x0) { return x0 + 32; }
// bits [a, b) of a word, 0 <= a < b <= 32
__device__ __forceinline__ uint32_t bitrange(int a, int b) {
    return (b >= 32 ? 0xFFFFFFFFu : ((1u << b) - 1u)) & ~((1u << a) - 1u);
}

__device__ __forceinline__ void tsort(int* buf, int m, int lane) {
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

// Sorted crossings of row j's centre line into cross[0, m); returns m, or -1
// when the row has more crossings than the buffer holds.
__device__ __forceinline__ int row_crossings(int j, const int4* edge, int nb, bool overflow, const int2* pv, int n,
                                             int* cross, int lane) {
    const int32_t cy = j * kSub + kSub / 2;
    int m = 0;
    const int ne = overflow ? n : nb;
    for (int e0 = 0; e0 < ne; e0 += 32) {
        const int e = e0 + lane;
        bool c = false;
        int L = 0;
        if (e < ne) {
            int4 q;
            if (!overflow) {
                q = edge[e];
            } else {
                const int2 A = pv[e];
                const int2 B = pv[(e + 1 == n) ? 0 : e + 1];
                q = make_int4(A.x, A.y, B.x, B.y);
            }
            if (cross_row(q.y, q.w, cy)) { c = true; L = cross_L(q.x, q.y, q.z, q.w, cy); }
        }
        const unsigned bm = __ballot_sync(0xffffffffu, c);
        const int pos = m + __popc(bm & ((1u << lane) - 1u));
        if (c && pos < kTCrossCap) cross[pos] = L;
        m += __popc(bm);
    }
    __syncwarp();
    if (m > kTCrossCap) return -1;
    if (m > 1) tsort(cross, m, lane);
    return m;
}

// Row crossings by all edges of the polygon, one pixel at a time (a row with
// more crossings than the buffer: pathological polygons only).
__device__ __forceinline__ bool pixel_inside(const int2* pv, int n, int i, int j) {
    const int32_t cy = j * kSub + kSub / 2;
    bool inside = false;
    for (int k = 0; k < n; ++k) {
        const int2 A = pv[k];
        const int2 B = pv[(k + 1 == n) ? 0 : k + 1];
        if (cross_row(A.y, B.y, cy)) inside ^= (i < cross_L(A.x, A.y, B.x, B.y, cy));
    }
    return inside;
}

template <int MODE>
__global__ void __launch_bounds__(kTW * 32) k_tier_pass(PolyPassArgs a, TierArgs tr) {
    extern __shared__ int4 s_tier[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int TP = a.T * a.P;
    const int total = a.band_start[TP];
    int4* my_edge = s_tier + (size_t)warp * kTEdgeCap;
    int* my_cross = reinterpret_cast<int*>(s_tier + (size_t)kTW * kTEdgeCap) + (size_t)warp * kTCrossCap;
    uint32_t* my_I = reinterpret_cast<uint32_t*>(reinterpret_cast<int*>(s_tier + (size_t)kTW * kTEdgeCap) +
                                                 (size_t)kTW * kTCrossCap) + (size_t)warp * 2 * kTWords;
    uint32_t* my_U = my_I + kTWords;
    for (;;) {
        int item = 0, tp = 0;
        if (lane == 0) {
            item = (int)atomicAdd(a.work_ctr, 1u);
            if (item < total) {
                int lo = 0, hi = TP - 1;
                while (lo < hi) {
                    int mid = (lo + hi + 1) >> 1;
                    if (a.band_start[mid] <= item) lo = mid; else hi = mid - 1;
                }
                tp = lo;
            }
        }
        item = __shfl_sync(FULL, item, 0);
        tp = __shfl_sync(FULL, tp, 0);
        if (item >= total) break;
        const int t = tp / a.P, p = tp - t * a.P;
        const int band = item - a.band_start[tp];
        const int4 ia = a.info_a[tp];
        const int2 ib = a.info_b[tp];
        const int i_lo = ia.x, i_hi = ia.y, j_lo = ib.x, j_hi = ib.y;
        const int jb = ia.z + band * kTBand;            // a multiple of 16
        const int br = jb >> 4;
        const int v0 = __ldg(a.pindex + p);
        const int n = __ldg(a.pindex + p + 1) - v0;
        const int2* pv = a.wv + (size_t)t * a.V + v0;
        const size_t blk0 = (size_t)t * tr.bw * tr.bh + (size_t)br * tr.bw;
        const int w_lo = i_lo >> 5, w_hi = i_hi >> 5;
        if (w_hi - w_lo >= kTWords) continue;            // never: resx <= 8192

        // stage the edges that can cross a row centre of the band
        const int64_t band_lo = (int64_t)jb * kSub - kSub;
        const int64_t band_hi = (int64_t)(jb + kTBand) * kSub + kSub;
        int nb = 0;
        for (int k0 = 0; k0 < n; k0 += 32) {
            const int k = k0 + lane;
            bool take = false;
            int4 e = make_int4(0, 0, 0, 0);
            if (k < n) {
                const int2 A = pv[k];
                const int2 B = pv[(k + 1 == n) ? 0 : k + 1];
                const int lo = min(A.y, B.y), hi = max(A.y, B.y);
                take = (hi >= band_lo) && (lo <= band_hi);
                e = make_int4(A.x, A.y, B.x, B.y);
            }
            const unsigned m = __ballot_sync(FULL, take);
            const int pos = nb + __popc(m & ((1u << lane) - 1u));
            if (take && pos < kTEdgeCap) my_edge[pos] = e;
            nb += __popc(m);
        }
        const bool overflow = nb > kTEdgeCap;
        __syncwarp();

        // I: pixels covered on every row of the block row; U: on some row
        const bool rows_ok = jb + kTBand - 1 <= a.resy - 1;
        for (int w = w_lo + lane; w <= w_hi; w += 32) {
            const int x0 = w * 32;
            const int a0 = max(i_lo - x0, 0), b0 = min(i_hi + 1 - x0, 32);
            my_I[w - w_lo] = (rows_ok && a0 < b0) ? ((b0 >= 32 ? 0xFFFFFFFFu : ((1u << b0) - 1u)) & ~((1u << a0) - 1u)) : 0u;
            if (MODE == MODE_TIER_CLASSIFY) my_U[w - w_lo] = 0u;
        }
        __syncwarp();
        bool slow = false;
        for (int r = 0; r < kTBand && MODE != MODE_TIER_LABEL; ++r) {
            const int j = jb + r;
            const bool live = j <= a.resy - 1 && j >= j_lo && j <= j_hi;
            int m = live ? row_crossings(j, my_edge, nb, overflow, pv, n, my_cross, lane) : 0;
            if (m < 0) {
                slow = true;
                m = 0;
            }
            if (MODE == MODE_TIER_CLASSIFY) {
                for (int w = w_lo + lane; w <= w_hi; w += 32) {
                    const int x0 = w * 32;
                    uint32_t v = 0u;
                    for (int s = 0; s + 1 < m; s += 2) {
                        const int L = max(max(my_cross[s], i_lo), x0), R = min(min(my_cross[s + 1], i_hi + 1), x1_of(x0));
                        if (L < R) v |= bitrange(L - x0, R - x0);
                    }
                    if (slow && live) {
                        // pathological row: every pixel of the word by the full test
                        v = 0u;
                        for (int b = 0; b < 32; ++b) {
                            const int i = x0 + b;
                            if (i >= i_lo && i <= i_hi && pixel_inside(pv, n, i, j)) v |= 1u << b;
                        }
                    }
                    my_I[w - w_lo] &= v;
                    my_U[w - w_lo] |= v;
                }
                slow = false;
                __syncwarp();
            } else if (MODE == MODE_TIER_REDUCE) {
                // full blocks are counted once below; pixels of the others
                // (mixed blocks) are visited along the row's spans
                if (!live) {
                    for (int w = w_lo + lane; w <= w_hi; w += 32) my_I[w - w_lo] = 0u;
                    __syncwarp();
                    continue;
                }
                // I over the band must be complete before the pixel visits, so the
                // canvas modes make two sweeps: this one narrows I ...
                for (int w = w_lo + lane; w <= w_hi; w += 32) {
                    const int x0 = w * 32;
                    uint32_t v = 0u;
                    if (!slow) {
                        for (int s = 0; s + 1 < m; s += 2) {
                            const int L = max(max(my_cross[s], i_lo), x0), R = min(min(my_cross[s + 1], i_hi + 1), x1_of(x0));
                            if (L < R) v |= bitrange(L - x0, R - x0);
                        }
                    } else {
                        for (int b = 0; b < 32; ++b) {
                            const int i = x0 + b;
                            if (i >= i_lo && i <= i_hi && pixel_inside(pv, n, i, j)) v |= 1u << b;
                        }
                    }
                    my_I[w - w_lo] &= v;
                }
                slow = false;
                __syncwarp();
            }
        }
        if (MODE == MODE_TIER_CLASSIFY) {
            // block columns: full for p, or touched (mixed)
            const int bc_lo = i_lo >> 4, bc_hi = i_hi >> 4;
            for (int bc = bc_lo + lane; bc <= bc_hi; bc += 32) {
                const int w = (bc >> 1) - w_lo;
                const int sh = (bc & 1) * 16;
                const uint32_t iv = (my_I[w] >> sh) & 0xFFFFu, uv = (my_U[w] >> sh) & 0xFFFFu;
                const size_t b = blk0 + bc;
                if (iv == 0xFFFFu) {
                    if (atomicCAS(tr.full + b, kTierEmpty, (uint32_t)p) != kTierEmpty) atomicExch(tr.full + b, kTierMulti);
                } else if (uv) {
                    tr.mixed[b] = 1u;
                }
            }
            continue;
        }

        // ---- canvas modes: second sweep over the rows
        unsigned long long acc_c = 0;
        long long acc_s = 0;
        if (MODE == MODE_TIER_REDUCE) {
            // full blocks of p: one block sum each
            const int bc_lo = i_lo >> 4, bc_hi = i_hi >> 4;
            for (int bc = bc_lo + lane; bc <= bc_hi; bc += 32) {
                const int w = (bc >> 1) - w_lo;
                if (((my_I[w] >> ((bc & 1) * 16)) & 0xFFFFu) == 0xFFFFu) {
                    acc_c += __ldg(tr.bcnt + blk0 + bc);
                    if (tr.bsum) acc_s += __ldg(tr.bsum + blk0 + bc);
                }
            }
        }
        for (int r = 0; r < kTBand; ++r) {
            const int j = jb + r;
            if (!(j <= a.resy - 1 && j >= j_lo && j <= j_hi)) continue;
            const int m = row_crossings(j, my_edge, nb, overflow, pv, n, my_cross, lane);
            // block columns of the row's spans that are not full for p
            auto visit_block = [&](int bc, int L, int R) {
                // pixels [L, R) of block column bc on row j (mixed block)
                const size_t b = blk0 + bc;
                const int sl = __ldg(tr.slot + b);
                const size_t base = (size_t)sl * 256 + (size_t)(j & 15) * 16;
                for (int i = L; i < R; ++i) {
                    const size_t q = base + (i & 15);
                    if (MODE == MODE_TIER_LABEL) {
                        tr.plabel[q] = (uint16_t)p;
                        ++acc_c;
                    } else {
                        acc_c += __ldg(tr.pcnt + q);
                        if (tr.psum) acc_s += __ldg(tr.psum + q);
                    }
                }
            };
            if (m >= 0) {
                for (int s = 0; s + 1 < m; s += 2) {
                    const int L = max(my_cross[s], i_lo), R = min(my_cross[s + 1], i_hi + 1);
                    if (L >= R) continue;
                    for (int bc = (L >> 4) + lane; bc <= ((R - 1) >> 4); bc += 32) {
                        const int w = (bc >> 1) - w_lo;
                        const bool full = ((my_I[w] >> ((bc & 1) * 16)) & 0xFFFFu) == 0xFFFFu;
                        if (full && MODE == MODE_TIER_REDUCE) continue;
                        if (MODE == MODE_TIER_LABEL && !__ldg(tr.mixed + blk0 + bc)) continue;
                        visit_block(bc, max(L, bc * 16), min(R, bc * 16 + 16));
                    }
                }
            } else {
                for (int bc = (i_lo >> 4) + lane; bc <= (i_hi >> 4); bc += 32) {
                    const int w = (bc >> 1) - w_lo;
                    const bool full = ((my_I[w] >> ((bc & 1) * 16)) & 0xFFFFu) == 0xFFFFu;
                    if (full && MODE == MODE_TIER_REDUCE) continue;
                    if (MODE == MODE_TIER_LABEL && !__ldg(tr.mixed + blk0 + bc)) continue;
                    for (int i = max(bc * 16, i_lo); i < min(bc * 16 + 16, i_hi + 1); ++i)
                        if (pixel_inside(pv, n, i, j)) visit_block(bc, i, i + 1);
                }
            }
            __syncwarp();
        }
        acc_c = warp_sum_u64(acc_c);
        if (MODE == MODE_TIER_LABEL) {
            if (lane == 0 && acc_c) atomicAdd(a.covered, acc_c);
        } else {
            if (tr.bsum || tr.psum) acc_s = (long long)warp_sum_u64((unsigned long long)acc_s);
            if (lane == 0 && acc_c) atomicAdd(a.out_count + p, acc_c);
            if (lane == 0 && acc_s != 0) atomicAdd(a.out_sum + p, (unsigned long long)acc_s);
        }
    }
}

// code[b]: kTierMixed | slot for mixed blocks, else the full polygon (or
// empty / multi); counts the multi blocks (two polygons cover them whole).
__global__ void k_tier_codes(TierArgs tr, size_t nblk, unsigned long long* multi) {
    unsigned long long c = 0;
    for (size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x; b < nblk; b += (size_t)gridDim.x * blockDim.x) {
        const uint32_t f = tr.full[b];
        uint32_t code;
        if (tr.mixed[b]) code = kTierMixed | (uint32_t)tr.slot[b];
        else code = f;
        c += (f == kTierMulti);
        tr.code[b] = code;
    }
    c = warp_sum_u64(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(multi, c);
}

// labelled pixels of the mixed blocks (overlap check: equals the pixel writes
// when no two polygons share a pixel centre)
__global__ void k_tier_nonempty(const uint16_t* __restrict__ plabel, size_t n, unsigned long long* count) {
    unsigned long long c = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        c += plabel[i] != kEmptyLabel;
    c = warp_sum_u64(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

}  // namespace

size_t tier_smem_bytes() { return kTierSmem; }

void launch_tier_pass(int mode, const PolyPassArgs& a, const TierArgs& tr, int sms, cudaStream_t st) {
    ++g_kernel_launches;
    auto go = [&](auto kernel) {
        // every instance needs the opt-in (the three kernels share one pointer type)
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTierSmem);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTW * 32, kTierSmem);
        kernel<<<sms * std::max(per_sm, 1), kTW * 32, kTierSmem, st>>>(a, tr);
    };
    switch (mode) {
        case MODE_TIER_CLASSIFY: go(k_tier_pass<MODE_TIER_CLASSIFY>); break;
        case MODE_TIER_LABEL: go(k_tier_pass<MODE_TIER_LABEL>); break;
        default: go(k_tier_pass<MODE_TIER_REDUCE>); break;
    }
}

void launch_tier_codes(const TierArgs& tr, size_t nblk, unsigned long long* multi, int sms, cudaStream_t st) {
    const int blocks = (int)std::min<size_t>((nblk + 255) / 256, (size_t)sms * 16);
    k_tier_codes<<<std::max(blocks, 1), 256, 0, st>>>(tr, nblk, multi);
    ++g_kernel_launches;
}

void launch_tier_nonempty(const uint16_t* plabel, size_t n, unsigned long long* count, int sms, cudaStream_t st) {
    const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)sms * 16);
    k_tier_nonempty<<<std::max(blocks, 1), 256, 0, st>>>(plabel, n, count);
    ++g_kernel_launches;
}

}  // namespace rj
