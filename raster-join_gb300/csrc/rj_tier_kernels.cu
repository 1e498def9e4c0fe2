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
// crossings of the row centre lines; a pixel is inside when an odd number of
// crossings lie at or left of it), so every result is identical; the work
// becomes proportional to polygon perimeters and mixed blocks instead of
// polygon areas.
//
// One warp per (tile, polygon, band of 16 rows); bands are aligned to block
// rows.  The work of a band is proportional to the crossings of its rows and
// to the blocks the polygon's outline passes through (plus one entry per full
// block), not to the pixels of its area:
//   * the band's (edge, row) crossing pairs are spread over the lanes, one
//     exact division each;
//   * sweep 1 -- every crossing of a live row toggles one bit of a per-row
//     block bitmap (at the first block whose first pixel lies at or right of
//     it) and, when it falls strictly inside a block, flags that block; a
//     prefix XOR over the bitmap gives each block's coverage at its first
//     pixel, which holds for the whole block row unless the block is flagged.
//     Over the 16 rows: I = blocks covered throughout (full for the polygon),
//     U = blocks the polygon covers somewhere.
//   * the blocks whose pixels matter (labels: U and mixed; reduce: U and not
//     full, or full and mixed -- a mixed block's points are in its pixel slot
//     only) are listed, up to 64 at a time; sweep 2 toggles per-pixel bits of
//     the listed blocks only, and their 16-bit row masks follow from the
//     block's first-pixel coverage and a 16-bit prefix XOR;
//   * the listed blocks' pixel slots are then read or written by the whole
//     warp, eight pixels a lane with vector loads and stores.
#include "rj_device.cuh"
#include "rj_launch.h"
#include "rj_point_map.cuh"

namespace rj {

namespace {

constexpr int kTW = 8;            // warps per block
constexpr int kTBand = 16;        // rows per work item (one block row)
constexpr int kTEdgeCap = 256;    // staged edges per warp
constexpr int kTBW = 16;          // block-bitmap words per row: 512 block columns = 8192 pixels
constexpr int kTList = 64;        // blocks whose pixels one round visits

// Per-warp shared memory.  X, C and M are zero between work items.
struct TierWarp {
    int4 edge[kTEdgeCap];               // staged edges of the band
    uint32_t X[kTBand * kTBW];          // block toggles, then coverage at each block's first pixel
    uint32_t C[kTBand * kTBW];          // blocks with a crossing inside (pixel offsets 1..15)
    uint32_t M[kTList * kTBand / 2];    // listed blocks: pixel toggles, then row masks (two rows a word)
    uint16_t list[kTList];              // listed block columns (relative to bc_lo)
    uint8_t map[kTBW * 32];             // block column -> list index, 0xFF when not listed
};
static_assert(sizeof(TierWarp) % 16 == 0, "TierWarp keeps 16-byte alignment");
constexpr size_t kTierSmem = (size_t)kTW * sizeof(TierWarp);

// bits [a, b) of a word, 0 <= a < b <= 32
__device__ __forceinline__ uint32_t bitrange(int a, int b) {
    return (b >= 32 ? 0xFFFFFFFFu : ((1u << b) - 1u)) & ~((1u << a) - 1u);
}
// inclusive prefix parity: bit k = XOR of bits 0..k
__device__ __forceinline__ uint32_t prefix_xor(uint32_t x) {
    x ^= x << 1;
    x ^= x << 2;
    x ^= x << 4;
    x ^= x << 8;
    x ^= x << 16;
    return x;
}

// Rows [r0, r1] of the band (relative to jb) whose centre line the edge
// with fixed-point ends y = ay, by crosses: ylo < cy <= yhi, cy = j * 256 + 128.
__device__ __forceinline__ void edge_rows(int32_t ay, int32_t by, int jb, int& r0, int& r1) {
    const int64_t ylo = min(ay, by), yhi = max(ay, by);
    const int64_t a0 = ((ylo - kSub / 2) >> kSubpixelBits) + 1 - jb;
    const int64_t a1 = ((yhi - kSub / 2) >> kSubpixelBits) - jb;
    r0 = (int)(a0 < 0 ? 0 : a0);
    r1 = (int)(a1 > kTBand - 1 ? kTBand - 1 : a1);
}

// f(q, r) for every (edge, band row) pair whose row centre line the edge's
// y range spans, spread over the lanes: an edge crossing 16 rows gives 16
// lanes work instead of one lane 16 exact divisions.  Every lane calls this
// (warp-uniform loops); edge(e) returns staged edge e < ne.
template <class E, class F>
__device__ __forceinline__ void for_edge_rows(int ne, int jb, int lane, E&& edge, F&& f) {
    const unsigned FULL = 0xffffffffu;
    for (int e0 = 0; e0 < ne; e0 += 32) {
        const int e = e0 + lane;
        int4 q = make_int4(0, 0, 0, 0);
        int r0 = 0, cnt = 0;
        if (e < ne) {
            q = edge(e);
            int r1;
            edge_rows(q.y, q.w, jb, r0, r1);
            cnt = max(r1 - r0 + 1, 0);
        }
        int incl = cnt;
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(FULL, incl, 31);
        for (int base = 0; base < total; base += 32) {
            const int idx = base + lane;
            int lo = 0, hi = 31;   // the first lane whose inclusive count exceeds idx
            #pragma unroll
            for (int s = 0; s < 5; ++s) {
                const int mid = (lo + hi) >> 1;
                if (__shfl_sync(FULL, incl, mid) > idx) hi = mid; else lo = mid + 1;
            }
            const int4 qe = make_int4(__shfl_sync(FULL, q.x, lo), __shfl_sync(FULL, q.y, lo),
                                      __shfl_sync(FULL, q.z, lo), __shfl_sync(FULL, q.w, lo));
            const int first = __shfl_sync(FULL, r0, lo) + idx - (__shfl_sync(FULL, incl, lo) - __shfl_sync(FULL, cnt, lo));
            if (idx < total) f(qe, first);
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(kTW * 32) k_tier_pass(PolyPassArgs a, TierArgs tr) {
    extern __shared__ int4 s_tier[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int TP = a.T * a.P;
    const int total = a.band_start[TP];
    TierWarp& S = reinterpret_cast<TierWarp*>(s_tier)[warp];
    for (int w = lane; w < kTBand * kTBW; w += 32) {
        S.X[w] = 0u;
        S.C[w] = 0u;
    }
    for (int w = lane; w < kTList * kTBand / 2; w += 32) S.M[w] = 0u;
    __syncwarp();
    const int hw = lane & 15, half = lane >> 4;   // sweep 1: row 2k + half, block word hw
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
        const int jb = ia.z + band * kTBand;            // a multiple of 16
        const int br = jb >> 4;
        const int v0 = __ldg(a.pindex + p);
        const int n = __ldg(a.pindex + p + 1) - v0;
        const int2* pv = a.wv + (size_t)t * a.V + v0;
        const size_t blk0 = (size_t)t * tr.bw * tr.bh + (size_t)br * tr.bw;
        const int bc_lo = i_lo >> 4;
        const int nbc = (i_hi >> 4) - bc_lo + 1;        // block columns of the range (<= 512)
        if (nbc > kTBW * 32) continue;                  // never: resx <= 8192

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
            if (take && pos < kTEdgeCap) S.edge[pos] = e;
            nb += __popc(m);
        }
        const bool overflow = nb > kTEdgeCap;
        const int ne = overflow ? n : nb;
        __syncwarp();
        auto edge_at = [&](int e) -> int4 {
            if (!overflow) return S.edge[e];
            const int2 A = pv[e];
            const int2 B = pv[(e + 1 == n) ? 0 : e + 1];
            return make_int4(A.x, A.y, B.x, B.y);
        };
        if (MODE == MODE_TIER_CLASSIFY && tr.outline) {
            // blocks within two pixels of an edge near this band (rows
            // jb - 2 .. jb + 17) become mixed: the error-bound outline pass
            // reads per-pixel counts up to a pixel beside each edge, rows one
            // beyond the polygon's included
            const float ylo = (float)(jb - 2), yhi = (float)(jb + kTBand + 2);
            for (int e = lane; e < ne; e += 32) {
                const int4 q = edge_at(e);
                const float ax = q.x * (1.0f / kSub), ay = q.y * (1.0f / kSub);
                const float bx = q.z * (1.0f / kSub), by = q.w * (1.0f / kSub);
                const float y0 = fmaxf(fminf(ay, by), ylo), y1 = fminf(fmaxf(ay, by), yhi);
                if (!(y0 <= y1)) continue;
                float x0, x1;
                if (ay == by) {
                    x0 = fminf(ax, bx);
                    x1 = fmaxf(ax, bx);
                } else {
                    const float ta = fminf(fmaxf((y0 - ay) / (by - ay), 0.0f), 1.0f);
                    const float tb = fminf(fmaxf((y1 - ay) / (by - ay), 0.0f), 1.0f);
                    const float xa = ax + (bx - ax) * ta, xb = ax + (bx - ax) * tb;
                    x0 = fminf(xa, xb);
                    x1 = fmaxf(xa, xb);
                }
                const int c0 = max((int)floorf(x0) - 2, 0), c1 = min((int)floorf(x1) + 2, a.resx - 1);
                const int r0 = max((int)floorf(y0) - 2, 0), r1 = min((int)floorf(y1) + 2, a.resy - 1);
                if (c0 > c1 || r0 > r1) continue;
                const size_t tile0 = (size_t)t * tr.bw * tr.bh;
                for (int br2 = r0 >> 4; br2 <= (r1 >> 4); ++br2)
                    for (int bc = c0 >> 4; bc <= (c1 >> 4); ++bc) tr.mixed[tile0 + (size_t)br2 * tr.bw + bc] = 1u;
            }
        }

        __syncwarp();                                   // staged edges read; the next item restages them
        if (nbc <= 0) continue;                         // outline rows only

        // rows of the band inside the polygon's crossing rows and the canvas
        const int rl = max(j_lo, jb) - jb, rh = min(min(j_hi, a.resy - 1), jb + kTBand - 1) - jb;
        const uint32_t live = rl <= rh ? bitrange(rl, rh + 1) : 0u;
        if (!live) continue;

        // sweep 1: block toggles and inside-crossing flags per live row
        for_edge_rows(ne, jb, lane, edge_at, [&](const int4& q, int r) {
            const int32_t cy = (jb + r) * kSub + kSub / 2;
            if (!((live >> r) & 1u) || !cross_row(q.y, q.w, cy)) return;
            const int L = max(cross_L(q.x, q.y, q.z, q.w, cy), i_lo);
            if (L > i_hi) return;
            const int rb = ((L + 15) >> 4) - bc_lo;
            if (rb < nbc) atomicXor(&S.X[r * kTBW + (rb >> 5)], 1u << (rb & 31));
            if (L & 15) {
                const int cb = (L >> 4) - bc_lo;
                atomicOr(&S.C[r * kTBW + (cb >> 5)], 1u << (cb & 31));
            }
        });
        __syncwarp();
        // block columns [fb, lb] lie wholly inside [i_lo, i_hi]; word hw's valid blocks
        const int fb = ((i_lo + 15) >> 4) - bc_lo, lb = ((i_hi + 1) >> 4) - 1 - bc_lo;
        const int wa = max(fb - hw * 32, 0), wb = min(lb - hw * 32 + 1, 32);
        const int va = min(nbc - hw * 32, 32);
        const uint32_t valid = va > 0 ? bitrange(0, va) : 0u;
        uint32_t I = (live == 0xFFFFu && wa < wb) ? bitrange(wa, wb) : 0u, U = 0u;
        #pragma unroll 2
        for (int r2 = 0; r2 < kTBand; r2 += 2) {
            const int r = r2 + half;
            const int idx = r * kTBW + hw;
            const uint32_t tg = S.X[idx], c = S.C[idx];
            uint32_t x = prefix_xor(tg);
            const unsigned odd = __ballot_sync(FULL, (__popc(tg) & 1) != 0);
            if (__popc((odd >> (half * 16)) & ((1u << hw) - 1u)) & 1) x = ~x;
            S.X[idx] = x;
            S.C[idx] = 0u;
            if ((live >> r) & 1u) {
                I &= x & ~c;
                U |= (x | c) & valid;
            }
        }
        I &= __shfl_xor_sync(FULL, I, 16);
        U |= __shfl_xor_sync(FULL, U, 16);
        const int nbw = (nbc + 31) >> 5;

        if (MODE == MODE_TIER_CLASSIFY) {
            // block columns: full for p, or touched (mixed)
            for (int k = 0; k < nbw; ++k) {
                const uint32_t Iw = __shfl_sync(FULL, I, k), Uw = __shfl_sync(FULL, U, k);
                if (!Uw) continue;
                const int rel = k * 32 + lane;
                if (!((Uw >> lane) & 1u)) continue;
                const size_t b = blk0 + bc_lo + rel;
                if ((Iw >> lane) & 1u) {
                    if (atomicCAS(tr.full + b, kTierEmpty, (uint32_t)p) != kTierEmpty) atomicExch(tr.full + b, kTierMulti);
                } else {
                    tr.mixed[b] = 1u;
                }
            }
            for (int w = lane; w < kTBand * kTBW; w += 32) S.X[w] = 0u;
            __syncwarp();
            continue;
        }

        unsigned long long acc_c = 0;
        long long acc_s = 0;
        // listed blocks: reduce -- covered and not full, or full and mixed
        // (a mixed block's points are in its pixel slot only; the other full
        // blocks take their block totals); labels -- covered and mixed
        uint32_t Lw = 0u;   // lane k < nbw: listed blocks of word k
        for (int k = 0; k < nbw; ++k) {
            const uint32_t Iw = __shfl_sync(FULL, I, k), Uw = __shfl_sync(FULL, U, k);
            if (!Uw) continue;
            const int rel = k * 32 + lane;
            const size_t b = blk0 + bc_lo + rel;
            bool take = false;
            if (MODE == MODE_TIER_REDUCE) {
                if ((Iw >> lane) & 1u) {
                    if (__ldg(tr.mixed + b) != 0u) {
                        take = true;
                    } else {
                        acc_c += __ldg(tr.bcnt + b);
                        if (tr.bsum) acc_s += __ldg(tr.bsum + b);
                    }
                } else {
                    take = (Uw >> lane) & 1u;
                }
            } else {
                take = ((Uw >> lane) & 1u) && __ldg(tr.mixed + b) != 0u;
            }
            const uint32_t m = __ballot_sync(FULL, take);
            if (lane == k) Lw = m;
        }
        // list positions: exclusive prefix of the words' counts
        const int cnt = lane < nbw ? __popc(Lw) : 0;
        int pre = cnt;
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(FULL, pre, o);
            if (lane >= o) pre += v;
        }
        const int nlist = __shfl_sync(FULL, pre, 31);
        pre -= cnt;
        for (int start = 0; start < nlist; start += kTList) {
            const int nk = min(kTList, nlist - start);
            for (int w = lane; w < kTBW * 32 / 4; w += 32) reinterpret_cast<uint32_t*>(S.map)[w] = 0xFFFFFFFFu;
            __syncwarp();
            if (lane < nbw && pre < start + nk && pre + cnt > start) {
                uint32_t m = Lw;
                int g = pre;
                while (m && g < start + nk) {
                    const int bit = __ffs(m) - 1;
                    m &= m - 1u;
                    if (g >= start) {
                        S.map[lane * 32 + bit] = (uint8_t)(g - start);
                        S.list[g - start] = (uint16_t)(lane * 32 + bit);
                    }
                    ++g;
                }
            }
            __syncwarp();
            // sweep 2: pixel toggles of the listed blocks (crossings inside a
            // block only; one at a block's first pixel is in X already)
            for_edge_rows(ne, jb, lane, edge_at, [&](const int4& q, int r) {
                const int32_t cy = (jb + r) * kSub + kSub / 2;
                if (!((live >> r) & 1u) || !cross_row(q.y, q.w, cy)) return;
                const int L = max(cross_L(q.x, q.y, q.z, q.w, cy), i_lo);
                if (L > i_hi || !(L & 15)) return;
                const int k = S.map[(L >> 4) - bc_lo];
                if (k != 0xFF) atomicXor(&S.M[k * 8 + (r >> 1)], (1u << (L & 15)) << ((r & 1) * 16));
            });
            __syncwarp();
            // row masks: coverage at the block's first pixel, then the block's
            // own crossings, clipped to [i_lo, i_hi]
            for (int w = lane; w < nk * 8; w += 32) {
                const int k = w >> 3, rp = (w & 7) * 2;
                const int rel = S.list[k];
                const int x0 = (bc_lo + rel) * 16;
                const int ka = max(i_lo - x0, 0), kb = min(i_hi - x0, 15);
                const uint32_t rng = bitrange(ka, kb + 1);
                const uint32_t tg = S.M[w];
                uint32_t out = 0u;
                #pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int r = rp + h;
                    if (!((live >> r) & 1u)) continue;
                    uint32_t x = prefix_xor((tg >> (h * 16)) & 0xFFFFu) & 0xFFFFu;
                    if ((S.X[r * kTBW + (rel >> 5)] >> (rel & 31)) & 1u) x ^= 0xFFFFu;
                    out |= (x & rng) << (h * 16);
                }
                S.M[w] = out;
            }
            __syncwarp();
            // the listed blocks' pixels: lane = (row, half row of 8 pixels)
            const int pr = lane >> 1, ph = (lane & 1) * 8;
            #pragma unroll 4
            for (int k = 0; k < nk; ++k) {
                const uint32_t m8 = (S.M[k * 8 + (pr >> 1)] >> ((pr & 1) * 16 + ph)) & 0xFFu;
                if (!m8) continue;
                const size_t b = blk0 + bc_lo + S.list[k];
                const size_t q = (size_t)__ldg(tr.slot + b) * 256 + (size_t)pr * 16 + ph;
                if (MODE == MODE_TIER_LABEL) {
                    uint16_t* dst = tr.plabel + q;
                    if (m8 == 0xFFu) {
                        const uint32_t pp = (uint32_t)p | ((uint32_t)p << 16);
                        *reinterpret_cast<uint4*>(dst) = make_uint4(pp, pp, pp, pp);
                    } else {
                        #pragma unroll
                        for (int i = 0; i < 8; ++i)
                            if ((m8 >> i) & 1u) dst[i] = (uint16_t)p;
                    }
                    acc_c += (unsigned)__popc(m8);
                } else {
                    const uint4 c0 = __ldg(reinterpret_cast<const uint4*>(tr.pcnt + q));
                    const uint4 c1 = __ldg(reinterpret_cast<const uint4*>(tr.pcnt + q + 4));
                    acc_c += (unsigned long long)((m8 & 1u) ? c0.x : 0u) + ((m8 & 2u) ? c0.y : 0u) +
                             ((m8 & 4u) ? c0.z : 0u) + ((m8 & 8u) ? c0.w : 0u) + ((m8 & 16u) ? c1.x : 0u) +
                             ((m8 & 32u) ? c1.y : 0u) + ((m8 & 64u) ? c1.z : 0u) + ((m8 & 128u) ? c1.w : 0u);
                    if (tr.psum) {
                        const longlong2* ps = reinterpret_cast<const longlong2*>(tr.psum + q);
                        #pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const longlong2 v = __ldg(ps + i);
                            if ((m8 >> (2 * i)) & 1u) acc_s += v.x;
                            if ((m8 >> (2 * i + 1)) & 1u) acc_s += v.y;
                        }
                    }
                }
            }
            __syncwarp();   // every lane has read its masks
            for (int w = lane; w < nk * 8; w += 32) S.M[w] = 0u;
            __syncwarp();
        }
        for (int w = lane; w < kTBand * kTBW; w += 32) S.X[w] = 0u;
        __syncwarp();
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
