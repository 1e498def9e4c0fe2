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
constexpr int kTWords = 256;      // bitmap words per warp: 8192 pixel columns
constexpr size_t kTierSmem = (size_t)kTW * (kTEdgeCap * sizeof(int4) + 3 * kTWords * sizeof(uint32_t));

// bits [a, b) of a word, 0 <= a < b <= 32
__device__ __forceinline__ uint32_t bitrange(int a, int b) {
    return (b >= 32 ? 0xFFFFFFFFu : ((1u << b) - 1u)) & ~((1u << a) - 1u);
}

// Coverage of row j's pixel centres in [i_lo, i_hi], word by word: f(w, bits)
// receives word w of the row (bit b = pixel (w_lo + w) * 32 + b), called by
// lane w % 32.  A pixel is covered when an odd number of the row's crossings
// lie at or left of it (crossing pixel L = first pixel right of the crossing,
// exact integer arithmetic), so each crossing toggles one bit of R and a
// prefix XOR over the row gives the coverage: no sorting, O(crossings + words)
// per row.  Crossings left of i_lo act from i_lo; those right of i_hi do not
// matter.  R[0, nw) must be zero on entry and is zero again on return (the
// scan clears what the toggles set), so consecutive rows need no clearing.
// The words of the row's column range as a mask (bits outside [i_lo, i_hi]
// cleared): word w's mask.
__device__ __forceinline__ uint32_t range_mask(int w, int w_lo, int i_lo, int i_hi) {
    const int x0 = (w_lo + w) * 32;
    const int a0 = max(i_lo - x0, 0), b0 = min(i_hi + 1 - x0, 32);
    return a0 < b0 ? bitrange(a0, b0) : 0u;
}

// fu(w0, carry) takes a whole chunk of 32 words (w0 .. w0 + 31) that no
// crossing of the row touches: every pixel of it has the coverage `carry`.
// It is called by every lane (warp-uniform).
template <class F, class FU>
__device__ __forceinline__ void row_cover(int j, const int4* edge, int nb, bool overflow, const int2* pv, int n,
                                          int i_lo, int i_hi, int w_lo, int nw, uint32_t* R, int lane, F&& f,
                                          FU&& fu) {
    const int32_t cy = j * kSub + kSub / 2;
    const int ne = overflow ? n : nb;
    for (int e = lane; e < ne; e += 32) {
        int4 q;
        if (!overflow) {
            q = edge[e];
        } else {
            const int2 A = pv[e];
            const int2 B = pv[(e + 1 == n) ? 0 : e + 1];
            q = make_int4(A.x, A.y, B.x, B.y);
        }
        if (cross_row(q.y, q.w, cy)) {
            const int L = max(cross_L(q.x, q.y, q.z, q.w, cy), i_lo);
            if (L <= i_hi) atomicXor(R + ((L >> 5) - w_lo), 1u << (L & 31));
        }
    }
    __syncwarp();
    uint32_t carry = 0u;   // parity of the toggles in the words before this chunk
    for (int w0 = 0; w0 < nw; w0 += 32) {
        const int w = w0 + lane;
        const uint32_t t = w < nw ? R[w] : 0u;
        if (__ballot_sync(0xffffffffu, t != 0u) == 0u) {
            fu(w0, carry);
            continue;
        }
        const unsigned odd = __ballot_sync(0xffffffffu, (__popc(t) & 1) != 0);
        uint32_t x = t;   // inclusive prefix parity inside the word
        x ^= x << 1;
        x ^= x << 2;
        x ^= x << 4;
        x ^= x << 8;
        x ^= x << 16;
        if (((unsigned)__popc(odd & ((1u << lane) - 1u)) & 1u) ^ carry) x = ~x;
        if (w < nw) {
            if (t) R[w] = 0u;
            f(w, x & range_mask(w, w_lo, i_lo, i_hi));
        }
        carry ^= (unsigned)__popc(odd) & 1u;
    }
    __syncwarp();
}

// the 16-pixel halves of a word whose 16 bits of v are all set, as a mask
__device__ __forceinline__ uint32_t full_halves(uint32_t v) {
    return ((v & 0xFFFFu) == 0xFFFFu ? 0xFFFFu : 0u) | ((v >> 16) == 0xFFFFu ? 0xFFFF0000u : 0u);
}

template <int MODE>
__global__ void __launch_bounds__(kTW * 32) k_tier_pass(PolyPassArgs a, TierArgs tr) {
    extern __shared__ int4 s_tier[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned FULL = 0xffffffffu;
    const int TP = a.T * a.P;
    const int total = a.band_start[TP];
    int4* my_edge = s_tier + (size_t)warp * kTEdgeCap;
    uint32_t* my_I = reinterpret_cast<uint32_t*>(s_tier + (size_t)kTW * kTEdgeCap) + (size_t)warp * 3 * kTWords;
    uint32_t* my_U = my_I + kTWords;   // label pass: the mixed blocks' mask instead
    uint32_t* my_R = my_U + kTWords;
    for (int w = lane; w < kTWords; w += 32) my_R[w] = 0u;   // row_cover keeps it zero between rows
    __syncwarp();
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

        if (MODE == MODE_TIER_CLASSIFY && tr.outline) {
            // blocks within two pixels of an edge near this band (rows
            // jb - 2 .. jb + 17) become mixed: the error-bound outline pass
            // reads per-pixel counts up to a pixel beside each edge, rows one
            // beyond the polygon's included
            const float ylo = (float)(jb - 2), yhi = (float)(jb + kTBand + 2);
            const int ne = overflow ? n : nb;
            for (int e = lane; e < ne; e += 32) {
                int4 q;
                if (!overflow) {
                    q = my_edge[e];
                } else {
                    const int2 A = pv[e];
                    const int2 B = pv[(e + 1 == n) ? 0 : e + 1];
                    q = make_int4(A.x, A.y, B.x, B.y);
                }
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

        // I: pixels covered on every row of the block row; U: on some row
        const int nw = w_hi - w_lo + 1;
        const bool rows_ok = jb + kTBand - 1 <= a.resy - 1;
        for (int w = lane; w < nw; w += 32) {
            const int x0 = (w_lo + w) * 32;
            const int a0 = max(i_lo - x0, 0), b0 = min(i_hi + 1 - x0, 32);
            my_I[w] = (rows_ok && a0 < b0) ? bitrange(a0, b0) : 0u;
            my_U[w] = 0u;
        }
        __syncwarp();
        if (MODE != MODE_TIER_LABEL) {
            // per 32-word chunk (warp-uniform): I already zero, U already the
            // whole range -- both only ever move that way, so a chunk that no
            // crossing touches needs no update once its flag is set
            uint32_t izero = rows_ok ? 0u : 0xFFu, ufull = 0u;
            for (int r = 0; r < kTBand; ++r) {
                const int j = jb + r;
                const bool live = j <= a.resy - 1 && j >= j_lo && j <= j_hi;
                if (live) {
                    row_cover(
                        j, my_edge, nb, overflow, pv, n, i_lo, i_hi, w_lo, nw, my_R, lane,
                        [&](int w, uint32_t v) {
                            my_I[w] &= v;
                            if (MODE == MODE_TIER_CLASSIFY) my_U[w] |= v;
                        },
                        [&](int w0, uint32_t carry) {
                            const uint32_t c = 1u << (w0 >> 5);
                            const int w = w0 + lane;
                            if (carry) {
                                if (MODE == MODE_TIER_CLASSIFY && !(ufull & c)) {
                                    if (w < nw) my_U[w] |= range_mask(w, w_lo, i_lo, i_hi);
                                    ufull |= c;
                                }
                            } else if (!(izero & c)) {
                                if (w < nw) my_I[w] = 0u;
                                izero |= c;
                            }
                        });
                } else {
                    for (int w = lane; w < nw; w += 32) my_I[w] = 0u;
                    izero = 0xFFu;
                    __syncwarp();
                }
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

        // ---- canvas modes
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
        // covered pixels of the blocks that are not full for p (reduce) or of
        // the mixed blocks (labels): the pixel slots.  keep[w]: the halves of
        // word w whose pixels are visited, found once per band (labels: the
        // mixed blocks; reduce: all but p's full blocks).
        if (MODE == MODE_TIER_LABEL) {
            for (int w = lane; w < nw; w += 32) {
                const int bc = (w_lo + w) * 2;
                const bool m0 = __ldg(tr.mixed + blk0 + bc) != 0;
                const bool m1 = bc + 1 < tr.bw && __ldg(tr.mixed + blk0 + bc + 1) != 0;
                my_U[w] = (m0 ? 0xFFFFu : 0u) | (m1 ? 0xFFFF0000u : 0u);
            }
            __syncwarp();
        }
        for (int r = 0; r < kTBand; ++r) {
            const int j = jb + r;
            if (!(j <= a.resy - 1 && j >= j_lo && j <= j_hi)) continue;
            auto visit = [&](int w, uint32_t bits) {
                bits &= (MODE == MODE_TIER_LABEL) ? my_U[w] : ~full_halves(my_I[w]);
                if (!bits) return;
                const int x0 = (w_lo + w) * 32;
                #pragma unroll
                for (int half = 0; half < 2; ++half) {
                    uint32_t hb = (bits >> (half * 16)) & 0xFFFFu;
                    if (!hb) continue;
                    const size_t b = blk0 + (x0 >> 4) + half;
                    const size_t base = (size_t)__ldg(tr.slot + b) * 256 + (size_t)(j & 15) * 16;
                    while (hb) {
                        const int bit = __ffs(hb) - 1;
                        hb &= hb - 1u;
                        const size_t q = base + bit;   // (x0 + 16 * half + bit) & 15 == bit
                        if (MODE == MODE_TIER_LABEL) {
                            tr.plabel[q] = (uint16_t)p;
                            ++acc_c;
                        } else {
                            acc_c += __ldg(tr.pcnt + q);
                            if (tr.psum) acc_s += __ldg(tr.psum + q);
                        }
                    }
                }
            };
            row_cover(j, my_edge, nb, overflow, pv, n, i_lo, i_hi, w_lo, nw, my_R, lane, visit,
                      [&](int w0, uint32_t carry) {
                          // an untouched chunk: all covered (visit it) or none
                          const int w = w0 + lane;
                          if (carry && w < nw) visit(w, range_mask(w, w_lo, i_lo, i_hi));
                      });
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
