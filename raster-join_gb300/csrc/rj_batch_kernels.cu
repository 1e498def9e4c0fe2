// rj_batch_kernels.cu -- batched raster join point pass and the time index
// of the resident point table.
//
// Batched point pass.  A batch holds many raster-join queries (each with its
// own polygon set, canvas resolution, filters and aggregate) over one
// resident point table.  The table's rows are cut into segments: maximal row
// ranges covered by the same set of queries (each query touches the rows of
// its time window, or all rows).  A work item is a block of consecutive rows
// of one segment.  A thread block takes items from a device counter, stages
// the item's location pairs and every column the batch reads in shared
// memory once, and then runs each query of the segment over the staged rows:
// interval predicates, the query's canvas pixel, then the polygon label
// (label map) or an additive splat into the query's canvas.  So every point
// is read from HBM once per batch, however many queries admit it.
// Per-polygon counts and fixed-point sums go through a shared-memory
// histogram per (item, query) when the query's polygon count fits, else
// through warp-aggregated global atomics.
//
// Time index.  The table can be reordered into time buckets (a counting sort
// on the bucket of a uint32 time column): a query's time window then maps to
// a contiguous row range, and the exact time predicate still filters inside
// it.  Results do not depend on row order (counts are integers, sums are
// int64 fixed point).
#include "rj_batch_common.cuh"

namespace rj {

size_t batch_smem_bytes(const BatchShape& s, int nu, int hist_cap) {
    return (size_t)hist_cap * 16 + (s.direct ? 0 : (size_t)s.rows * (8 + 4 * (size_t)nu));
}

// Staged rows [0, nrows) of one query with the mapper of MODE (one loop per
// mode, so only that mapper's state is live in it).
template <int MODE, bool AGG, bool SMEM, int BLOCK>
__device__ __forceinline__ void staged_rows(const BatchArgs& a, const BatchQuery* __restrict__ Q, const float2* s_xy,
                                            const uint32_t* s_col, int nrows, const Hist<AGG, SMEM, true>& h,
                                            const QueryCols* qc) {
    const int tid = threadIdx.x;
    const int ncu = qc->n, aggc = qc->aggr;
    const int aggr_typ = Q->aggr_typ;
    const CanvasXf cx = Q->cx;
    for (int base = 0; base < nrows; base += 4 * BLOCK) {
        float x[4], y[4], v[4];
        uint32_t mask = 0u;
        #pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int r = base + k * BLOCK + tid;
            x[k] = y[k] = v[k] = 0.f;
            if (r >= nrows) continue;
            const float2 p = s_xy[r];
            x[k] = p.x;
            y[k] = p.y;
            bool ok = true;
            #pragma unroll 1
            for (int u = 0; u < ncu; ++u) {
                const uint32_t c = s_col[qc->slot[u] * a.rows + r];
                ok = ok && (order_key(qc->typ[u], c) - qc->lo[u] <= qc->span[u]);
                if (AGG && u == aggc) v[k] = agg_value(aggr_typ, c);
            }
            if (ok) mask |= 1u << k;
        }
        map_points4<MODE, AGG, SMEM>(Q, cx, x, y, v, mask, h);
    }
}

template <bool AGG, bool SMEM, int BLOCK>
__device__ __forceinline__ void batch_query(const BatchArgs& a, const BatchQuery* __restrict__ Q,
                                            const float2* s_xy, const uint32_t* s_col, int nrows,
                                            uint32_t* s_cnt, unsigned long long* s_sum, int* s_touch,
                                            int* s_ntouch, QueryCols* qc) {
    load_query_cols(a, Q, qc);
    Hist<AGG, SMEM, true> h{s_cnt, s_sum, Q->out_count, Q->out_sum, Q->out_nonfinite, Q->sum_scale};
    h.s_touched = s_touch;
    h.s_ntouched = s_ntouch;
    switch (Q->mode) {
        case BQ_TLABEL: staged_rows<BQ_TLABEL, AGG, SMEM, BLOCK>(a, Q, s_xy, s_col, nrows, h, qc); break;
        case BQ_TSPLAT: staged_rows<BQ_TSPLAT, AGG, SMEM, BLOCK>(a, Q, s_xy, s_col, nrows, h, qc); break;
        case BQ_LABEL: staged_rows<BQ_LABEL, AGG, SMEM, BLOCK>(a, Q, s_xy, s_col, nrows, h, qc); break;
        default: staged_rows<BQ_SPLAT, AGG, SMEM, BLOCK>(a, Q, s_xy, s_col, nrows, h, qc); break;
    }
    // the flush's barriers also keep qc until every thread is done with it
    if (SMEM) flush_touched<AGG, BLOCK>(Q, s_cnt, s_sum, s_touch, s_ntouch);
    else __syncthreads();
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, 768 / BLOCK) k_batch_points(BatchArgs a) {
    extern __shared__ unsigned long long smem_b[];
    unsigned long long* s_sum = smem_b;
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(s_sum + a.hist_cap);
    int* s_touch = reinterpret_cast<int*>(s_cnt + a.hist_cap);
    float2* s_xy = reinterpret_cast<float2*>(s_touch + a.hist_cap);   // hist_cap is even: 8-byte aligned
    uint32_t* s_col = reinterpret_cast<uint32_t*>(s_xy + a.rows);
    __shared__ unsigned long long s_item;
    __shared__ int s_seg;
    __shared__ int s_ntouch;
    __shared__ float4 s_box[BLOCK / 32 + 1];
    __shared__ QueryCols s_qc;
    const int tid = threadIdx.x;
    hist_init(s_cnt, s_sum, a.hist_cap, &s_ntouch);
    for (;;) {
        if (tid == 0) {
            const unsigned long long it = atomicAdd(a.work, 1ull);
            int seg = 0;
            if (it < a.nitems) {
                // last segment whose first item is <= it
                int lo = 0, hi = a.nseg - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (a.seg[mid].item0 <= it) lo = mid;
                    else hi = mid - 1;
                }
                seg = lo;
            }
            s_item = it;
            s_seg = seg;
        }
        __syncthreads();
        const unsigned long long item = s_item;
        if (item >= a.nitems) break;
        const BatchSeg sg = a.seg[s_seg];
        const uint64_t r0 = sg.r0 + (item - sg.item0) * (uint64_t)a.rows;
        const uint64_t rend = r0 + (uint64_t)a.rows < sg.r1 ? r0 + (uint64_t)a.rows : sg.r1;
        const int nrows = (int)(rend - r0);
        // stage the item's rows (read once per batch: evict-first)
        // (and the item's location bounds: queries whose canvas lies apart
        // from them skip the item; clustered tables make items compact)
        float bx0 = INFINITY, by0 = INFINITY, bx1 = -INFINITY, by1 = -INFINITY;
        #pragma unroll 4
        for (int i = tid; i < nrows; i += BLOCK) {
            const float2 p = __ldcs(a.xy + r0 + i);
            s_xy[i] = p;
            bx0 = fminf(bx0, p.x); bx1 = fmaxf(bx1, p.x);
            by0 = fminf(by0, p.y); by1 = fmaxf(by1, p.y);
        }
        #pragma unroll
        for (int u = 0; u < kBatchMaxCols; ++u) {
            if (u >= a.nu) break;
            const uint32_t* col = a.ucol[u] + r0;
            uint32_t* dst = s_col + u * a.rows;
            #pragma unroll 4
            for (int i = tid; i < nrows; i += BLOCK) dst[i] = __ldcs(col + i);
        }
        bx0 = warp_minf(bx0); bx1 = warp_maxf(bx1);
        by0 = warp_minf(by0); by1 = warp_maxf(by1);
        if ((tid & 31) == 0) s_box[tid >> 5] = make_float4(bx0, by0, bx1, by1);
        __syncthreads();
        if (tid == 0) {
            float4 b = s_box[0];
            for (int w = 1; w < BLOCK / 32; ++w) {
                const float4 o = s_box[w];
                b = make_float4(fminf(b.x, o.x), fminf(b.y, o.y), fmaxf(b.z, o.z), fmaxf(b.w, o.w));
            }
            s_box[BLOCK / 32] = b;
        }
        __syncthreads();
        const float4 ibox = s_box[BLOCK / 32];   // NaN coordinates drop out of fminf / fmaxf
        for (int qi = sg.qbegin; qi < sg.qend; ++qi) {
            const BatchQuery* Q = a.q + __ldg(a.qlist + qi);
            const int mode = Q->mode;
            if (mode == BQ_SKIP) continue;
            const float4 qb = Q->box;
            if (ibox.z < qb.x || ibox.x > qb.z || ibox.w < qb.y || ibox.y > qb.w) continue;   // uniform
            const bool agg = Q->aggr_u >= 0;
            const bool smem = Q->hist_smem != 0;
            if (agg) {
                if (smem) batch_query<true, true, BLOCK>(a, Q, s_xy, s_col, nrows, s_cnt, s_sum, s_touch, &s_ntouch, &s_qc);
                else batch_query<true, false, BLOCK>(a, Q, s_xy, s_col, nrows, s_cnt, s_sum, s_touch, &s_ntouch, &s_qc);
            } else {
                if (smem) batch_query<false, true, BLOCK>(a, Q, s_xy, s_col, nrows, s_cnt, s_sum, s_touch, &s_ntouch, &s_qc);
                else batch_query<false, false, BLOCK>(a, Q, s_xy, s_col, nrows, s_cnt, s_sum, s_touch, &s_ntouch, &s_qc);
            }
        }
        __syncthreads();   // the staged rows are overwritten by the next item
    }
}

int batch_blocks_per_sm(const BatchShape& s, int nu, int hist_cap) {
    const size_t smem = batch_smem_bytes(s, nu, hist_cap);
    if (s.direct) return batch_direct_blocks_per_sm(s.threads, smem);
    return s.threads == 512 ? blocks_per_sm_k(k_batch_points<512>, 512, smem) : blocks_per_sm_k(k_batch_points<256>, 256, smem);
}

bool launch_batch_points(const BatchArgs& a, const BatchShape& s, int sms, cudaStream_t st) {
    if (a.nitems == 0) return true;
    const size_t smem = batch_smem_bytes(s, a.nu, a.hist_cap);
    const int per_sm = batch_blocks_per_sm(s, a.nu, a.hist_cap);
    if (per_sm < 1) return false;
    uint64_t blocks = (uint64_t)sms * per_sm;
    if (blocks > a.nitems) blocks = a.nitems;
    if (s.direct) {
        launch_batch_direct(a, s.threads, (unsigned)blocks, smem, st);
    } else {
        if (s.threads == 512) k_batch_points<512><<<(unsigned)blocks, 512, smem, st>>>(a);
        else k_batch_points<256><<<(unsigned)blocks, 256, smem, st>>>(a);
    }
    ++g_kernel_launches;
    return true;
}

// ---------------------------------------------------------------------------
// Time index kernels.
__device__ __forceinline__ uint32_t time_bucket(uint32_t t, uint32_t tmin, uint32_t tmax, int nb) {
    if (t <= tmin) return 0u;
    if (t >= tmax) return (uint32_t)nb - 1u;
    return (uint32_t)(((uint64_t)(t - tmin) * (uint64_t)nb) / ((uint64_t)(tmax - tmin) + 1ull));
}

__global__ void k_time_minmax(const uint32_t* __restrict__ t, uint64_t n, unsigned* out_min, unsigned* out_max) {
    unsigned lo = 0xFFFFFFFFu, hi = 0u;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned v = __ldcs(t + i);
        lo = min(lo, v);
        hi = max(hi, v);
    }
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(out_min, lo);
        atomicMax(out_max, hi);
    }
}

void launch_time_minmax(const uint32_t* t, uint64_t n, unsigned* out_min, unsigned* out_max, int sms, cudaStream_t st) {
    uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8);
    if (blocks < 1) blocks = 1;
    k_time_minmax<<<(unsigned)blocks, 256, 0, st>>>(t, n, out_min, out_max);
    ++g_kernel_launches;
}

// ---------------------------------------------------------------------------
// Clustered row order: key = time bucket (major) then the Z-order of a
// 2^cb x 2^cb cell grid over the location bounds (minor).  A counting sort
// on the key puts the rows of one time slice and one cell next to each
// other, as the reference backend's spatio-temporal partitions do.
__device__ __forceinline__ uint32_t spread_bits(uint32_t v) {
    v &= 0xFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

__device__ __forceinline__ uint32_t cluster_key(const ClusterKey& k, uint64_t i) {
    const uint32_t tb = k.t ? time_bucket(k.t[i], k.tmin, k.tmax, k.nbt) : 0u;
    if (k.cb == 0) return tb;
    const float2 p = k.xy[i];
    const int top = (1 << k.cb) - 1;
    const float fx = (p.x - k.x0) * k.sx, fy = (p.y - k.y0) * k.sy;
    const int cx = fx >= 0.f ? min((int)fx, top) : 0;   // NaN -> 0
    const int cy = fy >= 0.f ? min((int)fy, top) : 0;
    return (tb << (2 * k.cb)) | spread_bits((uint32_t)cx) | (spread_bits((uint32_t)cy) << 1);
}

// float <-> unsigned with the same order (for atomicMin / atomicMax)
__device__ __forceinline__ unsigned float_order(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void k_xy_bounds(const float2* __restrict__ xy, uint64_t n, unsigned* __restrict__ out) {
    unsigned lx = 0xFFFFFFFFu, ly = 0xFFFFFFFFu, hx = 0u, hy = 0u;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float2 p = __ldcs(xy + i);
        if (isfinite(p.x)) { lx = min(lx, float_order(p.x)); hx = max(hx, float_order(p.x)); }
        if (isfinite(p.y)) { ly = min(ly, float_order(p.y)); hy = max(hy, float_order(p.y)); }
    }
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lx = min(lx, __shfl_xor_sync(0xffffffffu, lx, o));
        ly = min(ly, __shfl_xor_sync(0xffffffffu, ly, o));
        hx = max(hx, __shfl_xor_sync(0xffffffffu, hx, o));
        hy = max(hy, __shfl_xor_sync(0xffffffffu, hy, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(out + 0, lx);
        atomicMin(out + 1, ly);
        atomicMax(out + 2, hx);
        atomicMax(out + 3, hy);
    }
}

void launch_xy_bounds(const float2* xy, uint64_t n, unsigned* out, int sms, cudaStream_t st) {
    uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8);
    if (blocks < 1) blocks = 1;
    k_xy_bounds<<<(unsigned)blocks, 256, 0, st>>>(xy, n, out);
    ++g_kernel_launches;
}

// key histogram: lanes with the same key add once (global counters, up to 2^24 keys)
__global__ void k_cluster_hist(ClusterKey k, uint64_t n, unsigned* __restrict__ hist) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    for (uint64_t w0 = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u); w0 < n; w0 += stride) {
        const uint64_t i = w0 + lane;
        const bool valid = i < n;
        const uint32_t key = valid ? cluster_key(k, i) : 0u;
        const unsigned active = __ballot_sync(0xffffffffu, valid);
        if (!valid) continue;
        const unsigned peers = __match_any_sync(active, key);
        if (lane == __ffs(peers) - 1) atomicAdd(hist + key, (unsigned)__popc(peers));
    }
}

void launch_cluster_hist(const ClusterKey& k, uint64_t n, unsigned* hist, int sms, cudaStream_t st) {
    uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8);
    if (blocks < 1) blocks = 1;
    k_cluster_hist<<<(unsigned)blocks, 256, 0, st>>>(k, n, hist);
    ++g_kernel_launches;
}

__global__ void k_cluster_scatter(ClusterKey k, uint64_t n, unsigned long long* __restrict__ cursor, PermuteCols pc) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    for (uint64_t w0 = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u); w0 < n; w0 += stride) {
        const uint64_t i = w0 + lane;
        const bool valid = i < n;
        const uint32_t key = valid ? cluster_key(k, i) : 0u;
        const unsigned active = __ballot_sync(0xffffffffu, valid);
        if (!valid) continue;
        const unsigned peers = __match_any_sync(active, key);
        const int leader = __ffs(peers) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(cursor + key, (unsigned long long)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        const uint64_t pos = base + __popc(peers & ((1u << lane) - 1u));
        for (int c = 0; c < pc.ncol; ++c) {
            if (pc.esz[c] == 8)
                reinterpret_cast<uint2*>(pc.dst[c])[pos] = reinterpret_cast<const uint2*>(pc.src[c])[i];
            else
                reinterpret_cast<uint32_t*>(pc.dst[c])[pos] = reinterpret_cast<const uint32_t*>(pc.src[c])[i];
        }
    }
}

void launch_cluster_scatter(const ClusterKey& k, uint64_t n, unsigned long long* cursor, const PermuteCols& pc, int sms,
                            cudaStream_t st) {
    uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8);
    if (blocks < 1) blocks = 1;
    k_cluster_scatter<<<(unsigned)blocks, 256, 0, st>>>(k, n, cursor, pc);
    ++g_kernel_launches;
}

// rows whose bucket is below the previous row's (0: already in bucket order)
__global__ void k_time_unsorted(const uint32_t* __restrict__ t, uint64_t n, uint32_t tmin, uint32_t tmax, int nb,
                                unsigned long long* __restrict__ count) {
    unsigned long long c = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x + 1; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        c += time_bucket(__ldcs(t + i), tmin, tmax, nb) < time_bucket(t[i - 1], tmin, tmax, nb);
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

void launch_time_unsorted(const uint32_t* t, uint64_t n, uint32_t tmin, uint32_t tmax, int nb, unsigned long long* count,
                          int sms, cudaStream_t st) {
    uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8);
    if (blocks < 1) blocks = 1;
    k_time_unsorted<<<(unsigned)blocks, 256, 0, st>>>(t, n, tmin, tmax, nb, count);
    ++g_kernel_launches;
}

}  // namespace rj
