// rj_batch_direct.cu -- the direct form of the batched point pass (rows
// streamed per query through registers, re-read from L2 by the segment's
// other queries).  A translation unit of its own so the two forms of the
// batched pass compile in parallel.
#include "rj_batch_common.cuh"

namespace rj {

// Direct variant: no staging.  Each query of an item streams the item's rows
// straight into registers with 128-bit loads (four rows per thread), as the
// single-query point pass does; the first query brings the block of rows into
// L2 and the others of the segment hit it there (the last one reads with
// evict-first).  Items are longer (more rows per histogram flush); segment
// boundaries are multiples of four rows, so the vector loads stay aligned.
//
// direct_rows: rows [r0, r1) of one query with the mapper of MODE (one loop
// per mode, so only that mapper's state is live in it).
template <int MODE, bool AGG, bool SMEM, int BLOCK>
__device__ __forceinline__ void direct_rows(const BatchArgs& a, const BatchQuery* __restrict__ Q, uint64_t r0,
                                            uint64_t r1, bool last, const Hist<AGG, SMEM, true>& h, const QueryCols* dc) {
    const int tid = threadIdx.x;
    const int ncu = dc->n, aggc = dc->aggr;
    const int aggr_typ = Q->aggr_typ;
    const float4 qb = Q->box;
    const float4* zones = Q->zones;
    const CanvasXf cx = Q->cx;
    for (uint64_t tb = r0; tb < r1; tb += (uint64_t)BLOCK * 4) {
        if (zones) {
            // skip rows whose zones lie apart from the query's polygons (uniform)
            const uint64_t z0 = tb >> kZoneShift;
            const uint64_t z1 = (min(tb + (uint64_t)BLOCK * 4, r1) - 1) >> kZoneShift;
            bool meets = false;
            for (uint64_t z = z0; z <= z1; ++z) {
                const float4 b = __ldg(zones + z);
                meets |= !(b.z < qb.x || b.x > qb.z || b.w < qb.y || b.y > qb.w);
            }
            if (!meets) continue;
        }
        const uint64_t base = tb + (uint64_t)tid * 4;
        float x[4], y[4], v[4];
        uint32_t mask = 0u;
        if (base + 4 <= r1) {
            const float4 p0 = last ? __ldcs(reinterpret_cast<const float4*>(a.xy + base))
                                   : __ldcg(reinterpret_cast<const float4*>(a.xy + base));
            const float4 p1 = last ? __ldcs(reinterpret_cast<const float4*>(a.xy + base + 2))
                                   : __ldcg(reinterpret_cast<const float4*>(a.xy + base + 2));
            x[0] = p0.x; y[0] = p0.y; x[1] = p0.z; y[1] = p0.w;
            x[2] = p1.x; y[2] = p1.y; x[3] = p1.z; y[3] = p1.w;
            v[0] = v[1] = v[2] = v[3] = 0.f;
            mask = 0xFu;
            #pragma unroll 1
            for (int u = 0; u < ncu; ++u) {
                const uint4* cp = reinterpret_cast<const uint4*>(dc->col[u] + base);
                const uint4 c = last ? __ldcs(cp) : __ldcg(cp);
                const int t = dc->typ[u];
                const uint32_t lo = dc->lo[u], sp = dc->span[u];
                mask &= ((order_key(t, c.x) - lo <= sp) ? 1u : 0u) | ((order_key(t, c.y) - lo <= sp) ? 2u : 0u) |
                        ((order_key(t, c.z) - lo <= sp) ? 4u : 0u) | ((order_key(t, c.w) - lo <= sp) ? 8u : 0u);
                if (AGG && u == aggc) {
                    v[0] = agg_value(aggr_typ, c.x); v[1] = agg_value(aggr_typ, c.y);
                    v[2] = agg_value(aggr_typ, c.z); v[3] = agg_value(aggr_typ, c.w);
                }
            }
        } else {
            #pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint64_t i = base + k;
                x[k] = y[k] = v[k] = 0.f;
                if (i >= r1) continue;
                const float2 p = a.xy[i];
                x[k] = p.x;
                y[k] = p.y;
                bool ok = true;
                #pragma unroll 1
                for (int u = 0; u < ncu; ++u) {
                    const uint32_t c = dc->col[u][i];
                    ok = ok && (order_key(dc->typ[u], c) - dc->lo[u] <= dc->span[u]);
                    if (AGG && u == aggc) v[k] = agg_value(aggr_typ, c);
                }
                if (ok) mask |= 1u << k;
            }
        }
        map_points4<MODE, AGG, SMEM>(Q, cx, x, y, v, mask, h);
    }
}

template <bool AGG, bool SMEM, int BLOCK>
__device__ __forceinline__ void direct_query(const BatchArgs& a, const BatchQuery* __restrict__ Q, uint64_t r0,
                                             uint64_t r1, bool last, uint32_t* s_cnt, unsigned long long* s_sum,
                                             int* s_touch, int* s_ntouch, QueryCols* dc) {
    load_query_cols(a, Q, dc);
    Hist<AGG, SMEM, true> h{s_cnt, s_sum, Q->out_count, Q->out_sum, Q->out_nonfinite, Q->sum_scale};
    h.s_touched = s_touch;
    h.s_ntouched = s_ntouch;
    switch (Q->mode) {
        case BQ_TLABEL: direct_rows<BQ_TLABEL, AGG, SMEM, BLOCK>(a, Q, r0, r1, last, h, dc); break;
        case BQ_TSPLAT: direct_rows<BQ_TSPLAT, AGG, SMEM, BLOCK>(a, Q, r0, r1, last, h, dc); break;
        case BQ_LABEL: direct_rows<BQ_LABEL, AGG, SMEM, BLOCK>(a, Q, r0, r1, last, h, dc); break;
        default: direct_rows<BQ_SPLAT, AGG, SMEM, BLOCK>(a, Q, r0, r1, last, h, dc); break;
    }
    // the flush's barriers also keep dc until every thread is done with it
    if (SMEM) flush_touched<AGG, BLOCK>(Q, s_cnt, s_sum, s_touch, s_ntouch);
    else __syncthreads();
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, 768 / BLOCK) k_batch_direct(BatchArgs a) {
    extern __shared__ unsigned long long smem_b[];
    unsigned long long* s_sum = smem_b;
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(s_sum + a.hist_cap);
    int* s_touch = reinterpret_cast<int*>(s_cnt + a.hist_cap);
    __shared__ unsigned long long s_item;
    __shared__ int s_seg;
    __shared__ int s_ntouch;
    __shared__ QueryCols s_dc;
    const int tid = threadIdx.x;
    hist_init(s_cnt, s_sum, a.hist_cap, &s_ntouch);
    for (;;) {
        if (tid == 0) {
            const unsigned long long it = atomicAdd(a.work, 1ull);
            int seg = 0;
            if (it < a.nitems) {
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
        const uint64_t r1 = r0 + (uint64_t)a.rows < sg.r1 ? r0 + (uint64_t)a.rows : sg.r1;
        for (int qi = sg.qbegin; qi < sg.qend; ++qi) {
            const BatchQuery* Q = a.q + __ldg(a.qlist + qi);
            if (Q->mode == BQ_SKIP) continue;
            const bool last = qi + 1 == sg.qend;
            const bool agg = Q->aggr_u >= 0;
            const bool smem = Q->hist_smem != 0;
            if (agg) {
                if (smem) direct_query<true, true, BLOCK>(a, Q, r0, r1, last, s_cnt, s_sum, s_touch, &s_ntouch, &s_dc);
                else direct_query<true, false, BLOCK>(a, Q, r0, r1, last, s_cnt, s_sum, s_touch, &s_ntouch, &s_dc);
            } else {
                if (smem) direct_query<false, true, BLOCK>(a, Q, r0, r1, last, s_cnt, s_sum, s_touch, &s_ntouch, &s_dc);
                else direct_query<false, false, BLOCK>(a, Q, r0, r1, last, s_cnt, s_sum, s_touch, &s_ntouch, &s_dc);
            }
        }
        __syncthreads();   // s_item is rewritten for the next item
    }
}

int batch_direct_blocks_per_sm(int threads, size_t smem) {
    return threads == 512 ? blocks_per_sm_k(k_batch_direct<512>, 512, smem)
                          : blocks_per_sm_k(k_batch_direct<256>, 256, smem);
}

void launch_batch_direct(const BatchArgs& a, int threads, unsigned blocks, size_t smem, cudaStream_t st) {
    if (threads == 512) k_batch_direct<512><<<blocks, 512, smem, st>>>(a);
    else k_batch_direct<256><<<blocks, 256, smem, st>>>(a);
}

}  // namespace rj
