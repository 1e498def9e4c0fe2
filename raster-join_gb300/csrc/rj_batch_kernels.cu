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
#include "rj_device.cuh"
#include "rj_launch.h"
#include "rj_point_map.cuh"

namespace rj {

size_t batch_smem_bytes(const BatchShape& s, int nu, int hist_cap) {
    return (size_t)hist_cap * 12 + (size_t)s.rows * (8 + 4 * (size_t)nu);
}

template <bool AGG, bool SMEM, int BLOCK>
__device__ __forceinline__ void batch_query(const BatchArgs& a, const BatchQuery* __restrict__ Q,
                                            const float2* s_xy, const uint32_t* s_col, int nrows,
                                            uint32_t* s_cnt, unsigned long long* s_sum) {
    const int tid = threadIdx.x;
    const int mode = Q->mode;
    const int P = Q->P;
    uint32_t lo[kBatchMaxCols], span[kBatchMaxCols];
    #pragma unroll
    for (int u = 0; u < kBatchMaxCols; ++u) {
        lo[u] = Q->lo[u];
        span[u] = Q->span[u];
    }
    const int aggr_u = Q->aggr_u;
    const int aggr_typ = Q->aggr_typ;
    if (SMEM) {
        for (int b = tid; b < P; b += BLOCK) {
            s_cnt[b] = 0u;
            if (AGG) s_sum[b] = 0ull;
        }
        __syncthreads();
    }
    Hist<AGG, SMEM> h{s_cnt, s_sum, Q->out_count, Q->out_sum, Q->out_nonfinite, Q->sum_scale};
    const DeferQ dq{nullptr, nullptr, nullptr, nullptr};
    const CanvasXf cx = Q->cx;
    if (mode == BQ_LABEL) {
        const LabelMapper m{cx, Q->label};
        for (int base = 0; base < nrows; base += 4 * BLOCK) {
            float x[4], y[4], v[4];
            bool ok[4];
            LabelMapper::Key key[4];
            #pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int r = base + k * BLOCK + tid;
                ok[k] = r < nrows;
                x[k] = y[k] = v[k] = 0.f;
                key[k] = LabelMapper::kNone;
                if (ok[k]) {
                    const float2 p = s_xy[r];
                    x[k] = p.x;
                    y[k] = p.y;
                    #pragma unroll
                    for (int u = 0; u < kBatchMaxCols; ++u)
                        if (u < a.nu) ok[k] = ok[k] && (order_key(a.utyp[u], s_col[u * a.rows + r]) - lo[u] <= span[u]);
                    if (AGG && ok[k]) v[k] = agg_value(aggr_typ, s_col[aggr_u * a.rows + r]);
                    if (ok[k]) key[k] = m.lookup(x[k], y[k]);
                }
            }
            #pragma unroll
            for (int k = 0; k < 4; ++k) m.consume(ok[k], key[k], x[k], y[k], v[k], h, dq);
        }
    } else {
        const SplatMapper m{cx, Q->canvas_c, Q->canvas_s, Q->sum_scale, Q->out_nonfinite, SMEM ? 1 : 0};
        for (int base = 0; base < nrows; base += 4 * BLOCK) {
            float x[4], y[4], v[4];
            bool ok[4];
            SplatMapper::Key key[4];
            #pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int r = base + k * BLOCK + tid;
                ok[k] = r < nrows;
                x[k] = y[k] = v[k] = 0.f;
                key[k] = SplatMapper::kNone;
                if (ok[k]) {
                    const float2 p = s_xy[r];
                    x[k] = p.x;
                    y[k] = p.y;
                    #pragma unroll
                    for (int u = 0; u < kBatchMaxCols; ++u)
                        if (u < a.nu) ok[k] = ok[k] && (order_key(a.utyp[u], s_col[u * a.rows + r]) - lo[u] <= span[u]);
                    if (AGG && ok[k]) v[k] = agg_value(aggr_typ, s_col[aggr_u * a.rows + r]);
                    if (ok[k]) key[k] = m.lookup(x[k], y[k]);
                }
            }
            #pragma unroll
            for (int k = 0; k < 4; ++k) m.consume(ok[k], key[k], x[k], y[k], v[k], h, dq);
        }
    }
    if (SMEM) {
        __syncthreads();
        for (int b = tid; b < P; b += BLOCK) {
            const uint32_t c = s_cnt[b];
            if (c) {
                if (Q->out_count32) atomicAdd(Q->out_count32 + b, c);   // private splat canvas
                else atomicAdd(Q->out_count + b, (unsigned long long)c);
                if (AGG) atomicAdd(Q->out_sum + b, s_sum[b]);
            }
        }
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_batch_points(BatchArgs a) {
    extern __shared__ unsigned long long smem_b[];
    unsigned long long* s_sum = smem_b;
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(s_sum + a.hist_cap);
    float2* s_xy = reinterpret_cast<float2*>(s_cnt + a.hist_cap);   // hist_cap is even: 8-byte aligned
    uint32_t* s_col = reinterpret_cast<uint32_t*>(s_xy + a.rows);
    __shared__ unsigned long long s_item;
    __shared__ int s_seg;
    const int tid = threadIdx.x;
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
        #pragma unroll 4
        for (int i = tid; i < nrows; i += BLOCK) s_xy[i] = __ldcs(a.xy + r0 + i);
        #pragma unroll
        for (int u = 0; u < kBatchMaxCols; ++u) {
            if (u >= a.nu) break;
            const uint32_t* col = a.ucol[u] + r0;
            uint32_t* dst = s_col + u * a.rows;
            #pragma unroll 4
            for (int i = tid; i < nrows; i += BLOCK) dst[i] = __ldcs(col + i);
        }
        __syncthreads();
        for (int qi = sg.qbegin; qi < sg.qend; ++qi) {
            const BatchQuery* Q = a.q + __ldg(a.qlist + qi);
            const int mode = Q->mode;
            if (mode == BQ_SKIP) continue;
            const bool agg = Q->aggr_u >= 0;
            const bool smem = Q->hist_smem != 0;
            if (agg) {
                if (smem) batch_query<true, true, BLOCK>(a, Q, s_xy, s_col, nrows, s_cnt, s_sum);
                else batch_query<true, false, BLOCK>(a, Q, s_xy, s_col, nrows, s_cnt, s_sum);
            } else {
                if (smem) batch_query<false, true, BLOCK>(a, Q, s_xy, s_col, nrows, s_cnt, s_sum);
                else batch_query<false, false, BLOCK>(a, Q, s_xy, s_col, nrows, s_cnt, s_sum);
            }
        }
        __syncthreads();   // the staged rows are overwritten by the next item
    }
}

template <int BLOCK>
static int blocks_per_sm_t(size_t smem) {
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_batch_points<BLOCK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_points<BLOCK>, BLOCK, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return per_sm;
}

int batch_blocks_per_sm(const BatchShape& s, int nu, int hist_cap) {
    const size_t smem = batch_smem_bytes(s, nu, hist_cap);
    return s.threads == 512 ? blocks_per_sm_t<512>(smem) : blocks_per_sm_t<256>(smem);
}

bool launch_batch_points(const BatchArgs& a, const BatchShape& s, int sms, cudaStream_t st) {
    if (a.nitems == 0) return true;
    const size_t smem = batch_smem_bytes(s, a.nu, a.hist_cap);
    const int per_sm = batch_blocks_per_sm(s, a.nu, a.hist_cap);
    if (per_sm < 1) return false;
    uint64_t blocks = (uint64_t)sms * per_sm;
    if (blocks > a.nitems) blocks = a.nitems;
    if (s.threads == 512) k_batch_points<512><<<(unsigned)blocks, 512, smem, st>>>(a);
    else k_batch_points<256><<<(unsigned)blocks, 256, smem, st>>>(a);
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

// bucket histogram: per-block shared counts (nb <= 16384), flushed once
__global__ void k_time_hist(const uint32_t* __restrict__ t, uint64_t n, uint32_t tmin, uint32_t tmax, int nb,
                            unsigned* __restrict__ hist) {
    extern __shared__ unsigned s_h[];
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s_h[b] = 0u;
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(s_h + time_bucket(__ldcs(t + i), tmin, tmax, nb), 1u);
    __syncthreads();
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        if (s_h[b]) atomicAdd(hist + b, s_h[b]);
}

void launch_time_hist(const uint32_t* t, uint64_t n, uint32_t tmin, uint32_t tmax, int nb, unsigned* hist, int sms,
                      cudaStream_t st) {
    const size_t smem = (size_t)nb * sizeof(unsigned);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_time_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    uint64_t blocks = std::min<uint64_t>((n + 1023) / 1024, (uint64_t)sms * 2);
    if (blocks < 1) blocks = 1;
    k_time_hist<<<(unsigned)blocks, 1024, smem, st>>>(t, n, tmin, tmax, nb, hist);
    ++g_kernel_launches;
}

// Scatter every column of row i to its bucket slot.  Lanes of a warp with the
// same bucket reserve their slots with one atomic.
__global__ void k_time_scatter(const uint32_t* __restrict__ t, uint64_t n, uint32_t tmin, uint32_t tmax, int nb,
                               unsigned long long* __restrict__ cursor, PermuteCols pc) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    // warp-uniform trip count
    const uint64_t first = (blockIdx.x * (uint64_t)blockDim.x) + (threadIdx.x & ~31u);
    for (uint64_t w0 = first; w0 < n; w0 += stride) {
        const uint64_t i = w0 + lane;
        const bool valid = i < n;
        const uint32_t b = valid ? time_bucket(t[i], tmin, tmax, nb) : 0xFFFFFFFFu;
        const unsigned active = __ballot_sync(0xffffffffu, valid);
        if (!valid) continue;
        const unsigned peers = __match_any_sync(active, b);
        const int leader = __ffs(peers) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(cursor + b, (unsigned long long)__popc(peers));
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

void launch_time_scatter(const uint32_t* t, uint64_t n, uint32_t tmin, uint32_t tmax, int nb,
                         unsigned long long* cursor, const PermuteCols& pc, int sms, cudaStream_t st) {
    uint64_t blocks = std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8);
    if (blocks < 1) blocks = 1;
    k_time_scatter<<<(unsigned)blocks, 256, 0, st>>>(t, n, tmin, tmax, nb, cursor, pc);
    ++g_kernel_launches;
}

}  // namespace rj
