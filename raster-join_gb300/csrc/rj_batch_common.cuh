// rj_batch_common.cuh -- pieces shared by the two forms of the batched point
// pass (staged and direct): the touched-list histogram flush, the per-query
// column list and the per-mode point mapping.
#pragma once
#include "rj_device.cuh"
#include "rj_launch.h"
#include "rj_point_map.cuh"

namespace rj {

// The shared histogram stays zero between (item, query) visits: a flush
// visits only the keys whose count left zero (the touched list) and zeroes
// them again, so a visit costs its hits, not the query's polygon count.
template <bool AGG, int BLOCK>
__device__ __forceinline__ void flush_touched(const BatchQuery* __restrict__ Q, uint32_t* s_cnt,
                                              unsigned long long* s_sum, int* s_touch, int* s_ntouch) {
    __syncthreads();
    const int nt = *s_ntouch;
    for (int k = threadIdx.x; k < nt; k += BLOCK) {
        const int b = s_touch[k];
        const uint32_t c = s_cnt[b];
        if (Q->out_count32) atomicAdd(Q->out_count32 + b, c);   // private splat canvas
        else atomicAdd(Q->out_count + b, (unsigned long long)c);
        s_cnt[b] = 0u;
        if (AGG) {
            atomicAdd(Q->out_sum + b, s_sum[b]);
            s_sum[b] = 0ull;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *s_ntouch = 0;
    __syncthreads();
}

__device__ __forceinline__ void hist_init(uint32_t* s_cnt, unsigned long long* s_sum, int cap, int* s_ntouch) {
    for (int b = threadIdx.x; b < cap; b += blockDim.x) {
        s_cnt[b] = 0u;
        s_sum[b] = 0ull;
    }
    if (threadIdx.x == 0) *s_ntouch = 0;
    __syncthreads();
}

// The columns one query reads, in shared memory (read as broadcasts inside
// the row loops instead of being held in registers): device pointers for the
// direct pass, staged column slots for the staged one.
struct QueryCols {
    const uint32_t* col[kBatchMaxCols];
    int slot[kBatchMaxCols];
    uint32_t lo[kBatchMaxCols], span[kBatchMaxCols];
    int typ[kBatchMaxCols];
    int n;       // columns with a predicate or the aggregate
    int aggr;    // index of the aggregate column in the list, or -1
};

// Fills `qc` for query Q (thread 0) and publishes it to the block.
__device__ __forceinline__ void load_query_cols(const BatchArgs& a, const BatchQuery* __restrict__ Q, QueryCols* qc) {
    if (threadIdx.x == 0) {
        // a predicate narrower than the full range, or the aggregate
        int n = 0;
        qc->aggr = -1;
        for (int u = 0; u < a.nu; ++u) {
            const uint32_t lo = Q->lo[u], sp = Q->span[u];
            if (lo == 0u && sp == 0xFFFFFFFFu && u != Q->aggr_u) continue;
            if (u == Q->aggr_u) qc->aggr = n;
            qc->col[n] = a.ucol[u];
            qc->slot[n] = u;
            qc->typ[n] = a.utyp[u];
            qc->lo[n] = lo;
            qc->span[n] = sp;
            ++n;
        }
        qc->n = n;
    }
    __syncthreads();
}

// The four points x/y/v/mask of one thread through the mapper of MODE.
template <int MODE, bool AGG, bool SMEM>
__device__ __forceinline__ void map_points4(const BatchQuery* __restrict__ Q, const CanvasXf& cx, const float* x,
                                            const float* y, const float* v, uint32_t mask, const Hist<AGG, SMEM, true>& h) {
    const DeferQ dq{nullptr, nullptr, nullptr, nullptr};
    if constexpr (MODE == BQ_TLABEL) {
        const TierLabelMapper tm{cx, Q->tr};
        uint32_t key[4];
        #pragma unroll
        for (int k = 0; k < 4; ++k) key[k] = ((mask >> k) & 1u) ? tm.lookup(x[k], y[k]) : TierLabelMapper::kNone;
        #pragma unroll
        for (int k = 0; k < 4; ++k) tm.consume(((mask >> k) & 1u) != 0u, key[k], x[k], y[k], v[k], h, dq);
    } else if constexpr (MODE == BQ_TSPLAT) {
        const TierSplatMapper tm{cx, Q->tr, Q->sum_scale};
        uint32_t key[4];
        #pragma unroll
        for (int k = 0; k < 4; ++k) key[k] = ((mask >> k) & 1u) ? tm.lookup(x[k], y[k]) : TierSplatMapper::kNone;
        #pragma unroll
        for (int k = 0; k < 4; ++k) tm.consume(((mask >> k) & 1u) != 0u, key[k], x[k], y[k], v[k], h, dq);
    } else if constexpr (MODE == BQ_LABEL) {
        const LabelMapper lm{cx, Q->label};
        LabelMapper::Key key[4];
        #pragma unroll
        for (int k = 0; k < 4; ++k) key[k] = ((mask >> k) & 1u) ? lm.lookup(x[k], y[k]) : LabelMapper::kNone;
        #pragma unroll
        for (int k = 0; k < 4; ++k) lm.consume(((mask >> k) & 1u) != 0u, key[k], x[k], y[k], v[k], h, dq);
    } else {
        const SplatMapper sm{cx, Q->canvas_c, Q->canvas_s, Q->sum_scale, Q->out_nonfinite, SMEM ? 1 : 0};
        SplatMapper::Key key[4];
        #pragma unroll
        for (int k = 0; k < 4; ++k) key[k] = ((mask >> k) & 1u) ? sm.lookup(x[k], y[k]) : SplatMapper::kNone;
        #pragma unroll
        for (int k = 0; k < 4; ++k) sm.consume(((mask >> k) & 1u) != 0u, key[k], x[k], y[k], v[k], h, dq);
    }
}

template <class K>
inline int blocks_per_sm_k(K kernel, int block, size_t smem) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return per_sm;
}

// the direct form lives in its own translation unit (rj_batch_direct.cu)
int batch_direct_blocks_per_sm(int threads, size_t smem);
void launch_batch_direct(const BatchArgs& a, int threads, unsigned blocks, size_t smem, cudaStream_t st);

}  // namespace rj
