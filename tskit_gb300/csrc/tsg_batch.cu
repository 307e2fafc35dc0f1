// Batched stage kernels: one launch per stage of the compact item pipeline
// for every query of a batch, whatever tree sequence each query reads.  A
// query owns a contiguous range of each stage's blocks (a prefix array of
// per-query block counts, built on the host); a block finds its query by a
// binary search of that array and runs the same stage body as the
// single-query kernel on the query's descriptor, so every result is bitwise
// the one its own launch gives.  The replay is persistent: its blocks take
// (query, span) items from one counter over all queries' spans, so short and
// long tree sequences share the GPU's blocks.
#include "tsg_items.cuh"
#include "tsg_replay_compact.cuh"

namespace tsg {

// Zeroes each query's accumulators: the error and span-counter words, the
// running sums' start, the leaves' fixed-point areas and the exact site-sum
// counters (8-byte words, in that order).
__global__ void __launch_bounds__(256) kb_zero(const BatchQuery *bq, const int64_t *off, int nq)
{
    TSG_BATCH_QUERY();
    const QueryParams &p = Q.p;
    const int64_t n_err = 1, n_rs0 = p.R;
    const int64_t n_leaf = p.branch ? ((int64_t) p.Wn << p.K) * TSG_FX_LIMBS * 3 : 0;
    const int64_t n_site = p.site && p.site_int ? (int64_t) p.Wn * p.R * 2 : 0;
    const int64_t total = n_err + n_rs0 + n_leaf + n_site;
    for (int64_t i = bid * blockDim.x + threadIdx.x; i < total; i += nb * blockDim.x) {
        uint64_t *word;
        if (i < n_err) {
            word = (uint64_t *) Q.w.err;
        } else if (i < n_err + n_rs0) {
            word = (uint64_t *) Q.w.rs0 + (i - n_err);
        } else if (i < n_err + n_rs0 + n_leaf) {
            word = (uint64_t *) Q.w.leaf_area + (i - n_err - n_rs0);
        } else {
            word = (uint64_t *) Q.w.site_acc + (i - n_err - n_rs0 - n_leaf);
        }
        *word = 0;
    }
}

__global__ void __launch_bounds__(256) kb_node_mask(const BatchQuery *bq, const int64_t *off, int nq)
{
    TSG_BATCH_QUERY();
    node_mask_body(Q.v, Q.d, Q.w.node_mask, bid, nb);
}

template <int KQ>
__global__ void __launch_bounds__(1024) kb_compact_prefix(const BatchQuery *bq, const int64_t *off,
    int nq)
{
    TSG_BATCH_QUERY();
    compact_prefix_body<KQ>(Q.v, Q.p, Q.d, Q.w.cp0, bid, nb);
}

template <int KQ>
__global__ void __launch_bounds__(TSG_ROWS_THREADS, 8) kb_compact_rows(const BatchQuery *bq,
    const int64_t *off, int nq)
{
    __shared__ RowsWarp<KQ> sh[TSG_ROWS_THREADS / 32];
    TSG_BATCH_QUERY();
    compact_rows_body<KQ>(Q.v, Q.p, Q.d, Q.w, sh, bid, nb);
}

template <int KQ>
__global__ void __launch_bounds__(256) kb_compact_anchors(const BatchQuery *bq, const int64_t *off,
    int nq)
{
    TSG_BATCH_QUERY();
    compact_anchors_body<KQ>(Q.v, Q.p, Q.w.cp0, Q.w, bid, nb);
}

__global__ void __launch_bounds__(256) kb_span_windows(const BatchQuery *bq, const int64_t *off,
    int nq)
{
    TSG_BATCH_QUERY();
    span_windows_body(Q.v, Q.p, Q.d, Q.w, bid, nb);
}

__global__ void __launch_bounds__(256) kb_leaf_areas(const BatchQuery *bq, const int64_t *off, int nq)
{
    TSG_BATCH_QUERY();
    leaf_areas_body(Q.v, Q.p, Q.d, Q.w, bid, nb);
}

__global__ void __launch_bounds__(256) kb_leaf_prefix(const BatchQuery *bq, const int64_t *off,
    int nq)
{
    TSG_BATCH_QUERY();
    leaf_prefix_body(Q.p, Q.d, Q.w, bid, nb);
}

__global__ void __launch_bounds__(256) kb_leaf_terms(const BatchQuery *bq, const int64_t *off, int nq)
{
    TSG_BATCH_QUERY();
    leaf_terms_body<16>(Q.p, Q.w, bid, nb);
}

template <int KQ>
__global__ void __launch_bounds__(256) kb_site_sums(const BatchQuery *bq, const int64_t *off, int nq)
{
    TSG_BATCH_QUERY();
    site_sums_body<16, KQ>(Q.v, Q.p, Q.d, Q.w, bid, nb);
}

__global__ void __launch_bounds__(256) kb_site_sums_finish(const BatchQuery *bq, const int64_t *off,
    int nq)
{
    TSG_BATCH_QUERY();
    site_sums_finish_body(Q.p, Q.w, bid, nb);
}

__global__ void __launch_bounds__(512) kb_span_scan(const BatchQuery *bq, const int64_t *off, int nq)
{
    TSG_BATCH_QUERY();
    span_scan_body(Q.w.D, Q.w.rs0, Q.w.RS, Q.v.num_segs, Q.p.R, bid, nb);
}

__global__ void __launch_bounds__(256) kb_window_reduce(const BatchQuery *bq, const int64_t *off,
    int nq)
{
    TSG_BATCH_QUERY();
    window_reduce_body(Q.p, Q.d, Q.w, Q.span_normalise, 1, Q.result, bid, nb);
}

// The compact replay of every query: persistent blocks take global span
// indexes from `counter` (zeroed before the launch); span_off[b] is query
// b's first global span.
template <int KQ>
__global__ void __launch_bounds__(TSG_COMPACT_THREADS, 20) kb_replay_compact(const BatchQuery *bq,
    const int64_t *span_off, int nq, int32_t *counter)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_span;
    __shared__ CompactShared<KQ> sh;
    const int64_t total = span_off[nq];
    for (;;) {
        if (threadIdx.x == 0) {
            s_span = atomicAdd(counter, 1);
        }
        __syncthreads();
        const int64_t g = s_span;
        __syncthreads();
        if (g >= total) {
            break;
        }
        const int b = batch_find(span_off, nq, g);
        const BatchQuery &Q = bq[b];
        compact_span<KQ>(Q.v, Q.p, Q.d, Q.w, (int) (g - span_off[b]), smem_raw, sh.list,
            sh.stage);
    }
}

void *batch_replay_kernel(int kq)
{
    return kq == 1 ? (void *) kb_replay_compact<1> : (void *) kb_replay_compact<2>;
}

int batch_launch_replay(int kq, unsigned grid, size_t smem, cudaStream_t st, const BatchQuery *bq,
    int nq, const int64_t *span_off, int32_t *counter)
{
    if (kq == 1) {
        kb_replay_compact<1><<<grid, TSG_COMPACT_THREADS, smem, st>>>(bq, span_off, nq, counter);
    } else {
        kb_replay_compact<2><<<grid, TSG_COMPACT_THREADS, smem, st>>>(bq, span_off, nq, counter);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_ERR_CUDA;
}

int batch_launch_stage(int stage, int kq, int64_t blocks, cudaStream_t st, const BatchQuery *bq,
    int nq, const int64_t *off)
{
    if (blocks <= 0) {
        return 0;
    }
    const unsigned g = (unsigned) blocks;
    switch (stage) {
        case BS_ZERO: kb_zero<<<g, 256, 0, st>>>(bq, off, nq); break;
        case BS_NODE_MASK: kb_node_mask<<<g, 256, 0, st>>>(bq, off, nq); break;
        case BS_PREFIX:
            if (kq == 1) {
                kb_compact_prefix<1><<<g, 1024, 0, st>>>(bq, off, nq);
            } else {
                kb_compact_prefix<2><<<g, 1024, 0, st>>>(bq, off, nq);
            }
            break;
        case BS_ANCHORS:
            if (kq == 1) {
                kb_compact_anchors<1><<<g, 256, 0, st>>>(bq, off, nq);
            } else {
                kb_compact_anchors<2><<<g, 256, 0, st>>>(bq, off, nq);
            }
            break;
        case BS_ROWS:
            if (kq == 1) {
                kb_compact_rows<1><<<g, TSG_ROWS_THREADS, 0, st>>>(bq, off, nq);
            } else {
                kb_compact_rows<2><<<g, TSG_ROWS_THREADS, 0, st>>>(bq, off, nq);
            }
            break;
        case BS_SPAN_WINDOWS: kb_span_windows<<<g, 256, 0, st>>>(bq, off, nq); break;
        case BS_LEAF_AREAS: kb_leaf_areas<<<g, 256, 0, st>>>(bq, off, nq); break;
        case BS_LEAF_PREFIX: kb_leaf_prefix<<<g, 256, 0, st>>>(bq, off, nq); break;
        case BS_LEAF_TERMS: kb_leaf_terms<<<g, 256, 0, st>>>(bq, off, nq); break;
        case BS_SITE_SUMS:
            if (kq == 1) {
                kb_site_sums<1><<<g, 256, 0, st>>>(bq, off, nq);
            } else {
                kb_site_sums<2><<<g, 256, 0, st>>>(bq, off, nq);
            }
            break;
        case BS_SITE_FINISH: kb_site_sums_finish<<<g, 256, 0, st>>>(bq, off, nq); break;
        case BS_SPAN_SCAN: kb_span_scan<<<g, 512, 0, st>>>(bq, off, nq); break;
        case BS_REDUCE: kb_window_reduce<<<g, 256, 0, st>>>(bq, off, nq); break;
        default: return TSG_ERR_BAD_PARAM_VALUE;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : TSG_ERR_CUDA;
}

}  // namespace tsg
