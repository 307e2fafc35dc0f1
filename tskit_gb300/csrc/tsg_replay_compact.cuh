// The compact replay: the item pipeline's replay over the compact span plan
// (tsg_cplan.cu).  One block of one warp (TSG_COMPACT_THREADS) per span at a
// time, the span's node state (16-bit counts packed in 64-bit words and
// 16-bit parent entries) in shared memory: a few kilobytes, so about twenty
// blocks -- twenty sequential replays -- run on every SM.
//
//   seek     the prefix sum of the sample-set bits along the span's
//            depth-first sample order, TSG_SEEK_PER samples per lane and
//            step (warp shuffles), the next step's loads in flight, and at
//            each sorted range endpoint a node's count: P[hi] - P[lo] (the
//            start is stored first, the end then subtracts it);
//   replay   replay_span over the compact encodings.
//
// The first tree's items (its stateful nodes, the anchors) are written by
// k_compact_anchors from the prefix sum of the first span's order
// (k_compact_prefix); the replay writes every other item with its branch
// lengths, and k_eval_grouped values every chunk of items after it, all
// chunks in parallel.
#pragma once

#include "tsg_replay_kernel.cuh"

namespace tsg {

#define TSG_COMPACT_THREADS 32

// samples per thread in one step of the seek
#define TSG_SEEK_PER 4

// Counts of span s's compact nodes at the span start into sp.xq.  The seek
// takes TSG_COMPACT_THREADS x TSG_SEEK_PER samples of the span's order per
// step, each thread TSG_SEEK_PER consecutive ones, and loads the next step's
// order entries and sample masks while it scans the current one.  s_pre:
// (TSG_COMPACT_THREADS + 1) x 2 words, each thread's exclusive prefix (and
// the step's total); s_mask: the step's masks; s_wsum: 2 words per warp.
// Ends with the block synchronised.
template <int KQ>
__device__ __forceinline__ void compact_seek(const TSView &ts, const QueryDev &qd, int K, int s,
    const SpanState<uint16_t> &sp, uint64_t *s_pre, uint64_t *s_wsum, uint32_t *s_mask)
{
    constexpr int T = TSG_COMPACT_THREADS, PER = TSG_SEEK_PER, STEP = T * PER;
    constexpr int NW = T / 32;
    const int64_t n = ts.num_samples;
    const uint16_t *order = ts.c_order + (int64_t) s * n;
    const int2 *ep = ts.c_ep + ts.c_ep_off[s];
    const int64_t nep = ts.c_ep_off[s + 1] - ts.c_ep_off[s];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    uint32_t cur_m[PER], nxt_m[PER];
    auto fetch = [&](int64_t base, uint32_t (&mm)[PER]) {
        uint32_t o[PER];
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const int64_t i = base + (int64_t) tid * PER + j;
            o[j] = i < n ? (uint32_t) order[i] : 0u;
        }
#pragma unroll
        for (int j = 0; j < PER; j++) {
            const int64_t i = base + (int64_t) tid * PER + j;
            mm[j] = i < n ? qd.sample_mask[o[j]] : 0u;
        }
    };
    fetch(0, cur_m);
    uint64_t run_lo = 0, run_hi = 0;
    int64_t cur = 0;
    for (int64_t base = 0; base < n; base += STEP) {
        if (base + STEP < n) {
            fetch(base + STEP, nxt_m);
        }
        uint64_t t_lo = 0, t_hi = 0;
#pragma unroll
        for (int j = 0; j < PER; j++) {
            s_mask[tid * PER + j] = cur_m[j];
            const Pack v = pk_from_mask<16>(cur_m[j], K);
            t_lo += v.lo;
            t_hi += v.hi;
        }
        // inclusive scan of the threads' totals within the warp (fields
        // never carry: prefix counts stay within the set sizes)
        uint64_t inc_lo = t_lo, inc_hi = t_hi;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t a = __shfl_up_sync(0xffffffffu, inc_lo, o);
            const uint64_t b = KQ > 1 ? __shfl_up_sync(0xffffffffu, inc_hi, o) : 0ull;
            if (lane >= o) {
                inc_lo += a;
                inc_hi += b;
            }
        }
        if (lane == 31) {
            s_wsum[2 * wid] = inc_lo;
            s_wsum[2 * wid + 1] = inc_hi;
        }
        __syncthreads();
        uint64_t wp_lo = 0, wp_hi = 0, tot_lo = 0, tot_hi = 0;
#pragma unroll
        for (int j = 0; j < NW; j++) {
            const uint64_t a = s_wsum[2 * j], b = s_wsum[2 * j + 1];
            if (j < wid) {
                wp_lo += a;
                wp_hi += b;
            }
            tot_lo += a;
            tot_hi += b;
        }
        // P at position base + tid * PER (the samples before it)
        s_pre[2 * tid] = run_lo + wp_lo + inc_lo - t_lo;
        s_pre[2 * tid + 1] = run_hi + wp_hi + inc_hi - t_hi;
        if (tid == 0) {
            s_pre[2 * T] = run_lo + tot_lo;
            s_pre[2 * T + 1] = run_hi + tot_hi;
        }
        __syncthreads();
        // every endpoint at a position up to base + STEP (the sorted list's
        // next entries; earlier positions were taken by earlier steps):
        // P there is its thread's prefix plus the masks before it
        const int64_t lim = base + STEP;
        for (;;) {
            const int64_t j = cur + tid;
            int2 e = make_int2(0, 0);
            bool mine = false;
            if (j < nep) {
                e = ep[j];
                mine = e.x <= lim;
            }
            const int cnt = __syncthreads_count(mine);
            const int64_t l = e.y >> 1;
            uint64_t p_lo = 0, p_hi = 0;
            if (mine) {
                const int at = (int) (e.x - base);
                const int tt = at / PER, jj = at - tt * PER;
                p_lo = s_pre[2 * tt];
                p_hi = s_pre[2 * tt + 1];
                for (int q = 0; q < jj; q++) {
                    const Pack v = pk_from_mask<16>(s_mask[tt * PER + q], K);
                    p_lo += v.lo;
                    p_hi += v.hi;
                }
            }
            if (mine && !(e.y & 1)) {
                sp.xq[l * KQ] = p_lo;
                if (KQ > 1) {
                    sp.xq[l * KQ + (KQ > 1 ? 1 : 0)] = p_hi;
                }
            }
            __syncthreads();
            if (mine && (e.y & 1)) {
                sp.xq[l * KQ] = p_lo - sp.xq[l * KQ];
                if (KQ > 1) {
                    sp.xq[l * KQ + (KQ > 1 ? 1 : 0)] = p_hi - sp.xq[l * KQ + (KQ > 1 ? 1 : 0)];
                }
            }
            cur += cnt;
            if (cnt < T) {
                break;
            }
            __syncthreads();
        }
        run_lo = s_pre[2 * T];
        run_hi = s_pre[2 * T + 1];
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PER; j++) {
            cur_m[j] = nxt_m[j];
        }
    }
}

// Span s of the compact plan, by one block: the span-start parents and
// counts, then warp 0 replays the span's trees.  Ends with the block
// synchronised.
template <int KQ>
__device__ __forceinline__ void compact_span(const TSView &ts, const QueryParams &q,
    const QueryDev &qd, const WsDev &w, int s, unsigned char *smem_raw,
    TouchEntry<KQ> *s_list, ReplayStage *s_stage, uint64_t *s_pre, uint64_t *s_wsum,
    uint32_t *s_mask)
{
    SpanState<uint16_t> sp = span_state_at<uint16_t>(smem_raw, ts.c_max_local, KQ);
    sp.cnt = nullptr;
    const int32_t t0 = ts.c_span_tree[s], t1 = ts.c_span_tree[s + 1];
    const int64_t lo = ts.c_local_off[s];
    const int32_t Ls = (int32_t) (ts.c_local_off[s + 1] - lo);
    sp.time = ts.c_time + lo;
    // parents at the span start (0x7FFF, no parent, is the replay's
    // "no parent" entry)
    for (int32_t l = threadIdx.x; l < Ls; l += blockDim.x) {
        sp.par[l] = ts.c_par0[lo + l];
    }
    compact_seek<KQ>(ts, qd, q.K, s, sp, s_pre, s_wsum, s_mask);
    if (threadIdx.x < 32) {
        replay_span<16, KQ, uint16_t, false, true>(ts, q, qd, w, sp, s_list, s_stage, nullptr, t0,
            t1, Ls, ReplayEnc{ts.c_rem_enc, ts.c_ins_enc, ts.c_mut_enc});
    }
    __syncthreads();
}

// The block-shared arrays of the compact replay besides the span state
// (the seek's scratch and the replay's staging ring are never live at the
// same time: they share their bytes).
template <int KQ>
struct CompactShared {
    TouchEntry<KQ> list[TSG_TOUCH_CAP];  // the open touch list
    union {
        ReplayStage stage[4];            // prefetch ring, trees t .. t + 3
        struct {
            uint64_t pre[2 * (TSG_COMPACT_THREADS + 1)];
            uint32_t mask[TSG_COMPACT_THREADS * TSG_SEEK_PER];
        } seek;
    };
    uint64_t wsum[2 * (TSG_COMPACT_THREADS / 32)];
};

// Persistent blocks take spans from the query's counter until none is left.
template <int KQ>
__global__ void __launch_bounds__(TSG_COMPACT_THREADS) k_replay_compact(TSView ts, QueryParams q,
    QueryDev qd, WsDev w)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_span;
    __shared__ CompactShared<KQ> sh;
    for (;;) {
        if (threadIdx.x == 0) {
            s_span = atomicAdd(w.counter, 1);
        }
        __syncthreads();
        const int s = s_span;
        __syncthreads();
        if (s >= ts.c_num_spans) {
            break;
        }
        compact_span<KQ>(ts, q, qd, w, s, smem_raw, sh.list, sh.stage, sh.seek.pre, sh.wsum,
            sh.seek.mask);
    }
}

// Prefix sums of the sample-set bits along the first span's sample order,
// P0[i] for i = 0 .. n (two words each): block b takes samples
// [1024 b, 1024 (b + 1)), first summing every sample before them (a strided
// sum and a block reduction; the orders are short), then scanning its own.
template <int KQ>
__device__ __forceinline__ void compact_prefix_body(const TSView &ts, const QueryParams &q, const QueryDev &qd, uint64_t *P0,
    const int64_t bid, const int64_t nb)
{
    __shared__ uint64_t s_w[2 * 32];
    __shared__ uint64_t s_off[2];
    const int64_t n = ts.num_samples;
    const uint16_t *order = ts.c_order;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int nw = (int) (blockDim.x >> 5);
    const int64_t base = (int64_t) bid * blockDim.x;
    // the samples before this block
    uint64_t pre_lo = 0, pre_hi = 0;
    for (int64_t i = tid; i < base && i < n; i += blockDim.x) {
        const Pack v = pk_from_mask<16>(qd.sample_mask[order[i]], q.K);
        pre_lo += v.lo;
        pre_hi += v.hi;
    }
    for (int o = 16; o > 0; o >>= 1) {
        pre_lo += __shfl_xor_sync(0xffffffffu, pre_lo, o);
        pre_hi += __shfl_xor_sync(0xffffffffu, pre_hi, o);
    }
    if (lane == 0) {
        s_w[2 * wid] = pre_lo;
        s_w[2 * wid + 1] = pre_hi;
    }
    __syncthreads();
    if (tid == 0) {
        uint64_t a = 0, b = 0;
        for (int j = 0; j < nw; j++) {
            a += s_w[2 * j];
            b += s_w[2 * j + 1];
        }
        s_off[0] = a;
        s_off[1] = b;
    }
    __syncthreads();
    const uint64_t run_lo = s_off[0], run_hi = s_off[1];
    // this block's samples
    const int64_t i = base + tid;
    Pack v{0, 0};
    if (i < n) {
        v = pk_from_mask<16>(qd.sample_mask[order[i]], q.K);
    }
    uint64_t inc_lo = v.lo, inc_hi = v.hi;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t a = __shfl_up_sync(0xffffffffu, inc_lo, o);
        const uint64_t b = __shfl_up_sync(0xffffffffu, inc_hi, o);
        if (lane >= o) {
            inc_lo += a;
            inc_hi += b;
        }
    }
    __syncthreads();
    if (lane == 31) {
        s_w[2 * wid] = inc_lo;
        s_w[2 * wid + 1] = inc_hi;
    }
    __syncthreads();
    uint64_t wp_lo = 0, wp_hi = 0, tot_lo = 0, tot_hi = 0;
    for (int j = 0; j < nw; j++) {
        const uint64_t a = s_w[2 * j], b = s_w[2 * j + 1];
        if (j < wid) {
            wp_lo += a;
            wp_hi += b;
        }
        tot_lo += a;
        tot_hi += b;
    }
    if (i < n) {
        P0[2 * i] = run_lo + wp_lo + inc_lo - v.lo;
        P0[2 * i + 1] = run_hi + wp_hi + inc_hi - v.hi;
    }
    if (tid == 0 && base + (int64_t) blockDim.x >= n) {
        P0[2 * n] = run_lo + tot_lo;
        P0[2 * n + 1] = run_hi + tot_hi;
    }
}

template <int KQ>
__global__ void __launch_bounds__(1024) k_compact_prefix(TSView ts, QueryParams q, QueryDev qd,
    uint64_t *P0)
{
    compact_prefix_body<KQ>(ts, q, qd, P0, blockIdx.x, gridDim.x);
}

// The first tree's items: one per anchor (a stateful node alive in the first
// tree, in edge order) with its counts, P0[hi] - P0[lo], and its parent, in
// the anchors' numbering.
template <int KQ>
__device__ __forceinline__ void compact_anchors_body(const TSView &ts, const QueryParams &q,
    const uint64_t *P0, const WsDev &w, const int64_t bid, const int64_t nb)
{
    Item<KQ> *items = (Item<KQ> *) w.items;
    const int64_t base = ts.tree_item_off[0];
    // the first tree's items read the node times of the span that numbers them
    const double *time = ts.c_time + ts.c_local_off[ts.c_chunk_span[ts.tree_chunk_off[0]]];
    for (int64_t k = bid * (int64_t) blockDim.x + threadIdx.x; k < ts.c_num_anchors;
         k += (int64_t) nb * blockDim.x) {
        const int2 r = ts.c_anchor_range[k];
        Pack x;
        x.lo = P0[2 * r.y] - P0[2 * r.x];
        x.hi = P0[2 * r.y + 1] - P0[2 * r.x + 1];
        const int32_t p1 = ts.c_anchor_par[k];
        item_put<KQ>(items + base + k, Pack{0, 0}, x, (int32_t) k, -1, p1);
        // branch lengths (no branch before: bl0 = 0)
        const double bl1 = p1 >= 0 ? time[p1] - time[k] : 0.0;
        if (q.f32) {
            float *bls = (float *) w.bl;
            bls[2 * (base + k)] = (float) bl1;
            bls[2 * (base + k) + 1] = 0.0f;
        } else {
            double *bls = (double *) w.bl;
            bls[2 * (base + k)] = bl1;
            bls[2 * (base + k) + 1] = 0.0;
        }
    }
}

template <int KQ>
__global__ void k_compact_anchors(TSView ts, QueryParams q, const uint64_t *P0, WsDev w)
{
    compact_anchors_body<KQ>(ts, q, P0, w, blockIdx.x, gridDim.x);
}

}  // namespace tsg
