// The compact replay: the item pipeline's replay over the compact span plan
// (tsg_cplan.cu).  One block of one warp (TSG_COMPACT_THREADS) per span at a
// time, the span's node state (16-bit counts packed in 64-bit words and
// 16-bit parent entries) in shared memory: a few kilobytes, so about twenty
// blocks -- twenty sequential replays -- run on every SM.
//
//   rows     (k_compact_rows, before the replay, every span at once) each
//            span's depth-first sample order in rows of 32 positions: per
//            row a membership word per set (ballots) and the packed counts
//            before the row (prefix sums of population counts);
//   seek     at each of the span's sorted range endpoints a node's count,
//            P[hi] - P[lo], P read from the rows in O(1) (the start is
//            stored first, the end then subtracts it);
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

// rows of 32 positions of a compact span's depth-first sample order, plus
// the row holding the span's totals (k_compact_rows)
__host__ __device__ __forceinline__ int64_t compact_row_stride(int64_t n)
{
    return (n + 31) / 32 + 1;
}

#define TSG_ROWS_THREADS 256
// rows a warp of k_compact_rows loads at once
#define TSG_ROWS_BATCH 8

// The rows of compact span s's order (one block of TSG_ROWS_THREADS per span
// at a time, a lane per position): warp w takes rows w, w + 8, ... --
// TSG_ROWS_BATCH of them per round, their order entries and then their
// sample masks loaded together -- and ballots each set's membership bits
// into a 32-bit word (4 x KQ words per row, w.c_bits) whose population
// counts give the row's packed counts; then warp 0 turns the counts (held in
// w.c_rowpre) into exclusive prefix sums in row order, the row after the
// last taking the span's totals.  Counts fit their 16-bit fields (at most
// the set sizes), so packed words add without carries.
template <int KQ>
__device__ __forceinline__ void compact_rows_body(const TSView &ts, const QueryParams &q,
    const QueryDev &qd, const WsDev &w, const int64_t bid, const int64_t nb)
{
    constexpr int NW = TSG_ROWS_THREADS / 32, RB = TSG_ROWS_BATCH, KW = 4 * KQ;
    const int64_t n = ts.num_samples;
    const int64_t nrows = (n + 31) / 32, stride = compact_row_stride(n);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int K = q.K;
    for (int64_t s = bid; s < ts.c_num_spans; s += nb) {
        const uint16_t *order = ts.c_order + s * n;
        uint32_t *bits = w.c_bits + s * stride * KW;
        uint64_t *pre = w.c_rowpre + s * stride * KQ;
        for (int64_t r0 = wid; r0 < nrows; r0 += (int64_t) NW * RB) {
            uint32_t m[RB];
#pragma unroll
            for (int b = 0; b < RB; b++) {
                const int64_t i = (r0 + (int64_t) b * NW) * 32 + lane;
                m[b] = i < n ? (uint32_t) order[i] : 0xFFFFFFFFu;
            }
#pragma unroll
            for (int b = 0; b < RB; b++) {
                m[b] = m[b] != 0xFFFFFFFFu ? qd.sample_mask[m[b]] : 0u;
            }
#pragma unroll
            for (int b = 0; b < RB; b++) {
                const int64_t r = r0 + (int64_t) b * NW;
                if (r >= nrows) {
                    break;
                }
                uint64_t c[KQ];
#pragma unroll
                for (int h = 0; h < KQ; h++) {
                    c[h] = 0;
                }
#pragma unroll
                for (int k = 0; k < KW; k++) {
                    const uint32_t word = __ballot_sync(0xffffffffu, k < K && ((m[b] >> k) & 1u));
                    if (lane == k) {
                        bits[r * KW + k] = word;
                    }
                    c[k / 4] += (uint64_t) __popc(word) << (16 * (k % 4));
                }
                if (lane == 0) {
#pragma unroll
                    for (int h = 0; h < KQ; h++) {
                        pre[r * KQ + h] = c[h];
                    }
                }
            }
        }
        __syncthreads();
        if (wid == 0) {
            uint64_t run[KQ];
#pragma unroll
            for (int h = 0; h < KQ; h++) {
                run[h] = 0;
            }
            for (int64_t r0 = 0; r0 < nrows; r0 += 32) {
                const int64_t r = r0 + lane;
#pragma unroll
                for (int h = 0; h < KQ; h++) {
                    const uint64_t v = r < nrows ? pre[r * KQ + h] : 0ull;
                    uint64_t inc = v;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint64_t a = __shfl_up_sync(0xffffffffu, inc, o);
                        if (lane >= o) {
                            inc += a;
                        }
                    }
                    if (r < nrows) {
                        pre[r * KQ + h] = run[h] + inc - v;
                    }
                    run[h] += __shfl_sync(0xffffffffu, inc, 31);
                }
            }
            if (lane == 0) {
#pragma unroll
                for (int h = 0; h < KQ; h++) {
                    pre[nrows * KQ + h] = run[h];
                }
            }
        }
        __syncthreads();
    }
}

template <int KQ>
__global__ void __launch_bounds__(TSG_ROWS_THREADS) k_compact_rows(TSView ts, QueryParams q,
    QueryDev qd, WsDev w)
{
    compact_rows_body<KQ>(ts, q, qd, w, blockIdx.x, gridDim.x);
}

// Counts of span s's compact nodes at the span start into sp.xq, from the
// span's rows (k_compact_rows): the members before depth-first position x
// are the prefix of x's row plus, per set, the population count of the
// row's membership word below x.  The span's range endpoints, sorted, are
// taken TSG_COMPACT_THREADS at a time, a thread each; a node's start count
// is stored first and its end then subtracts it.  Ends with the block
// synchronised.
template <int KQ>
__device__ __forceinline__ void compact_seek(const TSView &ts, const WsDev &w, int s,
    const SpanState<uint16_t> &sp)
{
    constexpr int T = TSG_COMPACT_THREADS, KW = 4 * KQ;
    const int64_t stride = compact_row_stride(ts.num_samples);
    const uint32_t *bits = w.c_bits + (int64_t) s * stride * KW;
    const uint64_t *pre = w.c_rowpre + (int64_t) s * stride * KQ;
    const int2 *ep = ts.c_ep + ts.c_ep_off[s];
    const int64_t nep = ts.c_ep_off[s + 1] - ts.c_ep_off[s];
    const int tid = threadIdx.x;
    for (int64_t j0 = 0; j0 < nep; j0 += T) {
        const int64_t j = j0 + tid;
        const bool act = j < nep;
        int2 e = make_int2(0, 0);
        uint64_t p[KQ];
#pragma unroll
        for (int h = 0; h < KQ; h++) {
            p[h] = 0;
        }
        if (act) {
            e = ep[j];
            const int64_t row = e.x >> 5;
            const uint32_t below = (1u << (e.x & 31)) - 1u;
#pragma unroll
            for (int h = 0; h < KQ; h++) {
                p[h] = pre[row * KQ + h];
            }
            if (below != 0) {
#pragma unroll
                for (int h = 0; h < KQ; h++) {
                    const uint4 b = *(const uint4 *) (bits + row * KW + 4 * h);
                    p[h] += (uint64_t) __popc(b.x & below) + ((uint64_t) __popc(b.y & below) << 16)
                        + ((uint64_t) __popc(b.z & below) << 32)
                        + ((uint64_t) __popc(b.w & below) << 48);
                }
            }
        }
        const int64_t l = e.y >> 1;
        if (act && !(e.y & 1)) {
#pragma unroll
            for (int h = 0; h < KQ; h++) {
                sp.xq[l * KQ + h] = p[h];
            }
        }
        __syncthreads();
        if (act && (e.y & 1)) {
#pragma unroll
            for (int h = 0; h < KQ; h++) {
                sp.xq[l * KQ + h] = p[h] - sp.xq[l * KQ + h];
            }
        }
        __syncthreads();
    }
}

// Span s of the compact plan, by one block: the span-start parents and
// counts, then warp 0 replays the span's trees.  Ends with the block
// synchronised.
template <int KQ>
__device__ __forceinline__ void compact_span(const TSView &ts, const QueryParams &q,
    const QueryDev &qd, const WsDev &w, int s, unsigned char *smem_raw,
    TouchEntry<KQ> *s_list, ReplayStage *s_stage)
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
    compact_seek<KQ>(ts, w, s, sp);
    if (threadIdx.x < 32) {
        replay_span<16, KQ, uint16_t, false, true>(ts, q, qd, w, sp, s_list, s_stage, nullptr, t0,
            t1, Ls, ReplayEnc{ts.c_rem_enc, ts.c_ins_enc, ts.c_mut_enc});
    }
    __syncthreads();
}

// The block-shared arrays of the compact replay besides the span state.
template <int KQ>
struct CompactShared {
    TouchEntry<KQ> list[TSG_TOUCH_CAP];  // the open touch list
    ReplayStage stage[4];                // prefetch ring, trees t .. t + 3
};

// Persistent blocks take spans from the query's counter until none is left.
template <int KQ>
__global__ void __launch_bounds__(TSG_COMPACT_THREADS, 24) k_replay_compact(TSView ts, QueryParams q,
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
        compact_span<KQ>(ts, q, qd, w, s, smem_raw, sh.list, sh.stage);
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
