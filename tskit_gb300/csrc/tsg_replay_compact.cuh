// The compact replay: the item pipeline's replay over the compact span plan
// (tsg_cplan.cu).  One block of one warp (TSG_COMPACT_THREADS) per span at a
// time, the span's node state (16-bit counts packed in 64-bit words and
// 16-bit parent entries) in shared memory with a 64-entry touch list and a
// 16-entry staging ring: about 8 KB, so some thirty blocks -- thirty
// sequential replays -- run on every SM.
//
//   rows     (k_compact_rows, before the replay, every span at once) each
//            span's depth-first sample order in rows of 32 positions: per
//            row a membership word per set (ballots), the rows' counts
//            scanned per chunk of 64 rows, and at each of the span's range
//            endpoints the members before it within its chunk;
//   seek     at each of the span's sorted range endpoints P, that count plus
//            the totals of the chunks before, and a node's count P[hi] -
//            P[lo] (the start is stored first, the end then subtracts it);
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
// blocks an SM should hold at once (the register budget per thread follows:
// 64 with one count word per node, 80 with two)
#define TSG_COMPACT_MIN_BLOCKS(KQ) ((KQ) == 1 ? 32 : 24)

#define TSG_ROWS_THREADS 128
// rows whose sample masks a warp of k_compact_rows loads at once
#define TSG_ROWS_BATCH 8
// endpoints per lane a warp of k_compact_rows loads before its rows
#define TSG_ROWS_EPR 8

// A warp's shared arrays in k_compact_rows: its chunk's order entries, and
// per row the membership words (bit i: the row's i-th sample is in set k)
// and the packed counts of the chunk's rows before it (the entry after the
// last: the chunk's total).
template <int KQ>
struct __align__(16) RowsWarp {
    uint16_t ord[TSG_ROWS_PER_CHUNK * 32];
    uint4 word[TSG_ROWS_PER_CHUNK][KQ];
    uint64_t pre[TSG_ROWS_PER_CHUNK + 1][KQ];
};

// The members of every sample set before each compact span's range
// endpoints, a warp per (span, chunk of TSG_ROWS_PER_CHUNK rows of 32
// depth-first positions):
//   * the chunk's first TSG_ROWS_EPR x 32 endpoints are loaded, and its
//     order entries copied into shared memory (16 bytes a copy; each span's
//     order is padded to a multiple of 8 entries);
//   * a lane per position, TSG_ROWS_BATCH rows per round (their sample masks
//     loaded together): each set's membership bits of a row balloted into a
//     word, the row's 4 x KQ words stored by lane 0;
//   * a lane per two rows: their packed counts (population counts) and an
//     exclusive scan over the lanes give each row's count of the chunk's
//     members before it, and the chunk's total (w.c_ctot);
//   * a lane per endpoint: the count before its row plus the members of its
//     row below it, into w.c_pep (local to the chunk; the seek adds the
//     totals of the chunks before).
// Counts fit their 16-bit fields (at most the set sizes), so packed words
// add without carries.
template <int KQ>
__device__ __forceinline__ void compact_rows_body(const TSView &ts, const QueryParams &q,
    const QueryDev &qd, const WsDev &w, RowsWarp<KQ> *sh, const int64_t bid, const int64_t nb)
{
    static_assert(TSG_ROWS_PER_CHUNK == 64, "two rows per lane");
    constexpr int NW = TSG_ROWS_THREADS / 32, RB = TSG_ROWS_BATCH, EPR = TSG_ROWS_EPR;
    constexpr int CPR = TSG_ROWS_PER_CHUNK;
    const int64_t n = ts.num_samples;
    const int32_t nrows = (int32_t) ((n + 31) / 32);
    const int64_t CH = compact_row_chunks(n), nst = compact_order_stride(n);
    const int lane = threadIdx.x & 31;
    // the sets' bits of a sample mask (bits past the last set are clear)
    const uint32_t kmask = q.K >= 32 ? 0xFFFFFFFFu : (1u << q.K) - 1u;
    RowsWarp<KQ> &my = sh[threadIdx.x >> 5];
    const int64_t items = ts.c_num_spans * CH;
    for (int64_t it = bid * NW + (threadIdx.x >> 5); it < items; it += nb * NW) {
        const int64_t s = it / CH;
        const int32_t c = (int32_t) (it - s * CH);
        const int32_t rb = c * CPR;
        const int32_t nr = rb + CPR < nrows ? CPR : nrows - rb;
        const int2 *ep = ts.c_ep + ts.c_ep_off[s];
        uint64_t *pep = w.c_pep + ts.c_ep_off[s] * KQ;
        const int32_t *ec = ts.c_ep_chunk + s * (CH + 1);
        const int32_t ea = ec[c], eb = ec[c + 1];
        int2 epv[EPR];
#pragma unroll
        for (int u = 0; u < EPR; u++) {
            const int32_t j = ea + u * 32 + lane;
            epv[u] = j < eb ? ep[j] : make_int2(-1, 0);
        }
        {
            const uint16_t *order = ts.c_order + s * nst + rb * 32;
            const int32_t pend = (rb + nr) * 32 < (int32_t) nst ? (rb + nr) * 32 : (int32_t) nst;
            const int32_t pieces = (pend - rb * 32) / 8;
            for (int32_t k = lane; k < pieces; k += 32) {
                cp_async16(&my.ord[k * 8], order + k * 8);
            }
            cp_async_wait_all();
            __syncwarp();
        }
        for (int32_t l0 = 0; l0 < nr; l0 += RB) {
            uint32_t m[RB];
#pragma unroll
            for (int b = 0; b < RB; b++) {
                const int32_t i = (rb + l0 + b) * 32 + lane;
                m[b] = l0 + b < nr && i < n ? qd.sample_mask[my.ord[(l0 + b) * 32 + lane]] & kmask
                                            : 0u;
            }
#pragma unroll
            for (int b = 0; b < RB; b++) {
                const int32_t l = l0 + b;
                if (l >= nr) {
                    break;
                }
                uint32_t wd[4 * KQ];
#pragma unroll
                for (int k = 0; k < 4 * KQ; k++) {
                    wd[k] = __ballot_sync(0xffffffffu, (m[b] & (1u << k)) != 0u);
                }
                if (lane == 0) {
#pragma unroll
                    for (int h = 0; h < KQ; h++) {
                        my.word[l][h] = make_uint4(wd[4 * h], wd[4 * h + 1], wd[4 * h + 2],
                            wd[4 * h + 3]);
                    }
                }
            }
        }
        __syncwarp();
        // rows 2 lane and 2 lane + 1: packed counts, then the scan
        {
            uint64_t c0[KQ], c1[KQ];
#pragma unroll
            for (int h = 0; h < KQ; h++) {
                c0[h] = 0;
                c1[h] = 0;
                if (2 * lane < nr) {
                    const uint4 a = my.word[2 * lane][h];
                    c0[h] = (uint64_t) __popc(a.x) + ((uint64_t) __popc(a.y) << 16)
                        + ((uint64_t) __popc(a.z) << 32) + ((uint64_t) __popc(a.w) << 48);
                }
                if (2 * lane + 1 < nr) {
                    const uint4 a = my.word[2 * lane + 1][h];
                    c1[h] = (uint64_t) __popc(a.x) + ((uint64_t) __popc(a.y) << 16)
                        + ((uint64_t) __popc(a.z) << 32) + ((uint64_t) __popc(a.w) << 48);
                }
                const uint64_t v = c0[h] + c1[h];
                uint64_t inc = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint64_t x = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) {
                        inc += x;
                    }
                }
                const uint64_t ex = inc - v;
                if (2 * lane < nr) {
                    my.pre[2 * lane][h] = ex;
                }
                if (2 * lane + 1 < nr) {
                    my.pre[2 * lane + 1][h] = ex + c0[h];
                }
                if (lane == 31) {
                    my.pre[nr][h] = inc;
                    w.c_ctot[(s * CH + c) * KQ + h] = inc;
                }
            }
        }
        __syncwarp();
        auto value = [&](int32_t j, int32_t x) {
            const int32_t l = (x >> 5) - rb;  // nr only for x = n, n a multiple of 32
            const uint32_t below = (1u << (x & 31)) - 1u;
#pragma unroll
            for (int h = 0; h < KQ; h++) {
                uint64_t p = my.pre[l][h];
                if (below != 0) {
                    const uint4 a = my.word[l][h];
                    p += (uint64_t) __popc(a.x & below) + ((uint64_t) __popc(a.y & below) << 16)
                        + ((uint64_t) __popc(a.z & below) << 32)
                        + ((uint64_t) __popc(a.w & below) << 48);
                }
                pep[(int64_t) j * KQ + h] = p;
            }
        };
#pragma unroll
        for (int u = 0; u < EPR; u++) {
            if (epv[u].x >= 0) {
                value(ea + u * 32 + lane, epv[u].x);
            }
        }
        for (int32_t j = ea + EPR * 32 + lane; j < eb; j += 32) {
            value(j, ep[j].x);
        }
        __syncwarp();
    }
}

template <int KQ>
__global__ void __launch_bounds__(TSG_ROWS_THREADS, 8) k_compact_rows(TSView ts, QueryParams q,
    QueryDev qd, WsDev w)
{
    __shared__ RowsWarp<KQ> sh[TSG_ROWS_THREADS / 32];
    compact_rows_body<KQ>(ts, q, qd, w, sh, blockIdx.x, gridDim.x);
}

// endpoints a thread of the seek takes at once
#define TSG_SEEK_EPL 4

// Counts of span s's compact nodes at the span start into sp.xq, from
// k_compact_rows' counts at the span's range endpoints plus the totals of
// the chunks before each endpoint's (an exclusive scan over the lanes, lane
// c holding chunk c's offset).  The endpoints, sorted, are taken
// TSG_COMPACT_THREADS x TSG_SEEK_EPL at a time (each thread's loads issued
// together); within such a group every start count is stored before any end
// subtracts its node's start, and a node's start never follows its end in
// the sorted order.  Ends with the block synchronised.
template <int KQ>
__device__ __forceinline__ void compact_seek(const TSView &ts, const WsDev &w, int s,
    const SpanState<uint16_t> &sp)
{
    static_assert(TSG_COMPACT_THREADS == 32, "the seek's chunk offsets live in one warp");
    constexpr int T = TSG_COMPACT_THREADS, EPL = TSG_SEEK_EPL;
    const int64_t n = ts.num_samples;
    const int64_t CH = compact_row_chunks(n);
    const int64_t e0 = ts.c_ep_off[s];
    const int2 *ep = ts.c_ep + e0;
    const uint64_t *pep = w.c_pep + e0 * KQ;
    const int64_t nep = ts.c_ep_off[s + 1] - e0;
    const int tid = threadIdx.x;
    uint64_t coff[KQ];
#pragma unroll
    for (int h = 0; h < KQ; h++) {
        const uint64_t v = tid < CH ? w.c_ctot[((int64_t) s * CH + tid) * KQ + h] : 0ull;
        uint64_t inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t a = __shfl_up_sync(0xffffffffu, inc, o);
            if (tid >= o) {
                inc += a;
            }
        }
        coff[h] = inc - v;
    }
    for (int64_t j0 = 0; j0 < nep; j0 += (int64_t) T * EPL) {
        int2 e[EPL];
        uint64_t p[EPL][KQ];
#pragma unroll
        for (int u = 0; u < EPL; u++) {
            const int64_t j = j0 + (int64_t) u * T + tid;
            e[u] = make_int2(-1, 0);
#pragma unroll
            for (int h = 0; h < KQ; h++) {
                p[u][h] = 0;
            }
            if (j < nep) {
                e[u] = ep[j];
#pragma unroll
                for (int h = 0; h < KQ; h++) {
                    p[u][h] = pep[j * KQ + h];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < EPL; u++) {
            const int src = e[u].x >= 0 ? (int) compact_chunk_of(e[u].x, n) : 0;
#pragma unroll
            for (int h = 0; h < KQ; h++) {
                p[u][h] += __shfl_sync(0xffffffffu, coff[h], src);
            }
        }
#pragma unroll
        for (int u = 0; u < EPL; u++) {
            if (e[u].x >= 0 && !(e[u].y & 1)) {
                const int64_t l = e[u].y >> 1;
#pragma unroll
                for (int h = 0; h < KQ; h++) {
                    sp.xq[l * KQ + h] = p[u][h];
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < EPL; u++) {
            if (e[u].x >= 0 && (e[u].y & 1)) {
                const int64_t l = e[u].y >> 1;
#pragma unroll
                for (int h = 0; h < KQ; h++) {
                    sp.xq[l * KQ + h] = p[u][h] - sp.xq[l * KQ + h];
                }
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
__global__ void __launch_bounds__(TSG_COMPACT_THREADS, TSG_COMPACT_MIN_BLOCKS(KQ)) k_replay_compact(TSView ts, QueryParams q,
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
