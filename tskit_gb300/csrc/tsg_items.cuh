// Item pipeline of the shared-memory sweep (included by tsg_stats.cu).
//
// The sweep is split so that the sequential part carries no floating point:
//
//   k_replay_items  (one CTA per span, state in shared memory, integer only)
//       seek: rebuild the tree at the span start (parallel); the first span
//       also emits one item per stateful node alive in the first tree (its
//       counts and branch length: the running sum of that tree is the sum of
//       their values).  Then warp 0 replays the edge removals and insertions
//       of the transitions into the span's later trees and into the next
//       span's first tree, in reference order, and emits one item per
//       stateful node each transition touches (an edge's child, a node on a
//       root path): counts and branch length before the transition's first
//       touch and after the transition.  It also records the counts under
//       every mutation at its site's tree.  Items land at positions fixed by
//       the span plan, grouped by tree.  The edge events of a transition are
//       fetched by all lanes at once before the sequential part.
//   k_eval_items    (one warp per chunk, fully parallel)
//       the value of every item for every summary term,
//         F(x1) * bl1 - F(x0) * bl0
//       summed per chunk of at most 256 items of one tree (FP32 or FP64 per
//       lane, FP64 across lanes).
//   k_span_windows  (one warp per window segment of consecutive trees)
//       the running-sum change of each tree is the sum of its chunks; the
//       running sum of each tree relative to the segment's start is the
//       prefix sum of those changes (FP64); windows accumulate sum * overlap
//       length; the segment's total change goes to k_span_scan, which gives
//       every segment its starting sum (FP64, fixed order).
//   k_leaf_areas / k_leaf_prefix / k_leaf_terms
//       the branches of leaves, per edge (below).
//   k_site_eval / k_site_windows
//       every site's summary from the integer counts under its mutations
//       (FP64, one thread per site), then per-window sums in a fixed order.

#pragma once

#include "tsg_fixed.cuh"
#include "tsg_replay_kernel.cuh"

namespace tsg {

// node -> sample-set membership bits for this query
__device__ __forceinline__ void node_mask_body(const TSView &ts, const QueryDev &qd, uint32_t *node_mask,
    const int64_t bid, const int64_t nb)
{
    for (int64_t u = bid * (int64_t) blockDim.x + threadIdx.x; u < ts.num_nodes;
         u += (int64_t) nb * blockDim.x) {
        const int32_t si = ts.sample_index[u];
        node_mask[u] = si >= 0 ? qd.sample_mask[si] : 0u;
    }
}

static __global__ void k_node_mask(TSView ts, QueryDev qd, uint32_t *node_mask)
{
    node_mask_body(ts, qd, node_mask, blockIdx.x, gridDim.x);
}

// Leaves (nodes that are never a parent) keep their sample-set bits and
// their branch is constant while their edge lives, so their part of the
// branch running sum needs no replay: per window w and membership pattern p
// the area A[w][p] = sum over leaf edges of pattern p of branch length x (the
// edge's overlap with w).  Per edge: the first and last windows it reaches
// get exact partial areas; the windows in between get its branch length in
// a difference array (added where they start, subtracted past their end),
// so that an edge costs at most four exact fixed-point adds
// (tsg_fixed.cuh) whatever its length.  Layout of w.leaf_area: partial,
// plus and minus arrays of windows x patterns counters each.
__device__ __forceinline__ void leaf_areas_body(const TSView &ts, const QueryParams &q, const QueryDev &qd, const WsDev &w,
    const int64_t bid, const int64_t nb)
{
    const int NP = 1 << q.K;
    const int64_t block = (int64_t) q.Wn * NP * TSG_FX_LIMBS;
    unsigned long long *part = w.leaf_area, *plus = part + block, *minus = plus + block;
    for (int64_t i = bid * (int64_t) blockDim.x + threadIdx.x; i < ts.num_edges;
         i += (int64_t) nb * blockDim.x) {
        const int32_t c = ts.ins_child[i];
        if (ts.node_is_parent[c]) {
            continue;
        }
        const uint32_t pat = qd.node_mask[c] & (uint32_t) (NP - 1);
        const double bl = ts.node_time[ts.ins_parent[i]] - ts.node_time[c];
        const double left = ts.ins_left[i], right = ts.ins_right[i];
        int w0 = (int) upper_bound(qd.windows, (int64_t) q.Wn + 1, left) - 1;
        int w1 = (int) lower_bound(qd.windows, (int64_t) q.Wn + 1, right) - 1;
        w0 = w0 < 0 ? 0 : (w0 >= q.Wn ? q.Wn - 1 : w0);
        w1 = w1 < w0 ? w0 : (w1 >= q.Wn ? q.Wn - 1 : w1);
        if (w0 == w1) {
            fx_add(part + ((int64_t) w0 * NP + pat) * TSG_FX_LIMBS, bl * (right - left), w.err);
            continue;
        }
        fx_add(part + ((int64_t) w0 * NP + pat) * TSG_FX_LIMBS,
            bl * (qd.windows[w0 + 1] - left), w.err);
        fx_add(part + ((int64_t) w1 * NP + pat) * TSG_FX_LIMBS, bl * (right - qd.windows[w1]),
            w.err);
        if (w1 > w0 + 1) {
            fx_add(plus + ((int64_t) (w0 + 1) * NP + pat) * TSG_FX_LIMBS, bl, w.err);
            fx_add(minus + ((int64_t) w1 * NP + pat) * TSG_FX_LIMBS, bl, w.err);
        }
    }
}

static __global__ void __launch_bounds__(256) k_leaf_areas(TSView ts, QueryParams q, QueryDev qd,
    WsDev w)
{
    leaf_areas_body(ts, q, qd, w, blockIdx.x, gridDim.x);
}

// One block per pattern: the running sum over windows of the difference
// array (each window's exact plus - minus rounded once, then an FP64 prefix
// in a fixed order: per-thread runs of windows, a block scan of the run
// totals) gives the branch length alive over each whole window; area = that
// x window length + the window's partial areas.  w.leaf_dbl: windows x
// patterns doubles.
__device__ __forceinline__ void leaf_prefix_body(const QueryParams &q, const QueryDev &qd, const WsDev &w,
    const int64_t bid, const int64_t nb)
{
    __shared__ double s_run[256];
    const int NP = 1 << q.K;
    const int pat = bid;
    const int64_t block = (int64_t) q.Wn * NP * TSG_FX_LIMBS;
    const unsigned long long *part = w.leaf_area, *plus = part + block, *minus = plus + block;
    const int per = (q.Wn + blockDim.x - 1) / blockDim.x;
    const int w0 = threadIdx.x * per, w1 = min(q.Wn, w0 + per);
    double run = 0;
    for (int wi = w0; wi < w1; wi++) {
        const int64_t o = ((int64_t) wi * NP + pat) * TSG_FX_LIMBS;
        run += fx_diff_value(plus + o, minus + o);
    }
    s_run[threadIdx.x] = run;
    __syncthreads();
    if (threadIdx.x == 0) {
        double acc = 0;
        for (int j = 0; j < (int) blockDim.x; j++) {
            const double v = s_run[j];
            s_run[j] = acc;
            acc += v;
        }
    }
    __syncthreads();
    double active = s_run[threadIdx.x];
    for (int wi = w0; wi < w1; wi++) {
        const int64_t o = ((int64_t) wi * NP + pat) * TSG_FX_LIMBS;
        active += fx_diff_value(plus + o, minus + o);
        w.leaf_dbl[(int64_t) wi * NP + pat] =
            active * (qd.windows[wi + 1] - qd.windows[wi]) + fx_value(part + o);
    }
}

static __global__ void __launch_bounds__(256) k_leaf_prefix(QueryParams q, QueryDev qd, WsDev w)
{
    leaf_prefix_body(q, qd, w, blockIdx.x, gridDim.x);
}

// The leaves' window sums: sum over patterns of F_r(pattern) x A[w][pattern]
// (FP64), one thread per (window, term).
template <int W>
__device__ __forceinline__ void leaf_terms_body(const QueryParams &q, const WsDev &w,
    const int64_t bid, const int64_t nb)
{
    const int NP = 1 << q.K;
    const int64_t total = (int64_t) q.Wn * q.R;
    for (int64_t idx = bid * (int64_t) blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t) nb * blockDim.x) {
        const int64_t wi = idx / q.R;
        const int r = (int) (idx % q.R);
        double v = 0;
        for (int pat = 0; pat < NP; pat++) {
            const double area = w.leaf_dbl[wi * NP + pat];
            if (area != 0.0) {
                const Pack x = pk_from_mask<W>((uint32_t) pat, q.K);
                double mx, mc;
                pk_means<double, W>(q, x, mx, mc);
                const double f = q.polarised ? term_F<double, false, W>(q, r, x, mx, mc)
                                             : term_F<double, true, W>(q, r, x, mx, mc);
                v += f * area;
            }
        }
        w.leaf_win[idx] = v;
    }
}

template <int W>
__global__ void __launch_bounds__(256) k_leaf_terms(QueryParams q, WsDev w)
{
    leaf_terms_body<W>(q, w, blockIdx.x, gridDim.x);
}

// Windows of the branch running sum, one warp per window segment (a run of
// consecutive trees), lane r for term r: the running sum's change into each
// tree is the sum of its chunks (the first tree's is the sum itself); the
// segment's running sum relative to its start is the prefix of those
// changes (FP64); windows accumulate it times each tree's overlap (B) and
// the segment's overlap (A); the segment's total change (D) goes to
// k_span_scan, which gives every segment its starting sum in a fixed order.
__device__ __forceinline__ void span_windows_body(const TSView &ts, const QueryParams &q, const QueryDev &qd, const WsDev &w,
    const int64_t bid, const int64_t nb)
{
    const int lane = threadIdx.x & 31;
    const int64_t u = (int64_t) bid * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (u >= ts.num_segs) {
        return;
    }
    const int R = q.R;
    const int32_t t0 = ts.seg_tree[u], t1 = ts.seg_tree[u + 1];
    const int32_t wlo = qd.seg_wlo[u];
    const int64_t woff = qd.seg_woff[u];
    const int64_t nwin = qd.seg_woff[u + 1] - woff;
    const double *win = qd.windows;
    const double slo = ts.breakpoints[t0], shi = ts.breakpoints[t1];
    for (int64_t j = lane; j < nwin * R; j += 32) {
        w.B[woff * R + j] = 0;
    }
    for (int64_t j = lane; j < nwin; j += 32) {
        const double a = slo > win[wlo + j] ? slo : win[wlo + j];
        const double b = shi < win[wlo + j + 1] ? shi : win[wlo + j + 1];
        w.A[woff + j] = b - a;
    }
    __syncwarp();
    // the running sum and the open window's sum stay in registers (the
    // window's sum is stored once, when the window closes); trees are taken
    // four at a time, their chunk ranges, right ends and first chunk
    // changes loaded together (two round trips per four trees).  Genome
    // positions (never negative) are compared as the integers of their bits
    // (the same order), keeping the FP64 pipe -- a warp instruction every 16
    // cycles -- for the three sums per tree.
    auto key = [](double x) { return __double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFLL; };
    double cum = 0, bacc = 0;
    bool open = false;
    int32_t wi = wlo;
    double tl = slo;
    long long ktl = key(tl);
    double w_lo = win[wi], w_hi = win[wi + 1];
    long long kwlo = key(w_lo), kwhi = key(w_hi);
    for (int32_t tg = t0; tg < t1; tg += 4) {
        const int ng = t1 - tg < 4 ? t1 - tg : 4;
        int64_t co[5];
        double tr[4], fi[4], tn[4];
#pragma unroll
        for (int j = 0; j < 5; j++) {
            co[j] = ts.tree_chunk_off[tg + j < t1 ? tg + j : t1];
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            tr[j] = ts.breakpoints[tg + j + 1 < t1 ? tg + j + 1 : t1];
            tn[j] = ts.tree_len[tg + j < t1 ? tg + j : t1 - 1];
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            fi[j] = (lane < R && j < ng && co[j] < co[j + 1]) ? w.dD[co[j] * R + lane] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (j < ng) {
                const double trj = tr[j];
                const long long ktr = key(trj);
                if (lane < R && co[j] < co[j + 1]) {
                    cum += fi[j];
                    for (int64_t c = co[j] + 1; c < co[j + 1]; c++) {
                        cum += w.dD[c * R + lane];
                    }
                }
                if (wi < q.Wn && ktl >= kwlo && ktr < kwhi) {
                    // the tree lies inside the open window, which stays
                    // open: its length is the difference of its ends
                    // (bitwise), one FP64 operation fewer on GB300's slow
                    // FP64 pipe
                    bacc += cum * tn[j];
                    open = true;
                } else {
                    while (wi < q.Wn && kwlo < ktr) {
                        const double a = ktl > kwlo ? tl : w_lo;
                        const double b = ktr < kwhi ? trj : w_hi;
                        bacc += cum * (b - a);
                        open = true;
                        if (kwhi <= ktr) {
                            if (lane < R) {
                                w.B[(woff + (wi - wlo)) * R + lane] = bacc;
                            }
                            bacc = 0;
                            open = false;
                            wi++;
                            if (wi < q.Wn) {
                                w_lo = w_hi;
                                kwlo = kwhi;
                                w_hi = win[wi + 1];
                                kwhi = key(w_hi);
                            }
                        } else {
                            break;
                        }
                    }
                }
                tl = trj;
                ktl = ktr;
            }
        }
    }
    if (open && lane < R) {
        w.B[(woff + (wi - wlo)) * R + lane] = bacc;
    }
    if (lane < R) {
        w.D[u * R + lane] = cum;
    }
}

static __global__ void __launch_bounds__(128, 7) k_span_windows(TSView ts, QueryParams q, QueryDev qd,
    WsDev w)
{
    span_windows_body(ts, q, qd, w, blockIdx.x, gridDim.x);
}

// Each site's summary, summed over its alleles (skipping the ancestral one
// when polarised), from the integer counts under its mutations: one thread
// per site; the allele states (get_allele_weights, c/tskit/trees.c:1525-1612,
// in integers) of up to four alleles are kept in registers and the terms are
// valued one at a time (exact integer numerators when q.site_int, else FP64).
template <int W, int KQ>
__device__ __forceinline__ Pack site_allele_state(const TSView &ts, const QueryParams &q,
    const WsDev &w, int32_t m0, int32_t m1, int32_t a)
{
    constexpr int KM = 2 * (64 / W);
    int64_t st[KM];
#pragma unroll
    for (int k = 0; k < KM; k++) {
        st[k] = (a == 0 && k < q.K) ? (int64_t) q.set_size_i[k] : 0;
    }
    for (int32_t m = m0; m < m1; m++) {
        Pack xm;
        xm.lo = w.mcnt[(int64_t) m * KQ];
        xm.hi = KQ > 1 ? w.mcnt[(int64_t) m * KQ + (KQ > 1 ? 1 : 0)] : 0ull;
        const int al = ts.mutation_allele[m], alt = ts.mutation_alt[m];
#pragma unroll
        for (int k = 0; k < KM; k++) {
            const int64_t v = (int64_t) pk_get<W>(xm, k);
            st[k] += (al == a ? v : 0) - (alt == a ? v : 0);
        }
    }
    Pack ps{0, 0};
#pragma unroll
    for (int k = 0; k < KM; k++) {
        pk_set<W>(ps, k, (uint64_t) st[k] & ((1ull << W) - 1ull));
    }
    return ps;
}

template <int W>
__device__ __forceinline__ double site_term(const QueryParams &q, int r, const Pack &ps)
{
    if (q.site_int) {
        const Term &t = q.term[r];
        int64_t num;
        term_num(t.type, (int64_t) pk_get<W>(ps, t.idx[0]), (int64_t) pk_get<W>(ps, t.idx[1]),
            (int64_t) pk_get<W>(ps, t.idx[2]), (int64_t) pk_get<W>(ps, t.idx[3]),
            (int64_t) q.set_size[t.idx[0]], (int64_t) q.set_size[t.idx[1]],
            (int64_t) q.set_size[t.idx[2]], (int64_t) q.set_size[t.idx[3]], num);
        return (double) num * q.inv[r];
    }
    double mx, mc;
    pk_means<double, W>(q, ps, mx, mc);
    return term_F<double, false, W>(q, r, ps, mx, mc);
}

template <int RMAX, int W, int KQ>
__global__ void __launch_bounds__(256) k_site_eval(TSView ts, QueryParams q, WsDev w)
{
    const int64_t site = blockIdx.x * (int64_t) blockDim.x + threadIdx.x;
    if (site >= ts.num_sites) {
        return;
    }
    const int R = q.R;
    const int32_t m0 = ts.site_mut[site], m1 = ts.site_mut[site + 1];
    int32_t A = 1;
    for (int32_t m = m0; m < m1; m++) {
        A = max(A, ts.mutation_allele[m] + 1);
    }
    const int32_t a0 = q.polarised ? 1 : 0;
    const int32_t na = A - a0;
    if (q.site_int) {
        // exact integer numerators summed over the alleles (each below
        // 2^60 with set sizes below 2^15): the windows sum them exactly and
        // scale once (k_site_windows), no FP64 work per site; the states of
        // up to four alleles stay in registers
        Pack ps[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            ps[j] = j < na && na <= 4 ? site_allele_state<W, KQ>(ts, q, w, m0, m1, a0 + j)
                                      : Pack{0, 0};
        }
        int64_t *num_out = (int64_t *) w.site_val;
#pragma unroll 1
        for (int r = 0; r < R; r++) {
            const Term &t = q.term[r];
            auto numer = [&](const Pack &x) {
                int64_t num;
                term_num(t.type, (int64_t) pk_get<W>(x, t.idx[0]), (int64_t) pk_get<W>(x, t.idx[1]),
                    (int64_t) pk_get<W>(x, t.idx[2]), (int64_t) pk_get<W>(x, t.idx[3]),
                    (int64_t) q.set_size_i[t.idx[0]], (int64_t) q.set_size_i[t.idx[1]],
                    (int64_t) q.set_size_i[t.idx[2]], (int64_t) q.set_size_i[t.idx[3]], num);
                return num;
            };
            int64_t acc = 0;
            if (na <= 4) {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    if (j < na) {
                        acc += numer(ps[j]);
                    }
                }
            } else {
                for (int32_t a = a0; a < A; a++) {
                    acc += numer(site_allele_state<W, KQ>(ts, q, w, m0, m1, a));
                }
            }
            num_out[(int64_t) r * ts.num_sites + site] = acc;
        }
        return;
    }
    if (na <= 4) {
        Pack ps[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            ps[j] = j < na ? site_allele_state<W, KQ>(ts, q, w, m0, m1, a0 + j) : Pack{0, 0};
        }
#pragma unroll 1
        for (int r = 0; r < R; r++) {
            double v = 0;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (j < na) {
                    v += site_term<W>(q, r, ps[j]);
                }
            }
            w.site_val[(int64_t) r * ts.num_sites + site] = v;
        }
        return;
    }
#pragma unroll 1
    for (int r = 0; r < R; r++) {
        double v = 0;
        for (int32_t a = a0; a < A; a++) {
            v += site_term<W>(q, r, site_allele_state<W, KQ>(ts, q, w, m0, m1, a));
        }
        w.site_val[(int64_t) r * ts.num_sites + site] = v;
    }
}

// Exact sum of 128-bit integers across a warp (lane 0 holds it).
__device__ __forceinline__ __int128 warp_sum_i128(__int128 v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long lo = __shfl_down_sync(0xffffffffu, (unsigned long long) v, o);
        const unsigned long long hi =
            __shfl_down_sync(0xffffffffu, (unsigned long long) (v >> 64), o);
        v += (__int128) (((unsigned __int128) hi << 64) | (unsigned __int128) lo);
    }
    return v;
}

// A 128-bit integer as the nearest double (one rounding while it fits 64
// bits; two beyond).
__device__ __forceinline__ double i128_to_double(__int128 v)
{
    const long long lo = (long long) v;
    if ((__int128) lo == v) {
        return (double) lo;
    }
    return (double) (long long) (v >> 64) * 18446744073709551616.0
        + (double) (unsigned long long) v;
}

// Exact per-window sums of the sites' integer numerators in one pass (the
// integer form of k_site_eval + k_site_windows, without the per-site array):
// a thread per site forms its allele states and each term's numerator
// summed over its alleles; a warp whose sites all lie in one window adds its
// exact 128-bit total, else every lane its own, into the window's counter
// pair (low 32 bits unsigned, the rest signed: the 64-bit atomic adds never
// carry, so their order does not matter and the sums are exact).
template <int W, int KQ>
__device__ __forceinline__ void site_sums_body(const TSView &ts, const QueryParams &q, const QueryDev &qd, const WsDev &w,
    const int64_t bid, const int64_t nb)
{
    const int64_t site = bid * (int64_t) blockDim.x + threadIdx.x;
    const bool valid = site < ts.num_sites;
    const int R = q.R;
    int32_t m0 = 0, m1 = 0, A = 1;
    int64_t wdx = 0;
    if (valid) {
        m0 = ts.site_mut[site];
        m1 = ts.site_mut[site + 1];
        for (int32_t m = m0; m < m1; m++) {
            A = max(A, ts.mutation_allele[m] + 1);
        }
        wdx = upper_bound(qd.win_site_lo, (int64_t) q.Wn + 1, (int32_t) site) - 1;
    }
    const int32_t a0 = q.polarised ? 1 : 0;
    const int32_t na = valid ? A - a0 : 0;
    const int64_t w_first = __shfl_sync(0xffffffffu, wdx, 0);
    const bool one_window = __all_sync(0xffffffffu, !valid || wdx == w_first)
        && __shfl_sync(0xffffffffu, (int) valid, 0);
    Pack ps[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        ps[j] = j < na && na <= 4 ? site_allele_state<W, KQ>(ts, q, w, m0, m1, a0 + j) : Pack{0, 0};
    }
    unsigned long long *acc = (unsigned long long *) w.site_acc;
#pragma unroll 1
    for (int r = 0; r < R; r++) {
        const Term &t = q.term[r];
        auto numer = [&](const Pack &x) {
            int64_t num;
            term_num(t.type, (int64_t) pk_get<W>(x, t.idx[0]), (int64_t) pk_get<W>(x, t.idx[1]),
                (int64_t) pk_get<W>(x, t.idx[2]), (int64_t) pk_get<W>(x, t.idx[3]),
                (int64_t) q.set_size_i[t.idx[0]], (int64_t) q.set_size_i[t.idx[1]],
                (int64_t) q.set_size_i[t.idx[2]], (int64_t) q.set_size_i[t.idx[3]], num);
            return num;
        };
        __int128 v = 0;
        if (na <= 4) {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (j < na) {
                    v += numer(ps[j]);
                }
            }
        } else {
            for (int32_t a = a0; a < A; a++) {
                v += numer(site_allele_state<W, KQ>(ts, q, w, m0, m1, a));
            }
        }
        auto add = [&](int64_t wi, __int128 x) {
            unsigned long long *c = acc + 2 * (wi * R + r);
            const unsigned long long lo = (unsigned long long) x & 0xFFFFFFFFull;
            const long long hi = (long long) (x >> 32);
            if (lo) {
                atomicAdd(c, lo);
            }
            if (hi) {
                atomicAdd(c + 1, (unsigned long long) hi);
            }
        };
        if (one_window) {
            v = warp_sum_i128(v);
            if ((threadIdx.x & 31) == 0) {
                add(w_first, v);
            }
        } else if (valid) {
            add(wdx, v);
        }
    }
}

template <int W, int KQ>
__global__ void __launch_bounds__(256) k_site_sums(TSView ts, QueryParams q, QueryDev qd, WsDev w)
{
    site_sums_body<W, KQ>(ts, q, qd, w, blockIdx.x, gridDim.x);
}

// The window sums of k_site_sums, each rounded once and scaled by the
// term's reciprocal denominator.
__device__ __forceinline__ void site_sums_finish_body(const QueryParams &q, const WsDev &w,
    const int64_t bid, const int64_t nb)
{
    const int64_t total = (int64_t) q.Wn * q.R;
    for (int64_t i = bid * (int64_t) blockDim.x + threadIdx.x; i < total;
         i += (int64_t) nb * blockDim.x) {
        const unsigned long long lo = w.site_acc[2 * i];
        const long long hi = (long long) w.site_acc[2 * i + 1];
        const __int128 v = ((__int128) hi << 32) + (__int128) lo;
        w.site_win[i] = i128_to_double(v) * q.inv[i % q.R];
    }
}

static __global__ void k_site_sums_finish(QueryParams q, WsDev w)
{
    site_sums_finish_body(q, w, blockIdx.x, gridDim.x);
}

// Per window: the sum of its sites' summaries for every term, one block of
// 32 warps per window, warp j taking terms j, j + 32, ...: lanes sum strided
// sites (term-major, coalesced), then a fixed-order warp reduction; with
// integer numerators the sums are exact (128-bit) and scaled once.
static __global__ void __launch_bounds__(1024) k_site_windows(QueryParams q, QueryDev qd, WsDev w,
    int64_t S, int integer)
{
    const int64_t wdx = blockIdx.x;
    const int lane = threadIdx.x & 31;
    const int64_t b = qd.win_site_lo[wdx], e = qd.win_site_lo[wdx + 1];
    if (integer) {
        // integer numerators (k_site_eval): summed exactly, scaled once
        for (int r = threadIdx.x >> 5; r < q.R; r += blockDim.x >> 5) {
            const int64_t *num = (const int64_t *) w.site_val + (int64_t) r * S;
            __int128 v = 0;
            for (int64_t i = b + lane; i < e; i += 32) {
                v += num[i];
            }
            v = warp_sum_i128(v);
            if (lane == 0) {
                w.site_win[wdx * q.R + r] = i128_to_double(v) * q.inv[r];
            }
        }
        return;
    }
    for (int r = threadIdx.x >> 5; r < q.R; r += blockDim.x >> 5) {
        const double *val = w.site_val + (int64_t) r * S;
        double v = 0;
        for (int64_t i = b + lane; i < e; i += 32) {
            v += val[i];
        }
        v = warp_sum(v);
        if (lane == 0) {
            w.site_win[wdx * q.R + r] = v;
        }
    }
}

// values a thread of the span scan loads at once
#define TSG_SCAN_U 8

// RS[s][r] = rs0[r] + sum_{s' < s} D[s'][r]: one block per r, each thread a
// contiguous run of units, then a scan of the run totals across the block
// (warp shuffles, then the warp totals in shared memory); fixed order.
__device__ __forceinline__ void span_scan_body(const double *D, const double *rs0, double *RS, int64_t NS, int R,
    const int64_t bid, const int64_t nb)
{
    __shared__ double s_warp[16];
    const int r = bid;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t run = (NS + blockDim.x - 1) / blockDim.x;
    const int64_t b = (int64_t) threadIdx.x * run < NS ? (int64_t) threadIdx.x * run : NS;
    const int64_t e = b + run < NS ? b + run : NS;
    // a thread's values are loaded TSG_SCAN_U at a time (independent loads)
    // and added in order; with at most TSG_SCAN_U they stay in registers for
    // the second pass
    constexpr int U = TSG_SCAN_U;
    double v[U];
    double sum = 0;
    for (int64_t i0 = b; i0 < e; i0 += U) {
#pragma unroll
        for (int u = 0; u < U; u++) {
            v[u] = i0 + u < e ? D[(i0 + u) * R + r] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (i0 + u < e) {
                sum += v[u];
            }
        }
    }
    double incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) {
            incl += y;
        }
    }
    double excl = __shfl_up_sync(0xffffffffu, incl, 1);
    excl = lane > 0 ? excl : 0.0;
    if (lane == 31) {
        s_warp[wid] = incl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double acc = rs0[r];
        for (int j = 0; j < (int) (blockDim.x >> 5); j++) {
            const double v = s_warp[j];
            s_warp[j] = acc;
            acc += v;
        }
    }
    __syncthreads();
    double acc = s_warp[wid] + excl;
    for (int64_t i0 = b; i0 < e; i0 += U) {
        if (e - b > U) {
#pragma unroll
            for (int u = 0; u < U; u++) {
                v[u] = i0 + u < e ? D[(i0 + u) * R + r] : 0.0;
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (i0 + u < e) {
                RS[(i0 + u) * R + r] = acc;
                acc += v[u];
            }
        }
    }
}

static __global__ void __launch_bounds__(512) k_span_scan(const double *D, const double *rs0, double *RS,
    int64_t NS, int R)
{
    span_scan_body(D, rs0, RS, NS, R, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void window_reduce_body(const QueryParams &q, const QueryDev &qd, const WsDev &w, int span_normalise, int items_mode, double *result,
    const int64_t bid, const int64_t nb)
{
    const int R = q.R;
    const int64_t total = (int64_t) q.Wn * R;
    for (int64_t idx = bid * (int64_t) blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t) nb * blockDim.x) {
        const int wdx = (int) (idx / R), r = (int) (idx % R);
        // units: window segments (item pipeline) or spans (general sweep)
        const int32_t *uwlo = items_mode ? qd.seg_wlo : qd.span_wlo;
        const int64_t *uwoff = items_mode ? qd.seg_woff : qd.span_woff;
        const int32_t s0 = items_mode ? qd.win_seg_lo[wdx] : qd.win_span_lo[wdx];
        const int32_t s1 = items_mode ? qd.win_seg_hi[wdx] : qd.win_span_hi[wdx];
        double vb = 0, vs = 0;
        for (int32_t s = s0; s <= s1; s++) {
            int64_t li = uwoff[s] + (wdx - uwlo[s]);
            if (q.branch) {
                vb += w.RS[(int64_t) s * R + r] * w.A[li] + w.B[li * R + r];
            }
            if (q.site && !items_mode) {
                vs += w.SITE[li * R + r];
            }
        }
        if (q.site && items_mode) {
            vs = w.site_win[(int64_t) wdx * R + r];
        }
        if (q.branch && items_mode && w.leaf_win != nullptr) {
            vb += w.leaf_win[(int64_t) wdx * R + r];
        }
        double span = qd.windows[wdx + 1] - qd.windows[wdx];
        if (span_normalise) {
            vb /= span;
            vs /= span;
        }
        int64_t o = 0;
        if (q.branch) {
            result[idx] = vb;
            o = total;
        }
        if (q.site) {
            result[o + idx] = vs;
        }
    }
}

static __global__ void k_window_reduce(QueryParams q, QueryDev qd, WsDev w, int span_normalise,
    int items_mode, double *result)
{
    window_reduce_body(q, qd, w, span_normalise, items_mode, result, blockIdx.x, gridDim.x);
}

}  // namespace tsg
