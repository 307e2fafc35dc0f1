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
//   k_span_windows  (one warp per span)
//       the running-sum change of each tree is the sum of its chunks; the
//       running sum of each tree relative to the span's first tree is the
//       prefix sum of those changes (FP64); windows accumulate sum * overlap
//       length; the span's total change goes to k_span_scan, which gives
//       every span its starting sum (FP64, fixed order).
//   k_leaf_areas / k_leaf_prefix / k_leaf_terms
//       the branches of leaves, per edge (below).
//   k_site_eval / k_site_windows
//       every site's summary from the integer counts under its mutations
//       (FP64, one thread per site), then per-window sums in a fixed order.

#pragma once

#include "tsg_fixed.cuh"
#include "tsg_replay.cuh"

namespace tsg {

// node -> sample-set membership bits for this query
__global__ void k_node_mask(TSView ts, QueryDev qd, uint32_t *node_mask)
{
    for (int64_t u = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; u < ts.num_nodes;
         u += (int64_t) gridDim.x * blockDim.x) {
        const int32_t si = ts.sample_index[u];
        node_mask[u] = si >= 0 ? qd.sample_mask[si] : 0u;
    }
}

template <int W, int KQ, typename IdxT>
__global__ void __launch_bounds__(512, 2) k_replay_items(TSView ts, QueryParams q, QueryDev qd,
    WsDev w, int64_t slot_bytes)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_span;
    __shared__ int s_scan[32];
    __shared__ TouchEntry<KQ> s_list[TSG_TOUCH_CAP];  // the open touch list
    const int64_t L = ts.max_local;
    constexpr uint32_t TSG_NO_PARENT = SpanState<IdxT>::NONE;
    SpanState<IdxT> sp = span_state_at<IdxT>(sizeof(IdxT) == 2
            ? smem_raw
            : (unsigned char *) w.state + (int64_t) blockIdx.x * slot_bytes,
        L, KQ);
    sp.cnt = w.seekcnt + (int64_t) blockIdx.x * L;
    // one bit per stateful node: touched since the touch list was opened
    uint32_t *touched = (uint32_t *) span_state_end(sp, L);
    const int K = q.K;
    const int lane = threadIdx.x & 31;
    Item<KQ> *items = (Item<KQ> *) w.items;

    for (;;) {
        if (threadIdx.x == 0) {
            s_span = atomicAdd(w.counter, 1);
        }
        __syncthreads();
        const int s = s_span;
        __syncthreads();
        if (s >= ts.num_spans) {
            break;
        }
        const int32_t t0 = ts.span_tree[s], t1 = ts.span_tree[s + 1];
        const int64_t lo = ts.span_local_off[s];
        const int32_t Ls = (int32_t) (ts.span_local_off[s + 1] - lo);
        const int32_t *l2g = ts.span_l2g + lo;
        const int64_t a0 = ts.span_alive_off[s], a1 = ts.span_alive_off[s + 1];
        sp.time = ts.span_time + lo;

        span_seek<W, KQ, IdxT>(ts, qd, w.err, sp, K, Ls, l2g, a0, a1);
        if (q.branch) {
            for (int32_t i = threadIdx.x; i < (Ls + 31) / 32; i += blockDim.x) {
                touched[i] = 0;
            }
        }

        // ---- first tree of the sequence: one item per stateful node alive
        // there, in alive-list order (leaves are accounted per edge,
        // k_leaf_areas); every later tree's sum follows from the items of
        // the transitions before it
        if (q.branch && s == 0) {
            int64_t nanchor = 0;
            for (int64_t base = a0; base < a1; base += blockDim.x) {
                const int64_t i = base + threadIdx.x;
                int2 pc = make_int2(0, -1);
                if (i < a1) {
                    pc = ts.span_alive_enc[i];
                }
                const bool mine = i < a1 && pc.y >= 0;
                // block-wide exclusive scan of the stateful flags
                const unsigned bal = __ballot_sync(0xffffffffu, mine);
                if (lane == 0) {
                    s_scan[threadIdx.x >> 5] = __popc(bal);
                }
                __syncthreads();
                int64_t before = 0, total = 0;
                for (int j = 0; j < (int) (blockDim.x >> 5); j++) {
                    before += j < (int) (threadIdx.x >> 5) ? s_scan[j] : 0;
                    total += s_scan[j];
                }
                __syncthreads();
                if (mine) {
                    const int64_t at = ts.tree_item_off[t0] + nanchor + before
                        + __popc(bal & ((1u << lane) - 1u));
                    if (at < ts.tree_item_off[t0 + 1]) {
                        item_put<KQ>(items + at, Pack{0, 0}, st_load(sp, pc.y), pc.y, -1, pc.x);
                    }
                }
                nanchor += total;
            }
            if (threadIdx.x == 0 && ts.tree_item_off[t0] + nanchor != ts.tree_item_off[t0 + 1]) {
                dev_error(w.err, DEV_ITEM_PLAN);
            }
        }

        // the first-tree items read the first tree's counts and the touch
        // bits must be clear: both before the replay starts
        __syncthreads();

        // ---- replay (warp 0).  A span replays the transitions into its
        // trees after the first and, for branch items, into the next span's
        // first tree.  Every stateful node a transition touches (an edge's
        // child, a node on a root path) gets one item: its state before the
        // first touch and after the transition.  The touch list holds at
        // most TSG_TOUCH_CAP nodes; a longer transition closes the list and
        // opens a new one (the span plan counts items the same way).
        if (threadIdx.x < 32) {
            int64_t cursor = 0;  // first item of the open list
            int64_t climit = 0;  // end of the transition's items in the plan
            int32_t nopen = 0;   // nodes in the open list
            auto close_list = [&]() {
                __syncwarp();
                for (int32_t i = lane; i < nopen; i += 32) {
                    const TouchEntry<KQ> en = s_list[i];
                    const uint32_t pu = sp.par[en.u];
                    if (cursor + i < climit) {
                        item_put<KQ>(items + cursor + i, item_pack<KQ>(en.x0),
                            st_load(sp, (int64_t) en.u), (int32_t) en.u, en.p0,
                            pu != TSG_NO_PARENT ? (int32_t) pu : -1);
                    }
                    atomicAnd(&touched[en.u >> 5], ~(1u << (en.u & 31)));
                }
                __syncwarp();
                cursor += nopen;
                nopen = 0;
            };
            // lanes with `active` set touch node u (distinct per lane) whose
            // counts and parent are still x0, p0.  A node is touched at most
            // once per edge event and every event ends with __syncwarp, so the
            // touch bits need no barrier here.
            auto touch = [&](bool active, uint32_t u, const Pack &x0, uint32_t p0) {
                bool fresh = active && !((touched[u >> 5] >> (u & 31)) & 1u);
                unsigned m = __ballot_sync(0xffffffffu, fresh);
                if (nopen + __popc(m) > TSG_TOUCH_CAP) {
                    close_list();
                    fresh = active;
                    m = __ballot_sync(0xffffffffu, fresh);
                }
                if (fresh) {
                    const int32_t at = nopen + __popc(m & ((1u << lane) - 1u));
                    TouchEntry<KQ> en;
                    en.x0[0] = x0.lo;
                    if (KQ > 1) {
                        en.x0[KQ > 1 ? 1 : 0] = x0.hi;
                    }
                    en.u = u;
                    en.p0 = p0 != TSG_NO_PARENT ? (int32_t) p0 : -1;
                    s_list[at] = en;
                    atomicOr(&touched[u >> 5], 1u << (u & 31));
                    if (cursor + at >= climit) {
                        dev_error(w.err, DEV_ITEM_PLAN);
                    }
                }
                nopen += __popc(m);
            };
            // one edge event; cm: membership bits of a leaf child (whose branch
            // is accounted per edge, k_leaf_areas)
            auto event = [&](int32_t p, int32_t c, int sign, uint32_t cm) {
                const Pack xc = c >= 0 ? st_load(sp, c) : pk_from_mask<W>(cm, K);
                if (c >= 0) {
                    if (q.branch) {
                        touch(lane == 0, (uint32_t) c, xc, (uint32_t) sp.par[c]);
                    }
                    sp.par[c] = sign > 0 ? (IdxT) p : (IdxT) TSG_NO_PARENT;
                }
                uint32_t v = (uint32_t) p;
                int32_t guard = 0;
                while (v != TSG_NO_PARENT) {
                    uint32_t mine = TSG_NO_PARENT;
#pragma unroll 1
                    for (int j = 0; j < 32 && v != TSG_NO_PARENT; j++) {
                        if (lane == j) {
                            mine = v;
                        }
                        v = sp.par[v];
                        if (++guard > Ls) {
                            dev_error(w.err, DEV_PATH_TOO_LONG);
                            v = TSG_NO_PARENT;
                        }
                    }
                    uint32_t up = __shfl_down_sync(0xffffffffu, mine, 1);
                    if (lane == 31) {
                        up = v;
                    }
                    const bool act = mine != TSG_NO_PARENT;
                    Pack xo{0, 0};
                    if (act) {
                        xo = st_load(sp, (int64_t) mine);
                    }
                    if (q.branch) {
                        touch(act, mine, xo, up);
                    }
                    if (act) {
                        Pack xn;
                        if (sign > 0) {
                            xn.lo = xo.lo + xc.lo;
                            xn.hi = xo.hi + xc.hi;
                        } else {
                            xn.lo = xo.lo - xc.lo;
                            xn.hi = xo.hi - xc.hi;
                        }
                        pk_store(sp, (int64_t) mine, xn);
                    }
                }
                __syncwarp();
            };
            const int32_t tend = q.branch && t1 < ts.num_trees ? t1 + 1 : t1;
            for (int32_t t = t0; t < tend; t++) {
                if (t > t0) {
                    cursor = ts.tree_item_off[t];
                    climit = ts.tree_item_off[t + 1];
                    const int32_t r0 = ts.tree_out[t], nr = ts.tree_out[t + 1] - r0;
                    const int32_t i0 = ts.tree_in[t], ni = ts.tree_in[t + 1] - i0;
                    for (int32_t base = 0; base < nr + ni; base += 32) {
                        // fetch up to 32 events of the transition at once
                        const int32_t j = base + lane;
                        int2 pc = make_int2(0, 0);
                        uint32_t cm = 0;
                        if (j < nr + ni) {
                            pc = j < nr ? ts.rem_enc[r0 + j] : ts.ins_enc[i0 + (j - nr)];
                            if (pc.y < 0) {
                                cm = qd.node_mask[-pc.y - 1];
                            }
                        }
                        const int32_t cnt = min(32, nr + ni - base);
                        for (int32_t e = 0; e < cnt; e++) {
                            const int32_t p = __shfl_sync(0xffffffffu, pc.x, e);
                            const int32_t c = __shfl_sync(0xffffffffu, pc.y, e);
                            const uint32_t m = __shfl_sync(0xffffffffu, cm, e);
                            event(p, c, base + e < nr ? -1 : +1, m);
                        }
                    }
                    if (q.branch) {
                        close_list();
                        if (cursor != ts.tree_item_off[t + 1]) {
                            dev_error(w.err, DEV_ITEM_PLAN);
                        }
                    }
                }
                if (q.site && t < t1) {
                    const int32_t m0 = ts.site_mut[ts.tree_sites[t]];
                    const int32_t m1 = ts.site_mut[ts.tree_sites[t + 1]];
                    for (int32_t m = m0 + lane; m < m1; m += 32) {
                        const int32_t enc = ts.mut_enc[m];
                        const Pack x = enc >= 0 ? st_load(sp, enc)
                                                : pk_from_mask<W>(qd.node_mask[-enc - 1], K);
                        w.mcnt[(int64_t) m * KQ] = x.lo;
                        if (KQ > 1) {
                            w.mcnt[(int64_t) m * KQ + (KQ > 1 ? 1 : 0)] = x.hi;
                        }
                    }
                    __syncwarp();
                }
            }
        }
        __syncthreads();
    }
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
__global__ void __launch_bounds__(256) k_leaf_areas(TSView ts, QueryParams q, QueryDev qd,
    WsDev w)
{
    const int NP = 1 << q.K;
    const int64_t block = (int64_t) q.Wn * NP * TSG_FX_LIMBS;
    unsigned long long *part = w.leaf_area, *plus = part + block, *minus = plus + block;
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < ts.num_edges;
         i += (int64_t) gridDim.x * blockDim.x) {
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

// One block per pattern: the running sum over windows of the difference
// array (each window's exact plus - minus rounded once, then an FP64 prefix
// in a fixed order: per-thread runs of windows, a block scan of the run
// totals) gives the branch length alive over each whole window; area = that
// x window length + the window's partial areas.  w.leaf_dbl: windows x
// patterns doubles.
__device__ __forceinline__ double fx_diff_value(const unsigned long long *a,
    const unsigned long long *b)
{
    long long run[TSG_FX_LIMBS + 2];
    for (int i = 0; i < TSG_FX_LIMBS; i++) {
        run[i] = (long long) a[i] - (long long) b[i];
    }
    run[TSG_FX_LIMBS] = run[TSG_FX_LIMBS + 1] = 0;
    for (int i = 0; i < TSG_FX_LIMBS + 1; i++) {
        const long long cy = run[i] >> 32;
        run[i] -= cy * (1ll << 32);
        run[i + 1] += cy;
    }
    double v = 0;
    for (int i = TSG_FX_LIMBS + 1; i >= 0; i--) {
        v = v * 4294967296.0 + (double) run[i];
    }
    return ldexp(v, -TSG_FX_FRAC);
}

__global__ void __launch_bounds__(256) k_leaf_prefix(QueryParams q, QueryDev qd, WsDev w)
{
    __shared__ double s_run[256];
    const int NP = 1 << q.K;
    const int pat = blockIdx.x;
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

// The leaves' window sums: sum over patterns of F_r(pattern) x A[w][pattern]
// (FP64), one thread per (window, term).
template <int W>
__global__ void __launch_bounds__(256) k_leaf_terms(QueryParams q, WsDev w)
{
    const int NP = 1 << q.K;
    const int64_t total = (int64_t) q.Wn * q.R;
    for (int64_t idx = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t) gridDim.x * blockDim.x) {
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

// Per span: running sums by prefix over trees, window accumulation.
__global__ void __launch_bounds__(256) k_span_windows(TSView ts, QueryParams q, QueryDev qd,
    WsDev w)
{
    const int lane = threadIdx.x & 31;
    const int64_t s = (int64_t) blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= ts.num_spans) {
        return;
    }
    const int R = q.R;
    const int32_t t0 = ts.span_tree[s], t1 = ts.span_tree[s + 1];
    const int32_t wlo = qd.span_wlo[s];
    const int64_t woff = qd.span_woff[s];
    const int64_t nwin = qd.span_woff[s + 1] - woff;
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
    // running sum relative to the span's first tree (the first span's first
    // tree carries the absolute sum)
    double cum = 0;
    int32_t wi = wlo;
    for (int32_t t = t0; t < t1; t++) {
        const double tl = ts.breakpoints[t], tr = ts.breakpoints[t + 1];
        if (lane < R && (t > t0 || s == 0)) {
            for (int64_t c = ts.tree_chunk_off[t]; c < ts.tree_chunk_off[t + 1]; c++) {
                cum += w.dD[c * R + lane];
            }
        }
        while (wi < q.Wn && win[wi] < tr) {
            const double a = tl > win[wi] ? tl : win[wi];
            const double b = tr < win[wi + 1] ? tr : win[wi + 1];
            const int64_t li = woff + (wi - wlo);
            if (lane < R) {
                w.B[li * R + lane] += cum * (b - a);
            }
            if (win[wi + 1] <= tr) {
                wi++;
            } else {
                break;
            }
        }
    }
    // the change into the next span's first tree completes the span's change
    if (lane < R) {
        if (t1 < ts.num_trees) {
            for (int64_t c = ts.tree_chunk_off[t1]; c < ts.tree_chunk_off[t1 + 1]; c++) {
                cum += w.dD[c * R + lane];
            }
        }
        w.D[s * R + lane] = cum;
    }
}

// Each site's summary, summed over its alleles (skipping the ancestral one
// when polarised), from the integer counts under its mutations.
template <int RMAX, int W, int KQ>
__global__ void __launch_bounds__(256) k_site_eval(TSView ts, QueryParams q, WsDev w)
{
    const int64_t site = blockIdx.x * (int64_t) blockDim.x + threadIdx.x;
    if (site >= ts.num_sites) {
        return;
    }
    const int R = q.R, K = q.K;
    const int32_t m0 = ts.site_mut[site], m1 = ts.site_mut[site + 1];
    int32_t A = 1;
    for (int32_t m = m0; m < m1; m++) {
        A = max(A, ts.mutation_allele[m] + 1);
    }
    double val[RMAX];
#pragma unroll
    for (int r = 0; r < RMAX; r++) {
        val[r] = 0;
    }
    for (int32_t a = q.polarised ? 1 : 0; a < A; a++) {
        // allele state: the set sizes for the ancestral allele, plus the counts
        // under mutations to a, minus those under mutations away from a
        // (c/tskit/trees.c:1525-1612), in integers
        constexpr int KM = 2 * (64 / W);
        int64_t st[KM];
#pragma unroll
        for (int k = 0; k < KM; k++) {
            st[k] = (a == 0 && k < K) ? (int64_t) q.set_size[k] : 0;
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
        double mx, mc;
        pk_means<double, W>(q, ps, mx, mc);
#pragma unroll
        for (int r = 0; r < RMAX; r++) {
            if (r < R) {
                val[r] += term_F<double, false, W>(q, r, ps, mx, mc);
            }
        }
    }
#pragma unroll
    for (int r = 0; r < RMAX; r++) {
        if (r < R) {
            w.site_val[site * R + r] = val[r];
        }
    }
}

// Per window and term: the sum of its sites' summaries, in site order split
// over the block's threads and reduced in a fixed tree order.
__global__ void __launch_bounds__(256) k_site_windows(QueryParams q, QueryDev qd, WsDev w)
{
    __shared__ double red[256];
    const int64_t wdx = blockIdx.x / q.R;
    const int r = (int) (blockIdx.x % q.R);
    const int64_t b = qd.win_site_lo[wdx], e = qd.win_site_lo[wdx + 1];
    const int64_t n = e - b;
    const int64_t chunk = (n + blockDim.x - 1) / blockDim.x;
    const int64_t cb = b + (int64_t) threadIdx.x * chunk;
    const int64_t ce = cb + chunk < e ? cb + chunk : e;
    double v = 0;
    for (int64_t i = cb; i < ce; i++) {
        v += w.site_val[i * q.R + r];
    }
    red[threadIdx.x] = v;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int) threadIdx.x < o) {
            red[threadIdx.x] += red[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        w.site_win[wdx * q.R + r] = red[0];
    }
}

}  // namespace tsg
