// The item replay kernel (see tsg_items.cuh for the pipeline).  With EVAL
// other warps value the span's items while the replay proceeds: warp 0
// publishes its completed trees in shared memory and the evaluating warps
// take the span's evaluation chunks in order, each once the replay has
// completed its tree (a bounded wait), so the evaluation runs in the shadow
// of the sequential replay.  The warps that would share warp 0's scheduler
// (warp index a multiple of 4, as warps are dealt to the SM's four
// schedulers) stay idle, leaving the replay its issue slots.  Included by tsg_stats.cu (EVAL off)
// and by the evaluation translation units (EVAL on).
#pragma once

#include "tsg_eval.cuh"

namespace tsg {

// bound of an evaluating warp's wait for one tree (with 128 ns sleeps: far
// longer than any span's replay); past it the kernel records an error
#define TSG_REPLAY_SPIN_LIMIT (1u << 27)
// the replay publishes its progress every few trees (a fence each time)
#define TSG_PUBLISH_EVERY 8

// The edge events of the transitions a span replays, and its mutations, in
// the span's node encoding (local ids of stateful nodes, -(global + 1) of
// leaves): the general plan's or the compact plan's.
struct ReplayEnc {
    const int2 *rem;
    const int2 *ins;
    const int32_t *mut;
};

// The sequential replay of one span by warp 0 of the block, integer only,
// in reference order (c/tskit/trees.c:1424-1507), from the state at the span
// start in `sp` (parents in the replay's encoding): the transitions into the
// span's trees after the first and, for branch items, into the next span's
// first tree; one item per stateful node a transition touches (its counts
// and parent before the first touch and after the transition); the counts
// under every mutation of the span's trees for site statistics.  With EVAL
// the replay publishes its completed trees in *s_ready every few trees.
template <int W, int KQ, typename IdxT, bool EVAL, bool BLS = false>
__device__ __forceinline__ void replay_span(const TSView &ts, const QueryParams &q,
    const QueryDev &qd, const WsDev &w, const SpanState<IdxT> &sp, TouchEntry<KQ> *s_list,
    ReplayStage *s_stage, int *s_ready, int32_t t0, int32_t t1, int32_t Ls, const ReplayEnc code)
{
    constexpr uint32_t PFLAG = sizeof(IdxT) == 2 ? 0x8000u : 0x80000000u;
    constexpr uint32_t PMASK = PFLAG - 1u;
    constexpr uint32_t TSG_NO_PARENT = PMASK;
    constexpr uint32_t NO_NODE = 0xffffffffu;
    const int K = q.K;
    const int lane = threadIdx.x & 31;
    Item<KQ> *items = (Item<KQ> *) w.items;
    int64_t cursor = 0;  // first item of the open list
    int64_t climit = 0;  // end of the transition's items in the plan
    int32_t nopen = 0;   // nodes in the open list
    auto close_list = [&]() {
        __syncwarp();
        for (int32_t i = lane; i < nopen; i += 32) {
            const TouchEntry<KQ> en = s_list[i];
            const uint32_t pu = (uint32_t) sp.par[en.u] & PMASK;
            if (cursor + i < climit) {
                const Pack x1 = st_load(sp, (int64_t) en.u);
                const int32_t p1 = pu != TSG_NO_PARENT ? (int32_t) pu : -1;
                item_put<KQ>(items + cursor + i, item_pack<KQ>(en.x0), x1, (int32_t) en.u,
                    en.p0, p1);
                if (BLS) {
                    // the item's branch lengths in the evaluation's
                    // arithmetic: (bl1, bl0), or (bl1 - bl0, bl0) for FP64
                    // integer summaries of an item whose counts did not
                    // change
                    const double tu = sp.time[en.u];
                    const double bl0 = en.p0 >= 0 ? sp.time[en.p0] - tu : 0.0;
                    const double bl1 = p1 >= 0 ? sp.time[p1] - tu : 0.0;
                    bool same = en.x0[0] == x1.lo;
                    if (KQ > 1) {
                        same = same && en.x0[KQ > 1 ? 1 : 0] == x1.hi;
                    }
                    const int64_t at = cursor + i;
                    if (q.f32) {
                        float *bls = (float *) w.bl;
                        bls[2 * at] = (float) bl1;
                        bls[2 * at + 1] = (float) bl0;
                    } else {
                        double *bls = (double *) w.bl;
                        bls[2 * at] = q.site_int && same ? bl1 - bl0 : bl1;
                        bls[2 * at + 1] = bl0;
                    }
                }
            }
            sp.par[en.u] = (IdxT) pu;  // clears the touch flag
        }
        __syncwarp();
        cursor += nopen;
        nopen = 0;
    };
    // Lanes with `active` set touch node u (distinct per lane) whose
    // counts are still x0 and whose parent entry (flag and parent) is
    // praw, read after the previous batch's touches; returns the
    // entry with the flag set, which the caller stores (with the
    // node's new parent, for an edge's child).  A node is touched at
    // most once per edge event and every event ends with __syncwarp.
    auto touch = [&](bool active, uint32_t u, const Pack &x0, uint32_t praw) {
        bool fresh = active && !(praw & PFLAG);
        unsigned m = __ballot_sync(0xffffffffu, fresh);
        if (nopen + __popc(m) > TSG_TOUCH_CAP) {
            close_list();
            fresh = active;
            m = __ballot_sync(0xffffffffu, fresh);
        }
        if (fresh) {
            const int32_t at = nopen + __popc(m & ((1u << lane) - 1u));
            const uint32_t p0 = praw & PMASK;
            TouchEntry<KQ> en;
            en.x0[0] = x0.lo;
            if (KQ > 1) {
                en.x0[KQ > 1 ? 1 : 0] = x0.hi;
            }
            en.u = u;
            en.p0 = p0 != TSG_NO_PARENT ? (int32_t) p0 : -1;
            s_list[at] = en;
            if (cursor + at >= climit) {
                dev_error(w.err, DEV_ITEM_PLAN);
            }
        }
        nopen += __popc(m);
        return (praw & PMASK) | PFLAG;
    };
    // the next (up to) 32 - first nodes of a root path from v, lane
    // first + j taking the j-th with its parent entry; advances v
    // past them
    auto chase = [&](uint32_t &v, uint32_t &mine, uint32_t &mraw, int first) {
        mine = NO_NODE;
        mraw = 0;
#pragma unroll 4
        for (int j = first; j < 32; j++) {
            if (v == TSG_NO_PARENT) {
                break;
            }
            const uint32_t raw = (uint32_t) sp.par[v];
            mine = lane == j ? v : mine;
            mraw = lane == j ? raw : mraw;
            v = raw & PMASK;
        }
    };
    // One edge event; cm: membership bits of a leaf child (whose
    // branch is accounted per edge, k_leaf_areas).  The nodes are
    // touched in batches of 32 lanes: a stateful child on lane 0
    // with the first 31 nodes of the parent's root path (the child is
    // not on it), then 32 path nodes at a time -- one touch-list
    // step per batch (the span plan counts items with the same
    // batches).  The child keeps its counts and takes its new parent;
    // the path nodes add or remove the child's counts.
    auto event = [&](int32_t p, int32_t c, int sign, uint32_t cm) {
        uint32_t v = (uint32_t) p, mine, mraw;
        const bool child = c >= 0;
        chase(v, mine, mraw, child ? 1 : 0);
        const Pack xc = child ? st_load(sp, c) : pk_from_mask<W>(cm, K);
        bool is_child = false;
        if (child && lane == 0) {
            mine = (uint32_t) c;
            mraw = (uint32_t) sp.par[c];
            is_child = true;
        }
        const uint32_t np = sign > 0 ? (uint32_t) p : TSG_NO_PARENT;
        for (int32_t batches = 1;; batches++) {
            const bool act = mine != NO_NODE;
            Pack xo{0, 0};
            if (act) {
                xo = is_child ? xc : st_load(sp, (int64_t) mine);
            }
            if (q.branch) {
                const uint32_t f = touch(act, mine, xo, mraw);
                if (act) {
                    sp.par[mine] = (IdxT) (is_child ? (np | PFLAG) : f);
                }
            } else if (is_child) {
                sp.par[mine] = (IdxT) np;
            }
            if (act && !is_child) {
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
            if (v == TSG_NO_PARENT) {
                break;
            }
            // a root path has at most Ls nodes: more means a cycle
            if (batches > (Ls >> 5) + 1) {
                dev_error(w.err, DEV_PATH_TOO_LONG);
                break;
            }
            chase(v, mine, mraw, 0);
            is_child = false;
        }
        __syncwarp();
    };
    const int32_t tend = q.branch && t1 < ts.num_trees ? t1 + 1 : t1;
    const bool site = q.site;
    // Prefetch ring: tree t's inputs are staged in three dependent
    // steps -- (a) its event, mutation and item ranges, (b) its event
    // and mutation encodings, (c) the masks of its leaf children and
    // leaf mutation nodes -- issued three, two and one trees ahead.
    auto stage_a = [&](int32_t t) {
        ReplayStage &S = s_stage[t & 3];
        if (lane == 0) {
            cp_async16(&S.ev, &ts.tree_ev[t]);
        } else if (lane == 1) {
            cp_async8(&S.mr, &ts.tree_mut[t]);
        } else if (lane == 2) {
            cp_async8(&S.ioff[0], &ts.tree_item_off[t]);
        } else if (lane == 3) {
            cp_async8(&S.ioff[1], &ts.tree_item_off[t + 1]);
        }
    };
    auto stage_b = [&](int32_t t) {
        ReplayStage &S = s_stage[t & 3];
        const int4 ev = S.ev;
        if (t > t0 && lane < TSG_STAGE_N && lane < ev.y + ev.w) {
            cp_async8(&S.pc[lane], lane < ev.y ? (const void *) &code.rem[ev.x + lane]
                                               : (const void *) &code.ins[ev.z + lane - ev.y]);
        }
        if (site && t < t1 && lane < TSG_STAGE_N && lane < S.mr.y - S.mr.x) {
            cp_async4(&S.menc[lane], &code.mut[S.mr.x + lane]);
        }
    };
    auto stage_c = [&](int32_t t) {
        ReplayStage &S = s_stage[t & 3];
        const int4 ev = S.ev;
        if (t > t0 && lane < TSG_STAGE_N && lane < ev.y + ev.w && S.pc[lane].y < 0) {
            cp_async4(&S.cm[lane], &qd.node_mask[-S.pc[lane].y - 1]);
        }
        if (site && t < t1 && lane < TSG_STAGE_N && lane < S.mr.y - S.mr.x
            && S.menc[lane] < 0) {
            cp_async4(&S.mmask[lane], &qd.node_mask[-S.menc[lane] - 1]);
        }
    };
    for (int32_t k = 0; k < 3; k++) {
        if (t0 + k < tend) {
            stage_a(t0 + k);
        }
    }
    cp_async_wait_all();
    __syncwarp();
    for (int32_t k = 0; k < 2; k++) {
        if (t0 + k < tend) {
            stage_b(t0 + k);
        }
    }
    cp_async_wait_all();
    __syncwarp();
    if (t0 < tend) {
        stage_c(t0);
    }
    cp_async_wait_all();
    __syncwarp();
    for (int32_t t = t0; t < tend; t++) {
        if (t + 3 < tend) {
            stage_a(t + 3);
        }
        if (t + 2 < tend) {
            stage_b(t + 2);
        }
        if (t + 1 < tend) {
            stage_c(t + 1);
        }
        cp_async_commit();
        const ReplayStage &S = s_stage[t & 3];
        if (t > t0) {
            cursor = S.ioff[0];
            climit = S.ioff[1];
            const int32_t r0 = S.ev.x, nr = S.ev.y, i0 = S.ev.z, ni = S.ev.w;
            for (int32_t base = 0; base < nr + ni; base += 32) {
                // up to 32 events of the transition at once (the
                // first TSG_STAGE_N from the ring)
                const int32_t j = base + lane;
                int2 pc = make_int2(0, 0);
                uint32_t cm = 0;
                if (j < nr + ni) {
                    if (j < TSG_STAGE_N) {
                        pc = S.pc[lane];
                        cm = pc.y < 0 ? S.cm[lane] : 0u;
                    } else {
                        pc = j < nr ? code.rem[r0 + j] : code.ins[i0 + (j - nr)];
                        if (pc.y < 0) {
                            cm = qd.node_mask[-pc.y - 1];
                        }
                    }
                }
                const int32_t cnt = min(32, nr + ni - base);
                // each event's fields are fetched one event ahead
                int32_t pn = __shfl_sync(0xffffffffu, pc.x, 0);
                int32_t cn = __shfl_sync(0xffffffffu, pc.y, 0);
                uint32_t mn = __shfl_sync(0xffffffffu, cm, 0);
                for (int32_t e = 0; e < cnt; e++) {
                    const int32_t p = pn, c = cn;
                    const uint32_t m = mn;
                    pn = __shfl_sync(0xffffffffu, pc.x, (e + 1) & 31);
                    cn = __shfl_sync(0xffffffffu, pc.y, (e + 1) & 31);
                    mn = __shfl_sync(0xffffffffu, cm, (e + 1) & 31);
                    event(p, c, base + e < nr ? -1 : +1, m);
                }
            }
            if (q.branch) {
                close_list();
                if (cursor != climit) {
                    dev_error(w.err, DEV_ITEM_PLAN);
                }
                if (EVAL && (t - t0) % TSG_PUBLISH_EVERY == 0) {
                    // publish the tree's items to the evaluating warps
                    __threadfence_block();
                    __syncwarp();
                    if (lane == 0) {
                        *(volatile int *) s_ready = t;
                    }
                }
            }
        }
        if (site && t < t1) {
            const int32_t m0 = S.mr.x, m1 = S.mr.y;
            for (int32_t m = m0 + lane; m < m1; m += 32) {
                int32_t enc;
                uint32_t mask = 0;
                if (m - m0 < TSG_STAGE_N) {
                    enc = S.menc[lane];
                    if (enc < 0) {
                        mask = S.mmask[lane];
                    }
                } else {
                    enc = code.mut[m];
                    if (enc < 0) {
                        mask = qd.node_mask[-enc - 1];
                    }
                }
                const Pack x = enc >= 0 ? st_load(sp, enc) : pk_from_mask<W>(mask, K);
                w.mcnt[(int64_t) m * KQ] = x.lo;
                if (KQ > 1) {
                    w.mcnt[(int64_t) m * KQ + (KQ > 1 ? 1 : 0)] = x.hi;
                }
            }
        }
        cp_async_wait_all();
        __syncwarp();
    }
    if (EVAL && q.branch) {
        __threadfence_block();
        __syncwarp();
        if (lane == 0) {
            *(volatile int *) s_ready = tend;
        }
    }
}

// The evaluating warps of a span's block: they take the span's evaluation
// chunks in order and value each once the replay has completed its tree (a
// bounded wait).
template <typename F, bool UNPOL, int W, int KQ>
__device__ __forceinline__ void eval_span_chunks(const TSView &ts, const QueryParams &q,
    const WsDev &w, int s, int32_t t0, int32_t t1, int *s_ready, int *s_next)
{
    const int lane = threadIdx.x & 31;
    // ---- the other warps value the span's chunks as the replay
    // completes their trees
    const int32_t ta = s == 0 ? 0 : t0 + 1;
    const int32_t tb = t1 < ts.num_trees ? t1 + 1 : t1;
    const int64_t cfirst = ts.tree_chunk_off[ta], clast = ts.tree_chunk_off[tb];
    for (;;) {
        int c0 = 0;
        if (lane == 0) {
            c0 = atomicAdd(s_next, 1);
        }
        const int64_t c = cfirst + __shfl_sync(0xffffffffu, c0, 0);
        if (c >= clast) {
            break;
        }
        const int32_t tc = ts.chunk_tree[c];
        for (uint32_t spin = 0; *(volatile int *) s_ready < tc; spin++) {
            if (spin >= q.spin_limit) {
                dev_error(w.err, DEV_WAIT_TIMEOUT);
                break;
            }
            __nanosleep(128);
        }
        __threadfence_block();
        eval_chunk<F, UNPOL, W, KQ>(ts, q, w, c, lane,
            ts.span_time + ts.span_local_off[ts.chunk_span[c]]);
    }
}

// A summary term's integer numerator with its type fixed at compile time
// (term_num32's cases), plus the same at n - x when unpolarised.
template <int TYPE, bool UNPOL>
__device__ __forceinline__ int64_t typed_num(int32_t xi, int32_t xj, int32_t xk, int32_t xl,
    int32_t ni, int32_t nj, int32_t nk, int32_t nl)
{
    int64_t v = term_num32(TYPE, xi, xj, xk, xl, ni, nj, nk, nl);
    if (UNPOL) {
        v += term_num32(TYPE, ni - xi, nj - xj, nk - xk, nl - xl, ni, nj, nk, nl);
    }
    return v;
}

// One lane's walk over its chunk's items for a term of type TYPE (integer
// numerators, FP64 sums): the four counts the term reads are taken out of
// the packed words with shifts fixed per lane; about one FP64 fused
// multiply-add per item.  Returns the chunk's unscaled sum.
template <int TYPE, bool UNPOL, int KQ>
__device__ __forceinline__ double lane_walk_num(const Item<KQ> *items, const double *bls,
    int64_t b, int64_t e, const Term &t, const int32_t *set_size)
{
    const int32_t i0 = t.idx[0], i1 = t.idx[1], i2 = t.idx[2], i3 = t.idx[3];
    const int32_t ni = set_size[i0], nj = set_size[i1], nk = set_size[i2], nl = set_size[i3];
    const int s0 = 16 * (i0 & 3), s1 = 16 * (i1 & 3), s2 = 16 * (i2 & 3), s3 = 16 * (i3 & 3);
    const bool h0 = i0 >= 4, h1 = i1 >= 4, h2 = i2 >= 4, h3 = i3 >= 4;
    auto cnt = [](uint64_t lo, uint64_t hi, bool h, int sh) {
        return (int32_t) (((h ? hi : lo) >> sh) & 0xFFFFull);
    };
    auto num = [&](uint64_t lo, uint64_t hi) {
        return typed_num<TYPE, UNPOL>(cnt(lo, hi, h0, s0), cnt(lo, hi, h1, s1),
            cnt(lo, hi, h2, s2), cnt(lo, hi, h3, s3), ni, nj, nk, nl);
    };
    double acc = 0;
    // the next item's counts and branch lengths are loaded while this one
    // is valued (the walk is bound by these loads' latency)
    ulonglong2 na = make_ulonglong2(0, 0), nc = make_ulonglong2(0, 0);
    double2 nf = make_double2(0, 0);
    if (b < e) {
        na = *(const ulonglong2 *) items[b].x0;
        if (KQ > 1) {
            nc = *(const ulonglong2 *) items[b].x1;
        }
        nf = *(const double2 *) (bls + 2 * b);
    }
    for (int64_t i = b; i < e; i++) {
        const ulonglong2 ca = na, cc = nc;
        const double2 f = nf;
        if (i + 1 < e) {
            na = *(const ulonglong2 *) items[i + 1].x0;
            if (KQ > 1) {
                nc = *(const ulonglong2 *) items[i + 1].x1;
            }
            nf = *(const double2 *) (bls + 2 * (i + 1));
        }
        uint64_t x0lo, x0hi = 0, x1lo, x1hi = 0;
        if (KQ == 1) {
            x0lo = ca.x;
            x1lo = ca.y;
        } else {
            x0lo = ca.x;
            x0hi = ca.y;
            x1lo = cc.x;
            x1hi = cc.y;
        }
        const bool same = x0lo == x1lo && x0hi == x1hi;
        const uint64_t ba = (uint64_t) __double_as_longlong(f.x);
        const uint64_t bb = (uint64_t) __double_as_longlong(f.y);
        // one uniform FP64 fused multiply-add per item: the multiplier is
        // N(x1) with unchanged counts (bl1 - bl0 in f.x) or no old branch,
        // N(x1) - N(x0) with an unchanged branch (exact in integers), N(x1)
        // when both changed -- whose bl0 N(x0) term, the only other FP64
        // operation, is taken first (the lanes of a warp walk different
        // items, so per-case FP64 instructions would each issue with part
        // of the warp: the FP64 pipe issues a warp instruction every 16
        // cycles whatever its active lanes)
        const int64_t n1 = num(x1lo, x1hi);
        const bool plain = same || bb == 0;
        const int64_t n0 = plain ? 0 : num(x0lo, x0hi);
        const bool both = !plain && ba != bb;
        const int64_t d = (plain || both) ? n1 : n1 - n0;
        double a0 = acc;
        if (both) {
            a0 = fma(-f.y, i64_to_f64(n0), acc);
        }
        acc = fma(f.x, i64_to_f64(d), a0);
    }
    return acc;
}

// k_eval_grouped: a lane per (chunk, term) with every lane of a warp on terms
// of one summary type, so the warp runs one code path (a loop specialised
// to the type for integer numerators); the chunks are taken in decreasing
// item count, TSG_EVAL_BLOCK at a time by q.gwpb consecutive warps; each lane
// walks its chunk's items in order (no sum crosses lanes).  FP64 with integer summaries: exact
// numerators, about one FP64 fused multiply-add per item and lane (as
// eval_chunk); otherwise the summary functions in F (FP32: exact item
// values into a compensated pair).
template <typename F, bool UNPOL, int KQ>
__device__ __forceinline__ void eval_grouped_body(const TSView &ts, const QueryParams &q, const WsDev &w, int64_t total_warps,
    const int64_t bid, const int64_t nb)
{
    constexpr bool F32 = sizeof(F) == sizeof(float);
    const int lane = threadIdx.x & 31;
    const Item<KQ> *items = (const Item<KQ> *) w.items;
    const F *bls = (const F *) w.bl;
    const int64_t C = ts.num_chunks;
    const int R = q.R;
    const bool num_form = !F32 && q.site_int;
    const int64_t nwarps = (int64_t) nb * (blockDim.x >> 5);
    for (int64_t gw = bid * (int64_t) (blockDim.x >> 5) + (threadIdx.x >> 5);
         gw < total_warps; gw += nwarps) {
        // consecutive warps share a block of chunks, so a chunk's items are
        // read by the type groups while they are still in cache
        const int64_t blk = gw / q.gwpb;
        const int sub = (int) (gw % q.gwpb);
        const int g = q.gw_group[sub];
        const int gs = q.gfirst[g + 1] - q.gfirst[g];
        const int pos = q.gw_k[sub] * 32 + lane;
        const int j = pos / gs;
        const int64_t o = blk * TSG_EVAL_BLOCK + j;
        if (j >= TSG_EVAL_BLOCK || o >= C) {
            continue;
        }
        // chunks by decreasing item count: the chunks of a warp take about
        // the same time
        const int64_t c = ts.c_chunk_order[o];
        const int r = q.gterm[q.gfirst[g] + pos % gs];
        const int64_t b = ts.chunk_begin[c], e = ts.chunk_end[c];
        if (num_form) {
            const Term t = q.term[r];
            const double *bd = (const double *) bls;
            double acc = 0;
            switch (t.type) {
                case TSG_DIVERSITY:
                    acc = lane_walk_num<TSG_DIVERSITY, UNPOL, KQ>(items, bd, b, e, t, q.set_size_i);
                    break;
                case TSG_SEGREGATING_SITES:
                    acc = lane_walk_num<TSG_SEGREGATING_SITES, UNPOL, KQ>(items, bd, b, e, t,
                        q.set_size_i);
                    break;
                case TSG_DIVERGENCE:
                    acc = lane_walk_num<TSG_DIVERGENCE, UNPOL, KQ>(items, bd, b, e, t, q.set_size_i);
                    break;
                case TSG_Y3:
                    acc = lane_walk_num<TSG_Y3, UNPOL, KQ>(items, bd, b, e, t, q.set_size_i);
                    break;
                case TSG_Y1:
                    acc = lane_walk_num<TSG_Y1, UNPOL, KQ>(items, bd, b, e, t, q.set_size_i);
                    break;
                case TSG_Y2:
                    acc = lane_walk_num<TSG_Y2, UNPOL, KQ>(items, bd, b, e, t, q.set_size_i);
                    break;
                case TSG_F2:
                    acc = lane_walk_num<TSG_F2, UNPOL, KQ>(items, bd, b, e, t, q.set_size_i);
                    break;
                case TSG_F3:
                    acc = lane_walk_num<TSG_F3, UNPOL, KQ>(items, bd, b, e, t, q.set_size_i);
                    break;
                case TSG_F4:
                    acc = lane_walk_num<TSG_F4, UNPOL, KQ>(items, bd, b, e, t, q.set_size_i);
                    break;
                default:
                    acc = lane_walk_num<TSG_RELATEDNESS_NONCENTRED, UNPOL, KQ>(items, bd, b, e, t,
                        q.set_size_i);
                    break;
            }
            // a term whose denominator is zero (a set too small for it) is
            // NaN wherever the running sum takes a node's value, as in the
            // reference
            const double inv = q.inv[r];
            w.dD[c * R + r] = e <= b ? 0.0 : isfinite(inv) ? acc * inv : (double) NAN;
            continue;
        }
        F acc = 0, lo = 0;
        for (int64_t i = b; i < e; i++) {
            const Item<KQ> it = items[i];
            const F bl1 = bls[2 * i], bl0 = bls[2 * i + 1];
            const Pack x0 = item_pack<KQ>(it.x0);
            const Pack x1 = item_pack<KQ>(it.x1);
            const bool same = x0.lo == x1.lo && x0.hi == x1.hi;
            F m1x, m1c;
            pk_means<F, 16>(q, x1, m1x, m1c);
            const F f1 = term_F<F, UNPOL, 16>(q, r, x1, m1x, m1c);
            if (!same && bl0 != 0) {
                F m0x, m0c;
                pk_means<F, 16>(q, x0, m0x, m0c);
                const F f0 = term_F<F, UNPOL, 16>(q, r, x0, m0x, m0c);
                if constexpr (F32) {
                    acc2_add(acc, lo, bl1, f1, bl0, f0);
                } else {
                    acc += bl0 == bl1 ? bl1 * (f1 - f0) : bl1 * f1 - bl0 * f0;
                }
            } else {
                if constexpr (F32) {
                    acc2_add(acc, lo, bl1, f1, bl0, same ? f1 : (F) 0);
                } else {
                    acc += (same ? bl1 - bl0 : bl1) * f1;
                }
            }
        }
        w.dD[c * R + r] = (double) acc + (double) lo;
    }
}

template <typename F, bool UNPOL, int KQ>
__global__ void __launch_bounds__(256, 4) k_eval_grouped(TSView ts, QueryParams q, WsDev w,
    int64_t total_warps)
{
    eval_grouped_body<F, UNPOL, KQ>(ts, q, w, total_warps, blockIdx.x, gridDim.x);
}

template <int W, int KQ, typename IdxT, typename F, bool UNPOL, bool EVAL>
__global__ void __launch_bounds__(512, 2) k_replay_items(TSView ts, QueryParams q, QueryDev qd,
    WsDev w, int64_t slot_bytes)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_span;
    __shared__ int s_scan[32];
    __shared__ TouchEntry<KQ> s_list[TSG_TOUCH_CAP];  // the open touch list
    __shared__ ReplayStage s_stage[4];                 // prefetch ring, trees t .. t + 3
    __shared__ int s_ready;  // last tree whose items are complete (EVAL)
    __shared__ int s_next;   // next chunk to evaluate, from the span's first (EVAL)
    const int64_t L = ts.max_local;
    // The replay keeps a node's "touched since the touch list opened" flag in
    // the top bit of its parent entry, where the root-path walks read it for
    // free; "no parent" is the all-ones value below that bit.
    constexpr uint32_t PFLAG = sizeof(IdxT) == 2 ? 0x8000u : 0x80000000u;
    constexpr uint32_t PMASK = PFLAG - 1u;
    constexpr uint32_t TSG_NO_PARENT = PMASK;
    constexpr uint32_t NO_NODE = 0xffffffffu;
    SpanState<IdxT> sp = span_state_at<IdxT>(sizeof(IdxT) == 2
            ? smem_raw
            : (unsigned char *) w.state + (int64_t) blockIdx.x * slot_bytes,
        L, KQ);
    sp.cnt = w.seekcnt + (int64_t) blockIdx.x * L;
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
        for (int32_t l = threadIdx.x; l < Ls; l += blockDim.x) {
            if ((uint32_t) sp.par[l] == SpanState<IdxT>::NONE) {
                sp.par[l] = (IdxT) TSG_NO_PARENT;
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

        if (threadIdx.x == 0) {
            s_ready = t0;
            s_next = 0;
        }
        // the first-tree items read the first tree's counts and the parents
        // must be in the replay's encoding: both before the replay starts
        __syncthreads();

        // ---- replay (warp 0).  A span replays the transitions into its
        // trees after the first and, for branch items, into the next span's
        // first tree.  Every stateful node a transition touches (an edge's
        // child, a node on a root path) gets one item: its state before the
        // first touch and after the transition.  The touch list holds at
        // most TSG_TOUCH_CAP nodes; a longer transition closes the list and
        // opens a new one (the span plan counts items the same way).
        if (threadIdx.x < 32) {
            replay_span<W, KQ, IdxT, EVAL>(ts, q, qd, w, sp, s_list, s_stage, &s_ready, t0, t1, Ls,
                ReplayEnc{ts.rem_enc, ts.ins_enc, ts.mut_enc});
        } else if (EVAL && q.branch && (threadIdx.x >> 5) % 4 != 0) {
            // ---- the other warps value the span's chunks as the replay
            // completes their trees
            eval_span_chunks<F, UNPOL, W, KQ>(ts, q, w, s, t0, t1, &s_ready, &s_next);
        }
        __syncthreads();
    }
}


}  // namespace tsg
