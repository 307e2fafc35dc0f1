// Span plan: the topology-only, per-tree-sequence part of the span seek.
//
// Built once on the host (multi-threaded C++) when a tree sequence is
// loaded, deterministic, and uploaded to the device:
//
//   * span boundaries (tree indexes) with about equal edge-event work;
//   * for every span start b, the edges with left <= b < right in edge-table
//     order, i.e. by increasing parent time (the tree a seek must rebuild,
//     tsk_tree_position_seek_forward, c/tskit/trees.c:5701-5763);
//   * per span, a compact numbering of its "stateful" nodes: the nodes that
//     are a parent in the span (in the seek tree or in an inserted edge).
//     Only those carry per-node state (parent, counts, time) during the
//     replay; every other node the span meets is a leaf throughout the span,
//     whose counts are its own sample-set weights.  Node references in the
//     span's edges, edge events and mutations are encoded as the local id
//     (>= 0) of a stateful node or -(global id + 1) of a leaf.
//
// A span replays the transitions into its trees after the first and into
// the first tree of the next span, so every transition belongs to exactly
// one span and the event encodings can live in arrays parallel to the
// insertion and removal orders.
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "tsg_internal.cuh"

namespace tsg {

static void plan_boundaries(const std::vector<int32_t> &tree_in,
    const std::vector<int32_t> &tree_out, int64_t T, int64_t want, std::vector<int32_t> &span_tree)
{
    span_tree.clear();
    span_tree.push_back(0);
    want = std::max<int64_t>(1, std::min<int64_t>(want, T));
    const double total = (double) tree_in[(size_t) T] + (double) tree_out[(size_t) T];
    for (int64_t s = 1; s < want; s++) {
        double target = total * (double) s / (double) want;
        int64_t lo = 0, hi = T;
        while (lo < hi) {
            int64_t mid = (lo + hi) / 2;
            if ((double) tree_in[(size_t) mid] + (double) tree_out[(size_t) mid] < target) {
                lo = mid + 1;
            } else {
                hi = mid;
            }
        }
        if (lo > span_tree.back() && lo < T) {
            span_tree.push_back((int32_t) lo);
        }
    }
    span_tree.push_back((int32_t) T);
}

template <typename T>
static int upload_vec(tsg_treeseq_t *ts, const std::vector<T> &h, T **out)
{
    void *d = nullptr;
    size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(T);
    TSG_CUDA(cudaMalloc(&d, bytes));
    ts->owned.push_back(d);
    if (!h.empty()) {
        TSG_CUDA(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    }
    *out = (T *) d;
    return 0;
}

int build_span_plan(tsg_treeseq_t *ts, const HostTopology &h, int64_t num_spans)
{
    int ret;
    const int64_t E = (int64_t) h.left.size(), T = ts->v.num_trees, N = ts->v.num_nodes;
    plan_boundaries(h.tree_in, h.tree_out, T, num_spans, ts->h_span_tree);
    const int64_t NS = (int64_t) ts->h_span_tree.size() - 1;
    const auto &st = ts->h_span_tree;
    std::vector<double> span_pos((size_t) NS);
    for (int64_t s = 0; s < NS; s++) {
        span_pos[(size_t) s] = ts->h_breakpoints[(size_t) st[(size_t) s]];
    }

    // alive lists in edge order: count, offsets, fill
    std::vector<int32_t> lo((size_t) E), hi((size_t) E);
    std::vector<int64_t> cnt((size_t) NS + 1, 0);
    for (int64_t e = 0; e < E; e++) {
        int64_t a = std::lower_bound(span_pos.begin(), span_pos.end(), h.left[(size_t) e])
            - span_pos.begin();
        int64_t b = std::lower_bound(span_pos.begin(), span_pos.end(), h.right[(size_t) e])
            - span_pos.begin();
        lo[(size_t) e] = (int32_t) a;
        hi[(size_t) e] = (int32_t) b;
        for (int64_t s = a; s < b; s++) {
            cnt[(size_t) s]++;
        }
    }
    std::vector<int64_t> alive_off((size_t) NS + 1, 0);
    int64_t max_alive = 0;
    for (int64_t s = 0; s < NS; s++) {
        alive_off[(size_t) s + 1] = alive_off[(size_t) s] + cnt[(size_t) s];
        max_alive = std::max(max_alive, cnt[(size_t) s]);
    }
    std::vector<int32_t> alive_edge((size_t) alive_off[(size_t) NS]);
    {
        std::vector<int64_t> cur(alive_off.begin(), alive_off.end() - 1);
        for (int64_t e = 0; e < E; e++) {
            for (int32_t s = lo[(size_t) e]; s < hi[(size_t) e]; s++) {
                alive_edge[(size_t) cur[(size_t) s]++] = (int32_t) e;
            }
        }
    }

    // nodes that are a parent in some edge; every other node is a leaf in
    // every tree
    std::vector<uint8_t> is_parent((size_t) N, 0);
    for (int64_t e = 0; e < E; e++) {
        is_parent[(size_t) h.parent[(size_t) e]] = 1;
    }
    std::vector<int32_t> leaf_index((size_t) N, -1), leaves;
    for (int64_t u = 0; u < N; u++) {
        if (!is_parent[(size_t) u]) {
            leaf_index[(size_t) u] = (int32_t) leaves.size();
            leaves.push_back((int32_t) u);
        }
    }
    const int64_t num_leaves = (int64_t) leaves.size();

    // per-span local numbering and encodings, spans in parallel
    std::vector<int2> alive_global(alive_edge.size()), alive_enc(alive_edge.size());
    std::vector<int2> ins_enc((size_t) E), rem_enc((size_t) E);
    std::vector<int32_t> mut_enc(h.mut_node.size());
    std::vector<std::vector<int32_t>> l2g((size_t) NS);
    unsigned nthreads = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    nthreads = (unsigned) std::min<int64_t>(nthreads, NS);
    std::vector<std::thread> pool;
    for (unsigned tid = 0; tid < nthreads; tid++) {
        pool.emplace_back([&, tid]() {
            std::vector<int32_t> stamp((size_t) N, -1), map((size_t) N, 0);
            for (int64_t s = tid; s < NS; s += nthreads) {
                const int32_t t0 = st[(size_t) s], t1 = st[(size_t) s + 1];
                const int32_t tend = t1 < T ? t1 + 1 : t1;
                auto &list = l2g[(size_t) s];
                auto assign = [&](int32_t u) {
                    if (stamp[(size_t) u] != (int32_t) s) {
                        stamp[(size_t) u] = (int32_t) s;
                        map[(size_t) u] = (int32_t) list.size();
                        list.push_back(u);
                    }
                };
                auto enc = [&](int32_t u) {
                    return stamp[(size_t) u] == (int32_t) s ? map[(size_t) u] : -(u + 1);
                };
                const int64_t a0 = alive_off[(size_t) s], a1 = alive_off[(size_t) s + 1];
                for (int64_t i = a0; i < a1; i++) {
                    assign(h.parent[(size_t) alive_edge[(size_t) i]]);
                }
                const int32_t i0 = h.tree_in[(size_t) t0 + (t0 < t1 ? 1 : 0)];
                const int32_t i1 = h.tree_in[(size_t) tend];
                for (int32_t i = i0; i < i1; i++) {
                    assign(h.ins_parent[(size_t) i]);
                }
                // children that are parents elsewhere carry state too, so that
                // the span's leaves are exactly the tree sequence's leaves
                for (int64_t i = a0; i < a1; i++) {
                    const int32_t c = h.child[(size_t) alive_edge[(size_t) i]];
                    if (is_parent[(size_t) c]) {
                        assign(c);
                    }
                }
                for (int32_t i = i0; i < i1; i++) {
                    if (is_parent[(size_t) h.ins_child[(size_t) i]]) {
                        assign(h.ins_child[(size_t) i]);
                    }
                }
                for (int64_t i = a0; i < a1; i++) {
                    int32_t e = alive_edge[(size_t) i];
                    alive_global[(size_t) i] = make_int2(h.parent[(size_t) e], h.child[(size_t) e]);
                    alive_enc[(size_t) i] = make_int2(enc(h.parent[(size_t) e]), enc(h.child[(size_t) e]));
                }
                for (int32_t i = i0; i < i1; i++) {
                    ins_enc[(size_t) i] = make_int2(enc(h.ins_parent[(size_t) i]),
                        enc(h.ins_child[(size_t) i]));
                }
                const int32_t r0 = h.tree_out[(size_t) t0 + (t0 < t1 ? 1 : 0)];
                const int32_t r1 = h.tree_out[(size_t) tend];
                for (int32_t i = r0; i < r1; i++) {
                    rem_enc[(size_t) i] = make_int2(enc(h.rem_parent[(size_t) i]),
                        enc(h.rem_child[(size_t) i]));
                }
                const int32_t m0 = h.site_mut[(size_t) h.tree_sites[(size_t) t0]];
                const int32_t m1 = h.site_mut[(size_t) h.tree_sites[(size_t) t1]];
                for (int32_t m = m0; m < m1; m++) {
                    mut_enc[(size_t) m] = enc(h.mut_node[(size_t) m]);
                }
            }
        });
    }
    for (auto &th : pool) {
        th.join();
    }
    // Item plan: per tree, the number of items the replay emits.  The first
    // tree of the sequence has one per stateful node alive in it; every
    // later tree t has one per stateful node the transition into t touches
    // (the child of an edge event when stateful -- leaves are accounted per
    // edge -- and every node on the parent's root path), counted once per
    // touch list: the replay keeps at most TSG_TOUCH_CAP nodes in a list
    // and, when a touch batch (the stateful child with the first 31 nodes of
    // the parent's root path, then 32 path nodes at a time) would overflow
    // it, closes the list and opens a new one.
    // The transitions into a span's trees after the first and into the next
    // span's first tree belong to the span.  The path lengths are
    // topology-only, so the replay is simulated here.
    //
    // The same simulation records the "touches" of the reference's branch
    // allele frequency spectrum (c/tskit/trees.c:3640-3800), which settles a
    // node's accumulated area whenever the node's own edge is removed or a root
    // path walk passes through it, and not when its edge is inserted: a child
    // inserted after a parentless stretch is credited for that stretch too,
    // from its last touch.  ins_lu records that last touch for every insertion
    // where it precedes the insertion position.  A span simulates the
    // transitions into its trees after the first and into the next span's
    // first tree; a child untouched in the span before its insertion takes its
    // last touch from the earlier spans (resolved in span order below).
    std::vector<int64_t> tree_items((size_t) T + 1, 0);
    std::vector<int64_t> span_max_children((size_t) NS, 0);
    const double nan = std::nan("");
    std::vector<double> ins_lu((size_t) E, nan);
    std::vector<std::vector<std::pair<int32_t, double>>> span_touch((size_t) NS);
    std::vector<std::vector<std::pair<int32_t, int32_t>>> span_pending((size_t) NS);
    {
        std::vector<std::thread> pool2;
        for (unsigned tid = 0; tid < nthreads; tid++) {
            pool2.emplace_back([&, tid]() {
                std::vector<int32_t> par, nch, path, list;
                std::vector<double> lt;
                std::vector<uint8_t> touched, listed;
                for (int64_t s = tid; s < NS; s += nthreads) {
                    const int32_t t0 = st[(size_t) s], t1 = st[(size_t) s + 1];
                    const size_t Ls = l2g[(size_t) s].size();
                    par.assign(Ls, -1);
                    nch.assign(Ls, 0);
                    lt.assign(Ls, 0.0);
                    touched.assign(Ls, 0);
                    listed.assign(Ls, 0);
                    list.clear();
                    const int64_t a0 = alive_off[(size_t) s], a1 = alive_off[(size_t) s + 1];
                    for (int64_t i = a0; i < a1; i++) {
                        const int2 pc = alive_enc[(size_t) i];
                        if (pc.y >= 0) {
                            par[(size_t) pc.y] = pc.x;
                        }
                        span_max_children[(size_t) s] = std::max<int64_t>(
                            span_max_children[(size_t) s], ++nch[(size_t) pc.x]);
                    }
                    if (s == 0) {
                        int64_t anchors = 0;
                        for (int64_t i = a0; i < a1; i++) {
                            anchors += alive_enc[(size_t) i].y >= 0 ? 1 : 0;
                        }
                        tree_items[(size_t) t0] = anchors;
                    }
                    double x = 0;
                    auto touch = [&](int32_t l) {
                        lt[(size_t) l] = x;
                        touched[(size_t) l] = 1;
                    };
                    int64_t cnt = 0;
                    auto close_list = [&]() {
                        cnt += (int64_t) list.size();
                        for (int32_t u : list) {
                            listed[(size_t) u] = 0;
                        }
                        list.clear();
                    };
                    // one touch of the nodes path[b, e) (distinct)
                    auto list_touch = [&](size_t b, size_t e) {
                        size_t fresh = 0;
                        for (size_t k = b; k < e; k++) {
                            fresh += listed[(size_t) path[k]] ? 0 : 1;
                        }
                        if (list.size() + fresh > (size_t) TSG_TOUCH_CAP) {
                            close_list();
                        }
                        for (size_t k = b; k < e; k++) {
                            if (!listed[(size_t) path[k]]) {
                                listed[(size_t) path[k]] = 1;
                                list.push_back(path[k]);
                            }
                        }
                    };
                    // the stateful child c (if any) and the root path from v,
                    // touched in batches of 32: the child with the path's
                    // first 31 nodes, then 32 path nodes at a time
                    auto event = [&](int32_t c, int32_t v) {
                        path.clear();
                        if (c >= 0) {
                            path.push_back(c);
                        }
                        const size_t base = path.size();
                        while (v >= 0 && path.size() - base <= Ls) {
                            touch(v);
                            path.push_back(v);
                            v = par[(size_t) v];
                        }
                        for (size_t b = 0; b < path.size(); b += 32) {
                            list_touch(b, std::min(path.size(), b + 32));
                        }
                    };
                    const int32_t tlast = t1 < T ? t1 : t1 - 1;
                    for (int32_t t = t0 + 1; t <= tlast; t++) {
                        x = ts->h_breakpoints[(size_t) t];
                        cnt = 0;
                        for (int32_t i = h.tree_out[(size_t) t]; i < h.tree_out[(size_t) t + 1]; i++) {
                            const int2 pc = rem_enc[(size_t) i];
                            if (pc.y >= 0) {
                                touch(pc.y);
                            }
                            event(pc.y, pc.x);
                            if (pc.y >= 0) {
                                par[(size_t) pc.y] = -1;
                            }
                        }
                        for (int32_t i = h.tree_in[(size_t) t]; i < h.tree_in[(size_t) t + 1]; i++) {
                            const int2 pc = ins_enc[(size_t) i];
                            if (pc.y >= 0) {
                                if (!touched[(size_t) pc.y]) {
                                    span_pending[(size_t) s].emplace_back(i, l2g[(size_t) s][(size_t) pc.y]);
                                } else if (lt[(size_t) pc.y] < x) {
                                    ins_lu[(size_t) i] = lt[(size_t) pc.y];
                                }
                                par[(size_t) pc.y] = pc.x;
                            }
                            event(pc.y, pc.x);
                        }
                        close_list();
                        tree_items[(size_t) t] = cnt;
                    }
                    for (size_t l = 0; l < Ls; l++) {
                        if (touched[l]) {
                            span_touch[(size_t) s].emplace_back(l2g[(size_t) s][l], lt[l]);
                        }
                    }
                }
            });
        }
        for (auto &th : pool2) {
            th.join();
        }
    }
    {
        // last touches before each span, in span order (the reference starts
        // every node's last update at 0)
        std::vector<double> last((size_t) N, 0.0);
        for (int64_t s = 0; s < NS; s++) {
            for (const auto &pg : span_pending[(size_t) s]) {
                const double xi = h.left[(size_t) h.ins_edge[(size_t) pg.first]];
                if (last[(size_t) pg.second] < xi) {
                    ins_lu[(size_t) pg.first] = last[(size_t) pg.second];
                }
            }
            for (const auto &tc : span_touch[(size_t) s]) {
                last[(size_t) tc.first] = tc.second;
            }
        }
        // leaves are touched only by the removal of their own edges
        std::vector<int32_t> inv((size_t) E);
        for (int64_t i = 0; i < E; i++) {
            inv[(size_t) h.ins_edge[(size_t) i]] = (int32_t) i;
        }
        std::vector<int32_t> order;
        order.reserve((size_t) E);
        for (int64_t e = 0; e < E; e++) {
            if (!is_parent[(size_t) h.child[(size_t) e]]) {
                order.push_back((int32_t) e);
            }
        }
        std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
            const int32_t ca = h.child[(size_t) a], cb = h.child[(size_t) b];
            return ca != cb ? ca < cb : h.left[(size_t) a] < h.left[(size_t) b];
        });
        for (size_t k = 0; k < order.size(); k++) {
            const int32_t e = order[k];
            const bool first = k == 0 || h.child[(size_t) order[k - 1]] != h.child[(size_t) e];
            const double lu = first ? 0.0 : h.right[(size_t) order[k - 1]];
            if (lu < h.left[(size_t) e]) {
                ins_lu[(size_t) inv[(size_t) e]] = lu;
            }
        }
    }
    bool any_gap = false;
    for (int64_t i = 0; i < E && !any_gap; i++) {
        any_gap = !std::isnan(ins_lu[(size_t) i]);
    }
    std::vector<double> ins_right((size_t) E);
    for (int64_t i = 0; i < E; i++) {
        ins_right[(size_t) i] = h.right[(size_t) h.ins_edge[(size_t) i]];
    }
    std::vector<int64_t> tree_item_off((size_t) T + 1, 0);
    for (int64_t t = 0; t < T; t++) {
        tree_item_off[(size_t) t + 1] = tree_item_off[(size_t) t] + tree_items[(size_t) t];
    }
    // evaluation chunks: at most TSG_ITEM_CHUNK items, never across trees,
    // at least one per tree
    std::vector<int64_t> chunk_begin, tree_chunk_off((size_t) T + 1, 0);
    for (int64_t t = 0; t < T; t++) {
        tree_chunk_off[(size_t) t] = (int64_t) chunk_begin.size();
        const int64_t b = tree_item_off[(size_t) t], e = tree_item_off[(size_t) t + 1];
        int64_t c = b;
        do {
            chunk_begin.push_back(c);
            c += TSG_ITEM_CHUNK;
        } while (c < e);
    }
    tree_chunk_off[(size_t) T] = (int64_t) chunk_begin.size();
    chunk_begin.push_back(tree_item_off[(size_t) T]);
    // chunk ends: the next chunk's begin, clipped to the chunk's tree
    std::vector<int64_t> chunk_end(chunk_begin.size() - 1);
    for (int64_t t = 0; t < T; t++) {
        for (int64_t c = tree_chunk_off[(size_t) t]; c < tree_chunk_off[(size_t) t + 1]; c++) {
            chunk_end[(size_t) c] = std::min(chunk_begin[(size_t) c] + TSG_ITEM_CHUNK,
                tree_item_off[(size_t) t + 1]);
        }
    }

    // window segments: about 4,096 runs of consecutive trees, each windowed
    // by one warp (k_span_windows)
    const int64_t seg_len = std::max<int64_t>(1, (T + 4095) / 4096);
    auto &seg_tree = ts->h_seg_tree;
    seg_tree.clear();
    for (int64_t t = 0; t < T; t += seg_len) {
        seg_tree.push_back((int32_t) t);
    }
    seg_tree.push_back((int32_t) T);

    // per tree: its edge events and its mutations, one load each for the replay
    std::vector<int4> tree_ev((size_t) T);
    std::vector<int2> tree_mut((size_t) T);
    for (int64_t t = 0; t < T; t++) {
        const int32_t r0 = h.tree_out[(size_t) t], i0 = h.tree_in[(size_t) t];
        tree_ev[(size_t) t] = make_int4(r0, h.tree_out[(size_t) t + 1] - r0, i0,
            h.tree_in[(size_t) t + 1] - i0);
        tree_mut[(size_t) t] = make_int2(h.site_mut[(size_t) h.tree_sites[(size_t) t]],
            h.site_mut[(size_t) h.tree_sites[(size_t) t + 1]]);
    }

    // the span whose replay writes each chunk's items: the first span for the
    // first tree, else the span replaying the transition into the tree
    std::vector<int32_t> chunk_span(chunk_end.size()), chunk_tree(chunk_end.size());
    for (int64_t t = 0; t < T; t++) {
        for (int64_t c = tree_chunk_off[(size_t) t]; c < tree_chunk_off[(size_t) t + 1]; c++) {
            chunk_tree[(size_t) c] = (int32_t) t;
        }
    }
    for (int64_t sidx = 0; sidx < NS; sidx++) {
        const int32_t ta = sidx == 0 ? 0 : st[(size_t) sidx] + 1;
        const int32_t tb = sidx + 1 < NS ? st[(size_t) sidx + 1] + 1 : (int32_t) T;
        for (int64_t c = tree_chunk_off[(size_t) ta]; c < tree_chunk_off[(size_t) tb]; c++) {
            chunk_span[(size_t) c] = (int32_t) sidx;
        }
    }

    std::vector<int64_t> local_off((size_t) NS + 1, 0);
    int64_t max_local = 0;
    for (int64_t s = 0; s < NS; s++) {
        local_off[(size_t) s + 1] = local_off[(size_t) s] + (int64_t) l2g[(size_t) s].size();
        max_local = std::max<int64_t>(max_local, (int64_t) l2g[(size_t) s].size());
    }
    std::vector<int32_t> l2g_flat((size_t) local_off[(size_t) NS]);
    for (int64_t s = 0; s < NS; s++) {
        std::copy(l2g[(size_t) s].begin(), l2g[(size_t) s].end(),
            l2g_flat.begin() + local_off[(size_t) s]);
    }
    std::vector<double> span_time(l2g_flat.size());
    for (size_t i = 0; i < l2g_flat.size(); i++) {
        span_time[i] = h.node_time[(size_t) l2g_flat[i]];
    }

    int32_t *d_span_tree, *d_l2g, *d_mut_enc;
    int32_t *d_chunk_span, *d_chunk_tree, *d_seg_tree;
    int4 *d_tree_ev;
    int2 *d_tree_mut;
    int64_t *d_alive_off, *d_local_off, *d_tree_item_off, *d_chunk_begin, *d_chunk_end,
        *d_tree_chunk_off;
    int2 *d_alive, *d_alive_enc, *d_ins_enc, *d_rem_enc;
    uint8_t *d_is_parent = nullptr;
    int32_t *d_leaf_index = nullptr, *d_leaves = nullptr;
    double *d_span_time = nullptr;
    double *d_ins_right = nullptr, *d_ins_lu = nullptr;
    std::vector<int32_t> span_tree_v(st.begin(), st.end());
    if ((ret = upload_vec(ts, span_tree_v, &d_span_tree)) || (ret = upload_vec(ts, alive_off, &d_alive_off))
        || (ret = upload_vec(ts, alive_global, &d_alive)) || (ret = upload_vec(ts, alive_enc, &d_alive_enc))
        || (ret = upload_vec(ts, local_off, &d_local_off)) || (ret = upload_vec(ts, l2g_flat, &d_l2g))
        || (ret = upload_vec(ts, ins_enc, &d_ins_enc)) || (ret = upload_vec(ts, rem_enc, &d_rem_enc))
        || (ret = upload_vec(ts, mut_enc, &d_mut_enc))
        || (ret = upload_vec(ts, tree_item_off, &d_tree_item_off))
        || (ret = upload_vec(ts, chunk_begin, &d_chunk_begin))
        || (ret = upload_vec(ts, chunk_end, &d_chunk_end))
        || (ret = upload_vec(ts, chunk_span, &d_chunk_span))
        || (ret = upload_vec(ts, chunk_tree, &d_chunk_tree))
        || (ret = upload_vec(ts, seg_tree, &d_seg_tree))
        || (ret = upload_vec(ts, tree_ev, &d_tree_ev))
        || (ret = upload_vec(ts, tree_mut, &d_tree_mut))
        || (ret = upload_vec(ts, tree_chunk_off, &d_tree_chunk_off))
        || (ret = upload_vec(ts, is_parent, &d_is_parent))
        || (ret = upload_vec(ts, leaf_index, &d_leaf_index))
        || (ret = upload_vec(ts, leaves, &d_leaves))
        || (ret = upload_vec(ts, span_time, &d_span_time))
        || (ret = upload_vec(ts, ins_right, &d_ins_right))
        || (any_gap && (ret = upload_vec(ts, ins_lu, &d_ins_lu)))) {
        return ret;
    }
    ts->v.node_is_parent = d_is_parent;
    ts->v.leaf_index = d_leaf_index;
    ts->v.leaves = d_leaves;
    ts->v.span_time = d_span_time;
    ts->v.num_leaves = num_leaves;
    ts->v.ins_right = d_ins_right;
    ts->v.ins_lu = any_gap ? d_ins_lu : nullptr;
    ts->v.num_spans = NS;
    ts->v.span_tree = d_span_tree;
    ts->v.span_alive_off = d_alive_off;
    ts->v.span_alive = d_alive;
    ts->v.span_alive_enc = d_alive_enc;
    ts->v.span_local_off = d_local_off;
    ts->v.span_l2g = d_l2g;
    ts->v.ins_enc = d_ins_enc;
    ts->v.rem_enc = d_rem_enc;
    ts->v.mut_enc = d_mut_enc;
    ts->v.max_local = max_local;
    ts->v.tree_item_off = d_tree_item_off;
    ts->max_children = 0;
    for (int64_t s = 0; s < NS; s++) {
        ts->max_children = std::max(ts->max_children, span_max_children[(size_t) s]);
    }
    ts->v.chunk_begin = d_chunk_begin;
    ts->v.chunk_end = d_chunk_end;
    ts->v.chunk_span = d_chunk_span;
    ts->v.chunk_tree = d_chunk_tree;
    ts->v.seg_tree = d_seg_tree;
    ts->v.num_segs = (int64_t) seg_tree.size() - 1;
    ts->v.tree_ev = d_tree_ev;
    ts->v.tree_mut = d_tree_mut;
    ts->v.tree_chunk_off = d_tree_chunk_off;
    ts->v.num_chunks = (int64_t) chunk_end.size();
    ts->v.num_items = tree_item_off[(size_t) T];
    ts->max_alive = max_alive;
    ts->h_local_off = local_off;
    ts->h_tree_item0 = T > 0 ? tree_items[0] : 0;
    ts->h_tree_chunk_off = tree_chunk_off;
    ts->h_chunk_items.resize(chunk_end.size());
    for (size_t c = 0; c < chunk_end.size(); c++) {
        ts->h_chunk_items[c] = (int32_t) (chunk_end[c] - chunk_begin[c]);
    }
    return 0;
}

}  // namespace tsg
