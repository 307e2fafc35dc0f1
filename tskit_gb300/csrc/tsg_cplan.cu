// Compact span plan: the topology-only part of the compact replay, the fast
// form of the item pipeline's replay for trees of up to 65,535 samples.
//
// A span's replay only ever reads and writes the nodes its transitions touch
// (an edge event's stateful child and every node on the parent's root path,
// c/tskit/trees.c:1424-1507) and the nodes carrying its trees' mutations.  A
// few hundred nodes per span for hundreds of edge events, against the ~2n
// nodes of a whole tree: so the spans can be short and many, each with a
// small node state in shared memory, and many replays run at once.
//
// Per span (built once, on the host, when a tree sequence is loaded):
//   * its compact node set, numbered in order of first touch, then its
//     mutation-only nodes; each node's parent at the span start (local id);
//   * a depth-first order of the samples of the tree at the span start, so
//     that every node's subtree is a contiguous range [lo, hi) of it; the
//     query's seek turns a prefix sum of the sample-set bits along this order
//     into every compact node's counts (count = P[hi] - P[lo]);
//   * the range endpoints, sorted by position;
//   * the span's edge events and mutations encoded as local ids (stateful
//     nodes) or -(global id + 1) (leaves, which carry their own bits).
// The first tree's items (one per stateful node alive in it) get their own
// numbering, the anchors, whose counts come from the first span's order.
#include <algorithm>
#include <thread>
#include <vector>

#include "tsg_internal.cuh"

namespace tsg {

namespace {

// A forest under edge insertions and removals: parents, ordered child lists
// and the list of roots that hold samples (a parentless node that is a
// sample or has children).
struct Forest {
    std::vector<int32_t> parent, lc, rc, ls, rs, nchild, rprev, rnext;
    std::vector<uint8_t> in_roots;
    const std::vector<uint8_t> *is_sample = nullptr;
    int32_t rhead = -1, rtail = -1;

    void init(int64_t N, const std::vector<uint8_t> &smp)
    {
        is_sample = &smp;
        parent.assign((size_t) N, -1);
        lc.assign((size_t) N, -1);
        rc.assign((size_t) N, -1);
        ls.assign((size_t) N, -1);
        rs.assign((size_t) N, -1);
        nchild.assign((size_t) N, 0);
        rprev.assign((size_t) N, -1);
        rnext.assign((size_t) N, -1);
        in_roots.assign((size_t) N, 0);
        rhead = rtail = -1;
        for (int64_t u = 0; u < N; u++) {
            fix_root((int32_t) u);
        }
    }
    void fix_root(int32_t u)
    {
        const bool want = parent[(size_t) u] < 0 && ((*is_sample)[(size_t) u] || nchild[(size_t) u] > 0);
        if (want && !in_roots[(size_t) u]) {
            in_roots[(size_t) u] = 1;
            rprev[(size_t) u] = rtail;
            rnext[(size_t) u] = -1;
            if (rtail >= 0) {
                rnext[(size_t) rtail] = u;
            } else {
                rhead = u;
            }
            rtail = u;
        } else if (!want && in_roots[(size_t) u]) {
            in_roots[(size_t) u] = 0;
            const int32_t a = rprev[(size_t) u], b = rnext[(size_t) u];
            if (a >= 0) {
                rnext[(size_t) a] = b;
            } else {
                rhead = b;
            }
            if (b >= 0) {
                rprev[(size_t) b] = a;
            } else {
                rtail = a;
            }
        }
    }
    void insert(int32_t c, int32_t p)
    {
        parent[(size_t) c] = p;
        ls[(size_t) c] = rc[(size_t) p];
        rs[(size_t) c] = -1;
        if (rc[(size_t) p] >= 0) {
            rs[(size_t) rc[(size_t) p]] = c;
        } else {
            lc[(size_t) p] = c;
        }
        rc[(size_t) p] = c;
        nchild[(size_t) p]++;
        fix_root(c);
        fix_root(p);
    }
    void remove(int32_t c, int32_t p)
    {
        const int32_t a = ls[(size_t) c], b = rs[(size_t) c];
        if (a >= 0) {
            rs[(size_t) a] = b;
        } else {
            lc[(size_t) p] = b;
        }
        if (b >= 0) {
            ls[(size_t) b] = a;
        } else {
            rc[(size_t) p] = a;
        }
        ls[(size_t) c] = rs[(size_t) c] = -1;
        parent[(size_t) c] = -1;
        nchild[(size_t) p]--;
        fix_root(c);
        fix_root(p);
    }
};

struct SpanOut {
    std::vector<int32_t> l2g;   // local -> global
    std::vector<int32_t> par0;  // parent at the span start (local; -1: none)
    std::vector<int2> ep;       // (position, local << 1 | is_end), sorted
    bool ok = true;             // every touched node's start parent is local
};

}  // namespace

int64_t compact_default_spans(int64_t T, int64_t events, int64_t n)
{
    if (n <= 0 || n > 65535 || T <= 1) {
        return 0;
    }
    // about 256 edge events per span (a few hundred touched nodes), and at
    // most 2^26 sample-order entries in all
    int64_t NC = std::max<int64_t>(1, events / 256);
    NC = std::min<int64_t>(NC, std::max<int64_t>(1, ((int64_t) 1 << 26) / n));
    return std::min<int64_t>(NC, T);
}

int build_compact_plan(tsg_treeseq_t *ts, const HostTopology &h, int64_t want)
{
    ts->v.c_num_spans = 0;
    for (void *p : ts->compact_owned) {
        cudaFree(p);
    }
    ts->compact_owned.clear();
    const int64_t T = ts->v.num_trees, N = ts->v.num_nodes, E = (int64_t) h.left.size();
    const int64_t n = ts->v.num_samples, M = (int64_t) h.mut_node.size();
    if (want <= 0 || n <= 0 || n > 65535 || T < 1) {
        return 0;
    }
    // span boundaries with about equal edge-event work
    std::vector<int32_t> st;
    st.push_back(0);
    {
        const double total = (double) h.tree_in[(size_t) T] + (double) h.tree_out[(size_t) T];
        for (int64_t s = 1; s < want; s++) {
            const double target = total * (double) s / (double) want;
            int64_t lo = 0, hi = T;
            while (lo < hi) {
                const int64_t mid = (lo + hi) / 2;
                if ((double) h.tree_in[(size_t) mid] + (double) h.tree_out[(size_t) mid] < target) {
                    lo = mid + 1;
                } else {
                    hi = mid;
                }
            }
            if (lo > st.back() && lo < T) {
                st.push_back((int32_t) lo);
            }
        }
        st.push_back((int32_t) T);
    }
    const int64_t NC = (int64_t) st.size() - 1;

    std::vector<uint8_t> is_parent((size_t) N, 0), is_sample((size_t) N, 0);
    for (int64_t e = 0; e < E; e++) {
        is_parent[(size_t) h.parent[(size_t) e]] = 1;
    }
    for (int64_t u = 0; u < N; u++) {
        is_sample[(size_t) u] = ts->h_sample_index[(size_t) u] >= 0 ? 1 : 0;
    }

    std::vector<SpanOut> out((size_t) NC);
    // each span's order padded to a multiple of 8 entries (16 bytes), so that
    // every span's starts 16-byte aligned
    const int64_t nst = compact_order_stride(n);
    std::vector<uint16_t> order((size_t) (NC * nst), 0);
    std::vector<int2> ins_enc((size_t) E, make_int2(0, 0)), rem_enc((size_t) E, make_int2(0, 0));
    std::vector<int32_t> mut_enc((size_t) M, 0);
    // the first tree's sample ranges (anchors), from the first span's order
    std::vector<int32_t> lo0, hi0;

    // spans in groups of consecutive spans with about equal work, one thread
    // each; a group rebuilds the forest up to its first span and sweeps on
    unsigned nthreads = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    nthreads = (unsigned) std::min<int64_t>(nthreads, NC);
    std::vector<int64_t> gfirst((size_t) nthreads + 1);
    for (unsigned g = 0; g <= nthreads; g++) {
        gfirst[g] = NC * (int64_t) g / (int64_t) nthreads;
    }
    std::vector<std::thread> pool;
    for (unsigned g = 0; g < nthreads; g++) {
        pool.emplace_back([&, g]() {
            const int64_t s_begin = gfirst[g], s_end = gfirst[(size_t) g + 1];
            if (s_begin >= s_end) {
                return;
            }
            Forest f;
            f.init(N, is_sample);
            std::vector<int32_t> lo((size_t) N, 0), hi((size_t) N, 0), dstamp((size_t) N, -1);
            std::vector<int32_t> lid((size_t) N, 0), lstamp((size_t) N, -1);
            auto apply = [&](int32_t t) {
                for (int32_t i = h.tree_out[(size_t) t]; i < h.tree_out[(size_t) t + 1]; i++) {
                    f.remove(h.rem_child[(size_t) i], h.rem_parent[(size_t) i]);
                }
                for (int32_t i = h.tree_in[(size_t) t]; i < h.tree_in[(size_t) t + 1]; i++) {
                    f.insert(h.ins_child[(size_t) i], h.ins_parent[(size_t) i]);
                }
            };
            // the forest at the group's first span start
            for (int32_t t = 0; t <= st[(size_t) s_begin]; t++) {
                apply(t);
            }
            for (int64_t s = s_begin; s < s_end; s++) {
                const int32_t t0 = st[(size_t) s], t1 = st[(size_t) s + 1];
                SpanOut &o = out[(size_t) s];
                // depth-first sample order of the tree at the span start
                uint16_t *ord = order.data() + s * nst;
                int32_t pos = 0;
                for (int32_t r = f.rhead; r >= 0; r = f.rnext[(size_t) r]) {
                    int32_t u = r;
                    bool done = false;
                    while (!done) {
                        // enter u: its samples start here
                        dstamp[(size_t) u] = (int32_t) s;
                        lo[(size_t) u] = pos;
                        const int32_t si = ts->h_sample_index[(size_t) u];
                        if (si >= 0 && pos < n) {
                            ord[pos++] = (uint16_t) si;
                        }
                        if (f.lc[(size_t) u] >= 0) {
                            u = f.lc[(size_t) u];
                            continue;
                        }
                        // leave u and every ancestor it completes
                        for (;;) {
                            hi[(size_t) u] = pos;
                            if (u == r) {
                                done = true;
                                break;
                            }
                            if (f.rs[(size_t) u] >= 0) {
                                u = f.rs[(size_t) u];
                                break;
                            }
                            u = f.parent[(size_t) u];
                        }
                    }
                }
                if (pos != n) {
                    o.ok = false;
                }
                if (s == 0) {
                    lo0.assign(lo.begin(), lo.end());
                    hi0.assign(hi.begin(), hi.end());
                    for (int64_t u = 0; u < N; u++) {
                        if (dstamp[(size_t) u] != 0) {
                            lo0[(size_t) u] = hi0[(size_t) u] = 0;
                        }
                    }
                }
                // replay the span's transitions: number the touched nodes,
                // recording each one's parent at its first touch (the span
                // start's: only an event's child changes parent, and it is
                // touched when it does)
                auto local = [&](int32_t u) {
                    if (lstamp[(size_t) u] != (int32_t) s) {
                        lstamp[(size_t) u] = (int32_t) s;
                        lid[(size_t) u] = (int32_t) o.l2g.size();
                        o.l2g.push_back(u);
                        o.par0.push_back(f.parent[(size_t) u]);  // global for now
                    }
                    return lid[(size_t) u];
                };
                auto walk = [&](int32_t v) {
                    for (int64_t guard = 0; v >= 0 && guard <= N; guard++) {
                        local(v);
                        v = f.parent[(size_t) v];
                    }
                };
                const int32_t tlast = t1 < T ? t1 : t1 - 1;
                for (int32_t t = t0 + 1; t <= tlast; t++) {
                    for (int32_t i = h.tree_out[(size_t) t]; i < h.tree_out[(size_t) t + 1]; i++) {
                        const int32_t c = h.rem_child[(size_t) i], p = h.rem_parent[(size_t) i];
                        const int32_t ec = is_parent[(size_t) c] ? local(c) : -(c + 1);
                        walk(p);
                        rem_enc[(size_t) i] = make_int2(local(p), ec);
                        f.remove(c, p);
                    }
                    for (int32_t i = h.tree_in[(size_t) t]; i < h.tree_in[(size_t) t + 1]; i++) {
                        const int32_t c = h.ins_child[(size_t) i], p = h.ins_parent[(size_t) i];
                        const int32_t ec = is_parent[(size_t) c] ? local(c) : -(c + 1);
                        walk(p);
                        ins_enc[(size_t) i] = make_int2(local(p), ec);
                        f.insert(c, p);
                    }
                }
                const size_t touched = o.l2g.size();
                // the span's mutations: stateful nodes join the set (counts
                // only; their parents are never read)
                const int32_t m0 = h.site_mut[(size_t) h.tree_sites[(size_t) t0]];
                const int32_t m1 = h.site_mut[(size_t) h.tree_sites[(size_t) t1]];
                for (int32_t m = m0; m < m1; m++) {
                    const int32_t u = h.mut_node[(size_t) m];
                    if (is_parent[(size_t) u]) {
                        const bool fresh = lstamp[(size_t) u] != (int32_t) s;
                        const int32_t l = local(u);
                        if (fresh) {
                            o.par0[(size_t) l] = -1;
                        }
                        mut_enc[(size_t) m] = l;
                    } else {
                        mut_enc[(size_t) m] = -(u + 1);
                    }
                }
                // start parents as local ids; sample ranges at the span start
                for (size_t l = 0; l < o.l2g.size(); l++) {
                    const int32_t pg = o.par0[l];
                    if (pg >= 0) {
                        if (lstamp[(size_t) pg] == (int32_t) s) {
                            o.par0[l] = lid[(size_t) pg];
                        } else {
                            o.par0[l] = -1;
                            o.ok = o.ok && l >= touched;
                        }
                    }
                    const int32_t u = o.l2g[l];
                    const bool in_tree = dstamp[(size_t) u] == (int32_t) s;
                    const int32_t a = in_tree ? lo[(size_t) u] : 0, b = in_tree ? hi[(size_t) u] : 0;
                    o.ep.push_back(make_int2(a, (int32_t) (l << 1)));
                    o.ep.push_back(make_int2(b, (int32_t) (l << 1 | 1)));
                }
                std::sort(o.ep.begin(), o.ep.end(), [](const int2 &x, const int2 &y) {
                    return x.x != y.x ? x.x < y.x : (x.y & 1) < (y.y & 1);
                });
            }
        });
    }
    for (auto &th : pool) {
        th.join();
    }
    int64_t max_local = 0;
    for (int64_t s = 0; s < NC; s++) {
        if (!out[(size_t) s].ok) {
            return 0;  // not representable: the general replay serves
        }
        max_local = std::max<int64_t>(max_local, (int64_t) out[(size_t) s].l2g.size());
    }
    if (max_local > TSG_COMPACT_MAX_LOCAL) {
        return 0;
    }

    // anchors: the stateful children of the first tree's edges in edge order
    // (the first tree's items), then the other nodes alive there
    std::vector<int32_t> a_l2g, a_par;
    std::vector<int2> a_range;
    {
        std::vector<int32_t> aid((size_t) N, -1);
        const double x0 = ts->h_breakpoints.empty() ? 0.0 : ts->h_breakpoints[0];
        std::vector<int64_t> alive;
        for (int64_t e = 0; e < E; e++) {
            if (h.left[(size_t) e] <= x0 && h.right[(size_t) e] > x0) {
                alive.push_back(e);
            }
        }
        for (int64_t e : alive) {
            const int32_t c = h.child[(size_t) e];
            if (is_parent[(size_t) c] && aid[(size_t) c] < 0) {
                aid[(size_t) c] = (int32_t) a_l2g.size();
                a_l2g.push_back(c);
                a_range.push_back(make_int2(lo0[(size_t) c], hi0[(size_t) c]));
            }
        }
        const size_t nitems = a_l2g.size();
        for (int64_t e : alive) {
            const int32_t p = h.parent[(size_t) e];
            if (aid[(size_t) p] < 0) {
                aid[(size_t) p] = (int32_t) a_l2g.size();
                a_l2g.push_back(p);
            }
        }
        std::vector<int32_t> par_of((size_t) N, -1);
        for (int64_t e : alive) {
            par_of[(size_t) h.child[(size_t) e]] = h.parent[(size_t) e];
        }
        a_par.resize(nitems);
        for (size_t k = 0; k < nitems; k++) {
            a_par[k] = aid[(size_t) par_of[(size_t) a_l2g[k]]];
        }
        if ((int64_t) nitems != ts->h_tree_item0) {
            return 0;
        }
    }

    // flatten: spans, then the anchors as the last numbering
    std::vector<int64_t> local_off((size_t) NC + 2, 0), ep_off((size_t) NC + 1, 0);
    for (int64_t s = 0; s < NC; s++) {
        local_off[(size_t) s + 1] = local_off[(size_t) s] + (int64_t) out[(size_t) s].l2g.size();
        ep_off[(size_t) s + 1] = ep_off[(size_t) s] + (int64_t) out[(size_t) s].ep.size();
    }
    local_off[(size_t) NC + 1] = local_off[(size_t) NC] + (int64_t) a_l2g.size();
    std::vector<double> time((size_t) local_off[(size_t) NC + 1]);
    std::vector<uint16_t> par0((size_t) local_off[(size_t) NC]);
    std::vector<int2> ep((size_t) ep_off[(size_t) NC]);
    for (int64_t s = 0; s < NC; s++) {
        const SpanOut &o = out[(size_t) s];
        for (size_t l = 0; l < o.l2g.size(); l++) {
            time[(size_t) local_off[(size_t) s] + l] = h.node_time[(size_t) o.l2g[l]];
            par0[(size_t) local_off[(size_t) s] + l] =
                o.par0[l] >= 0 ? (uint16_t) o.par0[l] : (uint16_t) 0x7FFF;
        }
        std::copy(o.ep.begin(), o.ep.end(), ep.begin() + ep_off[(size_t) s]);
    }
    for (size_t k = 0; k < a_l2g.size(); k++) {
        time[(size_t) local_off[(size_t) NC] + k] = h.node_time[(size_t) a_l2g[k]];
    }
    // per span and chunk of order rows, its first endpoint (the endpoints
    // are sorted by position, so each chunk's are consecutive)
    const int64_t CH = compact_row_chunks(n);
    std::vector<int32_t> ep_chunk((size_t) (NC * (CH + 1)));
    for (int64_t s = 0; s < NC; s++) {
        const std::vector<int2> &e = out[(size_t) s].ep;
        int32_t *row = ep_chunk.data() + s * (CH + 1);
        int64_t j = 0;
        for (int64_t c = 0; c < CH; c++) {
            while (j < (int64_t) e.size() && compact_chunk_of(e[(size_t) j].x, n) < c) {
                j++;
            }
            row[c] = (int32_t) j;
        }
        row[CH] = (int32_t) e.size();
    }
    // the numbering of each evaluation chunk's items: the anchors for the
    // first tree, else the span replaying the transition into the tree
    const std::vector<int64_t> &tco = ts->h_tree_chunk_off;
    std::vector<int32_t> chunk_span((size_t) tco[(size_t) T]);
    for (int64_t t = 0, s = 0; t < T; t++) {
        while (t > 0 && s + 1 < NC && st[(size_t) s + 1] < t) {
            s++;
        }
        for (int64_t c = tco[(size_t) t]; c < tco[(size_t) t + 1]; c++) {
            chunk_span[(size_t) c] = t == 0 ? (int32_t) NC : (int32_t) s;
        }
    }

    // evaluation order: the chunks by decreasing item count, so that the
    // chunks one warp values side by side take about the same time
    std::vector<int32_t> chunk_order(chunk_span.size());
    for (size_t c = 0; c < chunk_order.size(); c++) {
        chunk_order[c] = (int32_t) c;
    }
    std::stable_sort(chunk_order.begin(), chunk_order.end(), [&](int32_t a, int32_t b) {
        return ts->h_chunk_items[(size_t) a] > ts->h_chunk_items[(size_t) b];
    });

    int ret;
    std::vector<void *> &own = ts->compact_owned;
    int32_t *d_st, *d_mut_enc, *d_chunk_span, *d_apar, *d_chunk_order, *d_ep_chunk;
    int64_t *d_local_off, *d_ep_off;
    double *d_time;
    uint16_t *d_par0, *d_order;
    int2 *d_ep, *d_ins, *d_rem, *d_arange;
    if ((ret = upload_host_vec(own, st, &d_st)) || (ret = upload_host_vec(own, local_off, &d_local_off))
        || (ret = upload_host_vec(own, time, &d_time)) || (ret = upload_host_vec(own, par0, &d_par0))
        || (ret = upload_host_vec(own, ep_off, &d_ep_off)) || (ret = upload_host_vec(own, ep, &d_ep))
        || (ret = upload_host_vec(own, ep_chunk, &d_ep_chunk))
        || (ret = upload_host_vec(own, order, &d_order))
        || (ret = upload_host_vec(own, ins_enc, &d_ins)) || (ret = upload_host_vec(own, rem_enc, &d_rem))
        || (ret = upload_host_vec(own, mut_enc, &d_mut_enc))
        || (ret = upload_host_vec(own, chunk_span, &d_chunk_span))
        || (ret = upload_host_vec(own, chunk_order, &d_chunk_order))
        || (ret = upload_host_vec(own, a_par, &d_apar))
        || (ret = upload_host_vec(own, a_range, &d_arange))) {
        return ret;
    }
    TSView &v = ts->v;
    v.c_span_tree = d_st;
    v.c_local_off = d_local_off;
    v.c_time = d_time;
    v.c_par0 = d_par0;
    v.c_ep_off = d_ep_off;
    v.c_ep = d_ep;
    v.c_ep_chunk = d_ep_chunk;
    v.c_order = d_order;
    v.c_ins_enc = d_ins;
    v.c_rem_enc = d_rem;
    v.c_mut_enc = d_mut_enc;
    v.c_chunk_span = d_chunk_span;
    v.c_chunk_order = d_chunk_order;
    v.c_anchor_par = d_apar;
    v.c_anchor_range = d_arange;
    v.c_num_anchors = (int64_t) a_par.size();
    v.c_max_local = max_local;
    v.c_num_spans = NC;
    ts->h_compact_nodes = local_off[(size_t) NC];
    ts->h_compact_endpoints = ep_off[(size_t) NC];
    return 0;
}

}  // namespace tsg
