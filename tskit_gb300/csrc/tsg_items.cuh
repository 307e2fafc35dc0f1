// Item pipeline of the shared-memory sweep (included by tsg_stats.cu).
//
// The sweep is split so that the sequential part carries no floating point:
//
//   k_replay_items  (one CTA per span, state in shared memory, integer only)
//       seek: rebuild the tree at the span start (parallel); emit one item per
//       node alive there (its counts and branch length: the running sum of the
//       first tree is the sum of these items' values, so every span restarts
//       the sum exactly); then warp 0 replays the span's edge removals and
//       insertions in reference order, emitting one item for the edge's child
//       and one per node on the parent's root path (old counts, new counts,
//       branch length); it also records the counts under every mutation at its
//       site's tree.  Items land at positions fixed by the span plan, grouped
//       by tree.  The edge events of a transition are fetched by all lanes at
//       once (encodings, leaf weights, leaf times) before the sequential part.
//   k_eval_items    (one warp per tree, fully parallel)
//       the value of every item for every summary term,
//         path item    bl * (F(new) - F(old))
//         child item   +- bl * F(x)
//         leaf item    +- bl * F(pattern), F from a per-block table (K <= 4)
//       summed per chunk of at most 256 items of one tree (one warp per
//       chunk, FP32 or FP64 per lane, FP64 across lanes).
//   k_span_windows  (one warp per span)
//       the running-sum change of each tree is the sum of its chunks; the
//       running sum of each tree is the prefix sum of those changes over the
//       span's trees (FP64); windows accumulate sum * overlap length.
//   k_site_eval / k_site_windows
//       every site's summary from the integer counts under its mutations
//       (FP64, one thread per site), then per-window sums in a fixed order.
//
// Item values are differences of the summary function at integer counts, so
// no rounding accumulates across spans.

#define TSG_ITEM_PATH 0
#define TSG_ITEM_PLUS 1
#define TSG_ITEM_MINUS 2
#define TSG_ITEM_LEAF_PLUS 3
#define TSG_ITEM_LEAF_MINUS 4
#define TSG_LEAF_TABLE_KMAX 4

template <int KQ>
struct Item {
    uint64_t xo[KQ];
    uint64_t xn[KQ];
    double bl;
    int32_t kind;
    int32_t pad;
};

template <int KQ>
__device__ __forceinline__ Pack item_pack(const uint64_t *a)
{
    Pack p;
    p.lo = a[0];
    p.hi = KQ > 1 ? a[KQ > 1 ? 1 : 0] : 0ull;
    return p;
}

template <int KQ>
__device__ __forceinline__ void item_put(Item<KQ> *it, const Pack &xo, const Pack &xn, double bl,
    int kind)
{
    Item<KQ> v;
    v.xo[0] = xo.lo;
    v.xn[0] = xn.lo;
    if (KQ > 1) {
        v.xo[KQ > 1 ? 1 : 0] = xo.hi;
        v.xn[KQ > 1 ? 1 : 0] = xn.hi;
    }
    v.bl = bl;
    v.kind = kind;
    v.pad = 0;
    *it = v;
}

// item for an edge's child: a leaf (leaf_table) stores its membership bits
template <int KQ>
__device__ __forceinline__ void child_item(Item<KQ> *it, int32_t enc, uint32_t mask,
    const Pack &x, double bl, int sign, bool leaf_table)
{
    if (enc < 0 && leaf_table) {
        item_put<KQ>(it, Pack{0, 0}, Pack{(uint64_t) mask, 0}, bl,
            sign > 0 ? TSG_ITEM_LEAF_PLUS : TSG_ITEM_LEAF_MINUS);
    } else {
        item_put<KQ>(it, Pack{0, 0}, x, bl, sign > 0 ? TSG_ITEM_PLUS : TSG_ITEM_MINUS);
    }
}

// node -> sample-set membership bits for this query
__global__ void k_node_mask(TSView ts, QueryDev qd, uint32_t *node_mask)
{
    for (int64_t u = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; u < ts.num_nodes;
         u += (int64_t) gridDim.x * blockDim.x) {
        const int32_t si = ts.sample_index[u];
        node_mask[u] = si >= 0 ? qd.sample_mask[si] : 0u;
    }
}

template <int KQ>
__global__ void __launch_bounds__(512, 1) k_replay_items(TSView ts, QueryParams q, QueryDev qd,
    WsDev w)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_span;
    const int64_t L = ts.max_local;
    SmemSpan sp;
    sp.KQ = KQ;
    sp.time = (double *) smem_raw;
    sp.xq = (uint64_t *) (sp.time + L);
    sp.cnt = (uint32_t *) (sp.xq + L * KQ);
    sp.par = (uint16_t *) (sp.cnt + L);
    const int K = q.K;
    const int lane = threadIdx.x & 31;
    const bool leaf_table = K <= TSG_LEAF_TABLE_KMAX;
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

        // ---- seek: local nodes start as roots carrying their own weights
        for (int32_t l = threadIdx.x; l < Ls; l += blockDim.x) {
            const int32_t g = l2g[l];
            sp.time[l] = ts.node_time[g];
            sp.par[l] = (uint16_t) TSG_NO_PARENT;
            sp.cnt[l] = 0;
            pk_store(sp, l, pk_from_mask(qd.node_mask[g], K));
        }
        __syncthreads();
        for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
            const int2 pc = ts.span_alive_enc[i];
            if (pc.y >= 0) {
                sp.par[pc.y] = (uint16_t) pc.x;
            }
        }
        __syncthreads();
        // bottom-up counts: every node is added to its parent once, by the
        // last of the parent's children to complete (counter word per node:
        // children in the low half, arrivals in the high half)
        for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
            const int2 pc = ts.span_alive_enc[i];
            atomicAdd(&sp.cnt[pc.x], 1u);
        }
        __syncthreads();
        for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
            const int2 pc = ts.span_alive_enc[i];
            if (pc.y >= 0 && (sp.cnt[pc.y] & 0xFFFFu) != 0) {
                continue;  // an internal child: completed by its own children
            }
            Pack contrib = pc.y >= 0 ? pk_load(sp, pc.y)
                                     : pk_from_mask(qd.node_mask[-pc.y - 1], K);
            uint32_t v = (uint32_t) pc.x;
            for (int32_t guard = 0; v != TSG_NO_PARENT; guard++) {
                if (guard > Ls) {
                    dev_error(w.err, DEV_PATH_TOO_LONG);
                    break;
                }
                if (contrib.lo) {
                    atomicAdd((unsigned long long *) &sp.xq[v * KQ], (unsigned long long) contrib.lo);
                }
                if (KQ > 1 && contrib.hi) {
                    atomicAdd((unsigned long long *) &sp.xq[v * KQ + (KQ > 1 ? 1 : 0)],
                        (unsigned long long) contrib.hi);
                }
                __threadfence_block();
                const uint32_t old = atomicAdd(&sp.cnt[v], 0x10000u);
                if ((old >> 16) + 1 != (old & 0xFFFFu)) {
                    break;
                }
                __threadfence_block();
                contrib.lo = *(volatile unsigned long long *) &sp.xq[v * KQ];
                if (KQ > 1) {
                    contrib.hi = *(volatile unsigned long long *) &sp.xq[v * KQ + (KQ > 1 ? 1 : 0)];
                }
                v = sp.par[v];
            }
        }
        __syncthreads();

        // ---- anchor items: every node alive at the span start
        const int64_t ibase = ts.tree_item_off[t0];
        if (q.branch) {
            for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
                const int2 pc = ts.span_alive_enc[i];
                const int32_t g = pc.y >= 0 ? l2g[pc.y] : -pc.y - 1;
                const uint32_t m = qd.node_mask[g];
                const Pack x = pc.y >= 0 ? pk_load(sp, pc.y) : pk_from_mask(m, K);
                const double tc = pc.y >= 0 ? sp.time[pc.y] : ts.node_time[g];
                child_item<KQ>(items + ibase + (i - a0), pc.y, m, x, sp.time[pc.x] - tc, +1,
                    leaf_table);
            }
        }

        // the anchor items read the first tree's counts: finish them before
        // the replay starts changing counts and parents
        __syncthreads();

        // ---- replay (warp 0)
        if (threadIdx.x < 32) {
            int64_t cursor = ibase + (a1 - a0);
            // one edge event; cm / ct: membership bits and time of a leaf child
            auto event = [&](int32_t p, int32_t c, int sign, uint32_t cm, double ct) {
                const Pack xc = c >= 0 ? pk_load(sp, c) : pk_from_mask(cm, K);
                if (q.branch && lane == 0) {
                    const double tc = c >= 0 ? sp.time[c] : ct;
                    child_item<KQ>(items + cursor, c, cm, xc, sp.time[p] - tc, sign, leaf_table);
                }
                cursor++;
                if (c >= 0) {
                    sp.par[c] = sign > 0 ? (uint16_t) p : (uint16_t) TSG_NO_PARENT;
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
                    const unsigned active = __ballot_sync(0xffffffffu, mine != TSG_NO_PARENT);
                    if (mine != TSG_NO_PARENT) {
                        const Pack xo = pk_load(sp, (int32_t) mine);
                        Pack xn;
                        if (sign > 0) {
                            xn.lo = xo.lo + xc.lo;
                            xn.hi = xo.hi + xc.hi;
                        } else {
                            xn.lo = xo.lo - xc.lo;
                            xn.hi = xo.hi - xc.hi;
                        }
                        if (q.branch) {
                            const double bl = up != TSG_NO_PARENT ? sp.time[up] - sp.time[mine] : 0.0;
                            item_put<KQ>(items + cursor + lane, xo, xn, bl, TSG_ITEM_PATH);
                        }
                        pk_store(sp, (int32_t) mine, xn);
                    }
                    cursor += __popc(active);
                }
                __syncwarp();
            };
            for (int32_t t = t0; t < t1; t++) {
                if (t > t0) {
                    const int32_t r0 = ts.tree_out[t], nr = ts.tree_out[t + 1] - r0;
                    const int32_t i0 = ts.tree_in[t], ni = ts.tree_in[t + 1] - i0;
                    for (int32_t base = 0; base < nr + ni; base += 32) {
                        // fetch up to 32 events of the transition at once
                        const int32_t j = base + lane;
                        int2 pc = make_int2(0, 0);
                        uint32_t cm = 0;
                        double ct = 0;
                        if (j < nr + ni) {
                            pc = j < nr ? ts.rem_enc[r0 + j] : ts.ins_enc[i0 + (j - nr)];
                            if (pc.y < 0) {
                                cm = qd.node_mask[-pc.y - 1];
                                ct = ts.node_time[-pc.y - 1];
                            }
                        }
                        const int32_t cnt = min(32, nr + ni - base);
                        for (int32_t e = 0; e < cnt; e++) {
                            const int32_t p = __shfl_sync(0xffffffffu, pc.x, e);
                            const int32_t c = __shfl_sync(0xffffffffu, pc.y, e);
                            const uint32_t m = __shfl_sync(0xffffffffu, cm, e);
                            const double tc = __shfl_sync(0xffffffffu, ct, e);
                            event(p, c, base + e < nr ? -1 : +1, m, tc);
                        }
                    }
                    if (q.branch && cursor != ts.tree_item_off[t + 1]) {
                        dev_error(w.err, DEV_ITEM_PLAN);
                    }
                }
                if (q.site) {
                    const int32_t m0 = ts.site_mut[ts.tree_sites[t]];
                    const int32_t m1 = ts.site_mut[ts.tree_sites[t + 1]];
                    for (int32_t m = m0 + lane; m < m1; m += 32) {
                        const int32_t enc = ts.mut_enc[m];
                        const Pack x = enc >= 0 ? pk_load(sp, enc)
                                                : pk_from_mask(qd.node_mask[-enc - 1], K);
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

// Value of every item of a chunk for every term, summed per chunk (one
// warp per chunk; chunks never cross trees).
template <typename F, bool UNPOL, int RMAX, int KQ>
__global__ void __launch_bounds__(256, 2) k_eval_items(TSView ts, QueryParams q, WsDev w)
{
    __shared__ F s_leaf[1 << TSG_LEAF_TABLE_KMAX][RMAX];
    const int lane = threadIdx.x & 31;
    const int R = q.R;
    if (q.K <= TSG_LEAF_TABLE_KMAX) {
        // F of every membership pattern a leaf can have
        const int npat = 1 << q.K;
        for (int i = threadIdx.x; i < npat * R; i += blockDim.x) {
            const int pat = i / R, r = i % R;
            const Pack x = pk_from_mask((uint32_t) pat, q.K);
            F mx, mc;
            pk_means<F>(q, x, mx, mc);
            s_leaf[pat][r] = term_F<F, UNPOL>(q, r, x, mx, mc);
        }
        __syncthreads();
    }
    const int64_t c = (int64_t) blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= ts.num_chunks) {
        return;
    }
    const Item<KQ> *items = (const Item<KQ> *) w.items;
    const int64_t b = ts.chunk_begin[c], e = ts.chunk_end[c];
    // at most TSG_ITEM_CHUNK / 32 items per lane: plain sums in F, then FP64
    F acc[RMAX];
#pragma unroll
    for (int r = 0; r < RMAX; r++) {
        acc[r] = 0;
    }
    for (int64_t i = b + lane; i < e; i += 32) {
        const Item<KQ> it = items[i];
        const F bl = (F) it.bl;
        if (it.kind >= TSG_ITEM_LEAF_PLUS) {
            const int pat = (int) it.xn[0];
            const F sb = it.kind == TSG_ITEM_LEAF_PLUS ? bl : -bl;
#pragma unroll
            for (int r = 0; r < RMAX; r++) {
                if (r < R) {
                    acc[r] += sb * s_leaf[pat][r];
                }
            }
            continue;
        }
        const Pack xn = item_pack<KQ>(it.xn);
        F mxn, mcn;
        pk_means<F>(q, xn, mxn, mcn);
        if (it.kind == TSG_ITEM_PATH) {
            const Pack xo = item_pack<KQ>(it.xo);
            F mxo, mco;
            pk_means<F>(q, xo, mxo, mco);
#pragma unroll
            for (int r = 0; r < RMAX; r++) {
                if (r < R) {
                    acc[r] += bl * (term_F<F, UNPOL>(q, r, xn, mxn, mcn)
                        - term_F<F, UNPOL>(q, r, xo, mxo, mco));
                }
            }
        } else {
            const F sb = it.kind == TSG_ITEM_PLUS ? bl : -bl;
#pragma unroll
            for (int r = 0; r < RMAX; r++) {
                if (r < R) {
                    acc[r] += sb * term_F<F, UNPOL>(q, r, xn, mxn, mcn);
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < RMAX; r++) {
        if (r < R) {
            const double v = warp_sum((double) acc[r]);
            if (lane == r) {
                w.dD[c * R + r] = v;
            }
        }
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
    for (int64_t j = lane; j < nwin * R; j += 32) {
        w.B[woff * R + j] = 0;
    }
    __syncwarp();
    double cum = 0;
    int32_t wi = wlo;
    for (int32_t t = t0; t < t1; t++) {
        const double tl = ts.breakpoints[t], tr = ts.breakpoints[t + 1];
        if (lane < R) {
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
}

// Each site's summary, summed over its alleles (skipping the ancestral one
// when polarised), from the integer counts under its mutations.
template <int RMAX, int KQ>
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
        int32_t st[TSG_SMEM_KMAX];
#pragma unroll
        for (int k = 0; k < TSG_SMEM_KMAX; k++) {
            st[k] = (a == 0 && k < K) ? (int32_t) q.set_size[k] : 0;
        }
        for (int32_t m = m0; m < m1; m++) {
            Pack xm;
            xm.lo = w.mcnt[(int64_t) m * KQ];
            xm.hi = KQ > 1 ? w.mcnt[(int64_t) m * KQ + (KQ > 1 ? 1 : 0)] : 0ull;
            const int al = ts.mutation_allele[m], alt = ts.mutation_alt[m];
#pragma unroll
            for (int k = 0; k < TSG_SMEM_KMAX; k++) {
                const int32_t v = (int32_t) pk_get(xm, k);
                st[k] += (al == a ? v : 0) - (alt == a ? v : 0);
            }
        }
        Pack ps{0, 0};
#pragma unroll
        for (int k = 0; k < TSG_SMEM_KMAX; k++) {
            const uint64_t v = (uint64_t) (st[k] & 0xFFFF);
            if (k < 4) {
                ps.lo |= v << (16 * k);
            } else {
                ps.hi |= v << (16 * (k - 4));
            }
        }
        double mx, mc;
        pk_means<double>(q, ps, mx, mc);
#pragma unroll
        for (int r = 0; r < RMAX; r++) {
            if (r < R) {
                val[r] += term_F<double, false>(q, r, ps, mx, mc);
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
