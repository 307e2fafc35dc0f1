// Allele frequency spectrum on the GPU.
//
// Replaces tsk_treeseq_allele_frequency_spectrum (c/tskit/trees.c:3830-3928)
// with its site and branch modes (trees.c:3499-3637, 3639-3828).  Counts
// carry the K sample sets plus the count of all the tree sequence's samples
// (the reference's extra count column); a node or allele contributes only
// when that count is neither 0 nor the number of samples.
//
// Site mode: the item replay records the integer counts under every
// mutation; one thread per site forms the allele states (exact) and adds 1
// (polarised) or 1/2 to its bin.  Sums of halves are exact in FP64, so the
// atomic adds are order-independent.
//
// Branch mode follows the reference's lazy accounting: a node's area
// (elapsed length x branch length, split over time windows) is settled at
// each "touch" -- the removal of its own edge, a root-path walk through it,
// a window end -- into the bin of its counts at that moment.  Here:
//   * k_afs_replay: one CTA per span rebuilds the span's first tree (the
//     shared seek) and replays the span's edge events, settling a stateful
//     node's area at each of its touches and, at the span end, every node
//     with a parent ("records" [last touch, position) x branch length);
//   * k_afs_leaf_edges: leaves (nodes that are never a parent) are touched
//     only by the removal of their own edges, so a leaf edge's record is the
//     edge itself, from the leaf's last touch before the insertion;
//   * a child inserted after a parentless stretch is credited by the
//     reference for that stretch as well (its area runs from its last touch);
//     the span plan gives that last touch per insertion (ins_lu) and the
//     replay adds the extra record.
// Every record's area is accumulated exactly, as a 256-bit fixed-point
// integer (2^-128 resolution) split over 32-bit limbs of 64-bit counters, so
// the result does not depend on the order of the atomic adds; k_afs_finish
// rounds each bin once to FP64 and applies span normalisation.
#include "tsg_fixed.cuh"
#include "tsg_replay.cuh"

namespace tsg {

// The reference's fold (trees.c:3469-3497) in integers: with every count
// doubled the half-integer comparisons become exact integer ones.
// Returns -1 when a count lies outside [0, n_k] (an inconsistent tree
// sequence), so that no access goes outside the result.
__device__ __forceinline__ int64_t afs_bin(const AfsParams &a, int64_t *c)
{
#pragma unroll
    for (int k = 0; k < TSG_AFS_KMAX; k++) {
        if (k < a.K && (c[k] < 0 || c[k] >= a.dims[k])) {
            return -1;
        }
    }
    if (!a.polarised) {
        int64_t n2 = 0, s2 = 0;
#pragma unroll
        for (int k = 0; k < TSG_AFS_KMAX; k++) {
            if (k < a.K) {
                n2 += a.dims[k] - 1;
                s2 += 2 * c[k];
            }
        }
        int k = a.K;
        while (s2 == n2 && k > 0) {
            k--;
            n2 -= a.dims[k] - 1;
            s2 -= 2 * c[k];
        }
        if (s2 > n2) {
#pragma unroll
            for (int j = 0; j < TSG_AFS_KMAX; j++) {
                if (j < a.K) {
                    c[j] = a.dims[j] - 1 - c[j];
                }
            }
        }
    }
    int64_t bin = 0;
#pragma unroll
    for (int k = 0; k < TSG_AFS_KMAX; k++) {
        if (k < a.K) {
            bin += c[k] * a.stride[k];
        }
    }
    return bin;
}

// first window containing x (windows[w] <= x < windows[w + 1])
__device__ __forceinline__ int afs_window(const AfsParams &a, double x)
{
    int w = (int) upper_bound(a.windows, (int64_t) a.Wn + 1, x) - 1;
    return w < 0 ? 0 : (w >= a.Wn ? a.Wn - 1 : w);
}

// Settle the area of a node with counts x on the branch (tu, tp) over the
// genome stretch [xs, xe), split at window and time-window boundaries as the
// reference does (trees.c:3639-3690).
template <int W>
__device__ void afs_record(const AfsParams &a, const Pack &x, double tu, double tp, double xs,
    double xe)
{
    const int64_t all = (int64_t) pk_get<W>(x, a.K);
    if (all == 0 || all >= a.num_samples || !(xs < xe)) {
        return;
    }
    int64_t c[TSG_AFS_KMAX];
#pragma unroll
    for (int k = 0; k < TSG_AFS_KMAX; k++) {
        c[k] = k < a.K ? (int64_t) pk_get<W>(x, k) : 0;
    }
    const int64_t bin = afs_bin(a, c);
    if (bin < 0) {
        dev_error(a.err, DEV_NODE_OUT_OF_BOUNDS);
        return;
    }
    for (int w = afs_window(a, xs); w < a.Wn && a.windows[w] < xe; w++) {
        const double lo = xs > a.windows[w] ? xs : a.windows[w];
        const double hi = xe < a.windows[w + 1] ? xe : a.windows[w + 1];
        const double span = hi - lo;
        if (!(span > 0)) {
            continue;
        }
        for (int t = 0; t < a.TW && a.time_windows[t] < tp; t++) {
            const double top = a.time_windows[t + 1] < tp ? a.time_windows[t + 1] : tp;
            const double bot = a.time_windows[t] > tu ? a.time_windows[t] : tu;
            const double twbl = top - bot > 0.0 ? top - bot : 0.0;
            fx_add(a.acc + (((int64_t) w * a.TW + t) * a.afs_size + bin) * TSG_FX_LIMBS,
                span * twbl, a.err);
        }
    }
}

template <int W, int KQ, typename IdxT>
__global__ void __launch_bounds__(512, 1) k_afs_replay(TSView ts, QueryDev qd, AfsParams a,
    void *state, int64_t slot_bytes)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_span;
    const int64_t L = ts.max_local;
    constexpr uint32_t NONE = SpanState<IdxT>::NONE;
    unsigned char *base =
        sizeof(IdxT) == 2 ? smem_raw : (unsigned char *) state + (int64_t) blockIdx.x * slot_bytes;
    SpanState<IdxT> sp = span_state_at<IdxT>(base, L, KQ);
    double *last = (double *) span_state_end(sp, L);
    sp.cnt = a.seekcnt + (int64_t) blockIdx.x * L;
    const int KC = a.K + 1;
    const int lane = threadIdx.x & 31;

    for (;;) {
        if (threadIdx.x == 0) {
            s_span = atomicAdd(a.counter, 1);
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
        const double xs0 = ts.breakpoints[t0], xe0 = ts.breakpoints[t1];
        sp.time = ts.span_time + lo;

        span_seek<W, KQ, IdxT>(ts, qd, a.err, sp, KC, Ls, l2g, a0, a1);
        for (int32_t l = threadIdx.x; l < Ls; l += blockDim.x) {
            last[l] = xs0;
        }
        __syncthreads();

        // one transition (warp 0): records settle touched nodes' areas; the
        // final transition (into the next span's first tree) only adds the
        // parentless-stretch credit of inserted children
        auto transition = [&](int32_t t, bool records) {
            const double x = ts.breakpoints[t];
            const int32_t r0 = ts.tree_out[t], nr = ts.tree_out[t + 1] - r0;
            const int32_t i0 = ts.tree_in[t], ni = ts.tree_in[t + 1] - i0;
            for (int32_t b = 0; b < nr + ni; b += 32) {
                const int32_t j = b + lane;
                int2 pc = make_int2(0, 0);
                uint32_t cm = 0;
                double gap = NAN;
                if (j < nr + ni) {
                    pc = j < nr ? ts.rem_enc[r0 + j] : ts.ins_enc[i0 + (j - nr)];
                    if (pc.y < 0) {
                        cm = qd.node_mask[-pc.y - 1];
                    }
                    if (j >= nr && ts.ins_lu != nullptr) {
                        gap = ts.ins_lu[i0 + (j - nr)];
                    }
                }
                const int32_t cnt = min(32, nr + ni - b);
                for (int32_t e = 0; e < cnt; e++) {
                    const int32_t p = __shfl_sync(0xffffffffu, pc.x, e);
                    const int32_t c = __shfl_sync(0xffffffffu, pc.y, e);
                    const uint32_t m = __shfl_sync(0xffffffffu, cm, e);
                    const double g = __shfl_sync(0xffffffffu, gap, e);
                    const int sign = b + e < nr ? -1 : +1;
                    const Pack xc = c >= 0 ? st_load(sp, c) : pk_from_mask<W>(m, KC);
                    if (c >= 0 && lane == 0) {
                        if (sign < 0) {
                            if (records) {
                                afs_record<W>(a, xc, sp.time[c], sp.time[p], last[c], x);
                            }
                            sp.par[c] = (IdxT) NONE;
                        } else {
                            if (g < x) {
                                const double ws = a.windows[afs_window(a, x)];
                                afs_record<W>(a, xc, sp.time[c], sp.time[p], g > ws ? g : ws, x);
                            }
                            sp.par[c] = (IdxT) p;
                        }
                        last[c] = x;
                    }
                    __syncwarp();
                    uint32_t v = (uint32_t) p;
                    int32_t guard = 0;
                    while (v != NONE) {
                        uint32_t mine = NONE;
#pragma unroll 1
                        for (int jj = 0; jj < 32 && v != NONE; jj++) {
                            if (lane == jj) {
                                mine = v;
                            }
                            v = sp.par[v];
                            if (++guard > Ls) {
                                dev_error(a.err, DEV_PATH_TOO_LONG);
                                v = NONE;
                            }
                        }
                        uint32_t up = __shfl_down_sync(0xffffffffu, mine, 1);
                        if (lane == 31) {
                            up = v;
                        }
                        if (mine != NONE) {
                            const Pack xo = st_load(sp, (int64_t) mine);
                            if (records && up != NONE) {
                                afs_record<W>(a, xo, sp.time[mine], sp.time[up], last[mine], x);
                            }
                            last[mine] = x;
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
                }
            }
        };

        if (threadIdx.x < 32) {
            for (int32_t t = t0 + 1; t < t1; t++) {
                transition(t, true);
            }
        }
        __syncthreads();
        // span end: settle every node that has a parent
        for (int32_t l = threadIdx.x; l < Ls; l += blockDim.x) {
            const uint32_t p = (uint32_t) sp.par[l];
            if (p != NONE) {
                afs_record<W>(a, st_load(sp, l), sp.time[l], sp.time[p], last[l], xe0);
            }
        }
        __syncthreads();
        if (ts.ins_lu != nullptr && t1 < ts.num_trees && threadIdx.x < 32) {
            transition(t1, false);
        }
        __syncthreads();
    }
}

// Leaves: one record per edge, from the leaf's last touch (the previous
// removal of one of its edges, or the current window's start) to the edge's
// right end.
template <int W>
__global__ void __launch_bounds__(256) k_afs_leaf_edges(TSView ts, QueryDev qd, AfsParams a)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < ts.num_edges;
         i += (int64_t) gridDim.x * blockDim.x) {
        const int32_t c = ts.ins_child[i];
        if (ts.node_is_parent[c]) {
            continue;
        }
        const uint32_t m = qd.node_mask[c];
        if (!((m >> a.K) & 1u)) {
            continue;  // not a sample: no samples below
        }
        const double left = ts.ins_left[i];
        double start = left;
        if (ts.ins_lu != nullptr) {
            const double lu = ts.ins_lu[i];
            if (lu < left) {
                const double ws = a.windows[afs_window(a, left)];
                start = lu > ws ? lu : ws;
            }
        }
        afs_record<W>(a, pk_from_mask<W>(m, a.K + 1), ts.node_time[c],
            ts.node_time[ts.ins_parent[i]], start, ts.ins_right[i]);
    }
}

// One thread per site: allele states from the counts under its mutations
// (get_allele_weights, trees.c:1525-1612), then the site's AFS increments
// (trees.c:3499-3547).
template <int W, int KQ>
__global__ void __launch_bounds__(256) k_afs_site(TSView ts, AfsParams a, const uint64_t *mcnt)
{
    const int64_t site = blockIdx.x * (int64_t) blockDim.x + threadIdx.x;
    if (site >= ts.num_sites) {
        return;
    }
    const int KC = a.K + 1;
    const int32_t m0 = ts.site_mut[site], m1 = ts.site_mut[site + 1];
    int32_t A = 1;
    for (int32_t m = m0; m < m1; m++) {
        A = max(A, ts.mutation_allele[m] + 1);
    }
    const int w = afs_window(a, ts.site_position[site]);
    const double inc = a.polarised ? 1.0 : 0.5;
    constexpr int KM = 2 * (64 / W);
    for (int32_t al = a.polarised ? 1 : 0; al < A; al++) {
        int64_t st[KM];
#pragma unroll
        for (int k = 0; k < KM; k++) {
            st[k] = 0;
            if (al == 0 && k < KC) {
                st[k] = k < a.K ? a.dims[k] - 1 : a.num_samples;
            }
        }
        for (int32_t m = m0; m < m1; m++) {
            Pack xm;
            xm.lo = mcnt[(int64_t) m * KQ];
            xm.hi = KQ > 1 ? mcnt[(int64_t) m * KQ + (KQ > 1 ? 1 : 0)] : 0ull;
            const int mal = ts.mutation_allele[m], malt = ts.mutation_alt[m];
#pragma unroll
            for (int k = 0; k < KM; k++) {
                const int64_t v = (int64_t) pk_get<W>(xm, k);
                st[k] += (mal == al ? v : 0) - (malt == al ? v : 0);
            }
        }
        int64_t all = 0;
        int64_t c[TSG_AFS_KMAX];
#pragma unroll
        for (int k = 0; k < KM; k++) {
            if (k == a.K) {
                all = st[k];
            }
            if (k < TSG_AFS_KMAX) {
                c[k] = st[k];
            }
        }
        if (all > 0 && all < a.num_samples) {
            const int64_t bin = afs_bin(a, c);
            if (bin < 0) {
                dev_error(a.err, DEV_NODE_OUT_OF_BOUNDS);
            } else {
                atomicAdd(a.out + (int64_t) w * a.afs_size + bin, inc);
            }
        }
    }
}

// Round the branch counters and apply span normalisation (trees.c:3921-3923).
__global__ void __launch_bounds__(256) k_afs_finish(AfsParams a, int span_normalise, int branch,
    double *result)
{
    const int64_t per_window = (int64_t) a.TW * a.afs_size;
    const int64_t total = (int64_t) a.Wn * per_window;
    for (int64_t idx = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t) gridDim.x * blockDim.x) {
        double v = branch ? fx_value(a.acc + idx * TSG_FX_LIMBS) : result[idx];
        if (span_normalise) {
            const int64_t w = idx / per_window;
            v /= a.windows[w + 1] - a.windows[w];
        }
        result[idx] = v;
    }
}

static unsigned grid_of(int64_t n)
{
    const int64_t g = (n + 255) / 256;
    return (unsigned) (g < 1 ? 1 : (g > 65535LL * 4 ? 65535LL * 4 : g));
}

void *afs_replay_kernel(int form)
{
    switch (form) {
        case 0: return (void *) k_afs_replay<16, 1, uint16_t>;
        case 1: return (void *) k_afs_replay<16, 2, uint16_t>;
        case 2: return (void *) k_afs_replay<32, 1, int32_t>;
        default: return (void *) k_afs_replay<32, 2, int32_t>;
    }
}

int launch_afs_branch(int form, unsigned grid, size_t smem, int64_t slot_bytes, void *state,
    cudaStream_t st, const TSView &v, const QueryDev &qd, const AfsParams &a)
{
    switch (form) {
        case 0: k_afs_replay<16, 1, uint16_t><<<grid, 512, smem, st>>>(v, qd, a, state, 0); break;
        case 1: k_afs_replay<16, 2, uint16_t><<<grid, 512, smem, st>>>(v, qd, a, state, 0); break;
        case 2: k_afs_replay<32, 1, int32_t><<<grid, 512, 0, st>>>(v, qd, a, state, slot_bytes); break;
        default: k_afs_replay<32, 2, int32_t><<<grid, 512, 0, st>>>(v, qd, a, state, slot_bytes); break;
    }
    TSG_LAUNCHED();
    if (v.num_edges > 0) {
        if (form < 2) {
            k_afs_leaf_edges<16><<<grid_of(v.num_edges), 256, 0, st>>>(v, qd, a);
        } else {
            k_afs_leaf_edges<32><<<grid_of(v.num_edges), 256, 0, st>>>(v, qd, a);
        }
        TSG_LAUNCHED();
    }
    return 0;
}

int launch_afs_site(int form, cudaStream_t st, const TSView &v, const AfsParams &a,
    const uint64_t *mcnt)
{
    if (v.num_sites == 0) {
        return 0;
    }
    const unsigned g = grid_of(v.num_sites);
    switch (form) {
        case 0: k_afs_site<16, 1><<<g, 256, 0, st>>>(v, a, mcnt); break;
        case 1: k_afs_site<16, 2><<<g, 256, 0, st>>>(v, a, mcnt); break;
        case 2: k_afs_site<32, 1><<<g, 256, 0, st>>>(v, a, mcnt); break;
        default: k_afs_site<32, 2><<<g, 256, 0, st>>>(v, a, mcnt); break;
    }
    TSG_LAUNCHED();
    return 0;
}

int launch_afs_finish(cudaStream_t st, const AfsParams &a, int span_normalise, int branch,
    double *result)
{
    k_afs_finish<<<grid_of((int64_t) a.Wn * a.TW * a.afs_size), 256, 0, st>>>(a, span_normalise,
        branch, result);
    TSG_LAUNCHED();
    return 0;
}

}  // namespace tsg
