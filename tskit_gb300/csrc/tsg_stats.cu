// Sample-count statistics on the GPU: branch and site modes.
//
// Replaces tsk_treeseq_branch_general_stat / tsk_treeseq_site_general_stat
// (c/tskit/trees.c:1352-1523, 1654-1776) for the named summary functions
// (c/tskit/trees.c:3934-5309) with a span-parallel sweep:
//
//   * The trees are cut into spans (tree ranges).  One CTA takes a span,
//     rebuilds the tree at the span start from the span's alive-edge list
//     (parallel bottom-up accumulation of per-node sample-set counts x[u],
//     integer atomics, a "last child to arrive continues upward" climb), and
//     then one warp replays the span's edge removals and insertions exactly
//     as the reference does, walking root paths.  Lanes hold the K count
//     components (lane k owns x[.][k]) and evaluate the summary terms (lane r
//     owns term r), exchanging counts by shuffles.
//   * Branch mode is accumulated as the change of the reference's running sum
//     (sum over nodes of branch_length * f(x)) within the span: per window the
//     span reports A = covered length and B = sum of (running-sum change so
//     far) * length, plus the span's total change D.  A fixed-order scan of D
//     over spans recovers the running sum at every span start from its value
//     on the first tree, and result[w] = sum_s RS_s * A_sw + B_sw.
//   * Site mode reads the integer counts at each mutation node (exact) and
//     sums f over the alleles of each site (trees.c:1525-1652).
//   * Every reduction runs in a fixed order, so results are bitwise
//     reproducible; FP64 accumulates windows and the cross-span scan.  With
//     TSG_PRECISION_F32_KAHAN the per-node summary changes are evaluated in
//     FP32 and summed with Kahan compensation.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "tsg_items.cuh"
#include "tsg_replay_compact.cuh"
#include "tsg_query.cuh"

namespace tsg {

// ----------------------------------------------------------------- summary
template <typename F>
__device__ __forceinline__ F term_value(int type, F xi, F xj, F xk, F xl, F ni, F nj, F nk,
    F nl, bool ieqj, F meanx)
{
    switch (type) {
        case TSG_DIVERSITY:
            return xi * (ni - xi) / (ni * (ni - 1));
        case TSG_SEGREGATING_SITES:
            return (F) (xi > 0) * (1 - xi / ni);
        case TSG_Y1:
            return xi * (ni - xi) * (ni - xi - 1) / (ni * (ni - 1) * (ni - 2));
        case TSG_DIVERGENCE:
            return xi * (nj - xj) / (ni * (nj - (F) (ieqj ? 1 : 0)));
        case TSG_Y2:
            return xi * (nj - xj) * (nj - xj - 1) / (ni * nj * (nj - 1));
        case TSG_F2:
            return (xi * (xi - 1) * (nj - xj) * (nj - xj - 1) - xi * (ni - xi) * (nj - xj) * xj)
                / (ni * (ni - 1) * nj * (nj - 1));
        case TSG_Y3:
            return xi * (nj - xj) * (nk - xk) / (ni * nj * nk);
        case TSG_F3:
            return (xi * (xi - 1) * (nj - xj) * (nk - xk) - xi * (ni - xi) * (nj - xj) * xk)
                / (ni * (ni - 1) * nj * nk);
        case TSG_F4:
            return (xi * xk * (nj - xj) * (nl - xl) - xi * xl * (nj - xj) * (nk - xk))
                / (ni * nj * nk * nl);
        case TSG_RELATEDNESS:
            return (xi / ni - meanx) * (xj / nj - meanx);
        case TSG_RELATEDNESS_NONCENTRED:
            return xi * xj / (ni * nj);
        default:
            return (F) NAN;
    }
}


// Evaluate f at the count vector held one component per lane (xk on lane k)
// for the terms of pass p (term index lane + 32 p).  All 32 lanes must call.
template <typename F>
__device__ __forceinline__ F eval_f(const QueryParams &q, F xk, int pass)
{
    const int lane = threadIdx.x & 31;
    F meanx = 0;
    if (q.need_mean) {
        F c = lane < q.K ? xk / (F) q.set_size[lane] : (F) 0;
        meanx = warp_sum(c) / (F) q.K;
    }
    const int r = lane + 32 * pass;
    const Term &t = q.term[r < q.R ? r : 0];
    F xi = __shfl_sync(0xffffffffu, xk, t.idx[0]);
    F xj = __shfl_sync(0xffffffffu, xk, t.idx[1]);
    F xkk = __shfl_sync(0xffffffffu, xk, t.idx[2]);
    F xl = __shfl_sync(0xffffffffu, xk, t.idx[3]);
    if (r >= q.R) {
        return 0;
    }
    return term_value<F>(t.type, xi, xj, xkk, xl, (F) q.set_size[t.idx[0]],
        (F) q.set_size[t.idx[1]], (F) q.set_size[t.idx[2]], (F) q.set_size[t.idx[3]],
        t.idx[0] == t.idx[1], meanx);
}

// The branch summary: f(x), plus f(total - x) when unpolarised
// (c/tskit/trees.c:1944-1972).
template <typename F>
__device__ __forceinline__ F eval_branch(const QueryParams &q, int xk_int, int pass)
{
    const int lane = threadIdx.x & 31;
    F xk = (F) xk_int;
    F v = eval_f<F>(q, xk, pass);
    if (!q.polarised) {
        F ck = lane < q.K ? (F) q.set_size[lane] - xk : (F) 0;
        v += eval_f<F>(q, ck, pass);
    }
    return v;
}

template <typename F>
struct Acc {
    F s, c;  // c: Kahan compensation (FP32 only; the FP64 specialisation has none)
    __device__ __forceinline__ void zero()
    {
        s = 0;
        c = 0;
    }
    __device__ __forceinline__ void add(F v)
    {
        if (sizeof(F) == sizeof(float)) {
            F y = v - c;
            F t = s + y;
            c = (t - s) - y;
            s = t;
        } else {
            s += v;
        }
    }
    __device__ __forceinline__ double value() const { return (double) s - (double) c; }
};

template <>
struct Acc<double> {
    double s;
    __device__ __forceinline__ void zero() { s = 0; }
    __device__ __forceinline__ void add(double v) { s += v; }
    __device__ __forceinline__ double value() const { return s; }
};

__device__ __forceinline__ int32_t node_weight(const TSView &ts, const QueryDev &qd, int32_t u,
    int k)
{
    int32_t si = ts.sample_index[u];
    return si >= 0 ? (int32_t) ((qd.sample_mask[si] >> k) & 1u) : 0;
}

// ------------------------------------------------------------------ sweep
template <typename F>
__global__ void __launch_bounds__(256) k_sweep(TSView ts, QueryParams q, QueryDev qd, WsDev w)
{
    __shared__ int s_span;
    __shared__ double s_red[8][64];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int64_t N = ts.num_nodes;
    const int K = q.K, KP = q.KP;
    int32_t *parent = w.parent + (int64_t) blockIdx.x * N;
    int32_t *nchild = w.nchild + (int64_t) blockIdx.x * N;
    int32_t *arrive = w.arrive + (int64_t) blockIdx.x * N;
    int32_t *x = w.x + (int64_t) blockIdx.x * N * KP;
    const double *time = ts.node_time;

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
        const int64_t a0 = ts.span_alive_off[s], a1 = ts.span_alive_off[s + 1];
        const int2 *alive = ts.span_alive;

        // ---- phase 0: reset every node the span can touch
        auto init_node = [&](int32_t u) {
            if (u < 0 || u >= N) {
                dev_error(w.err, DEV_NODE_OUT_OF_BOUNDS);
                return;
            }
            parent[u] = -1;
            nchild[u] = 0;
            arrive[u] = 0;
            for (int k = 0; k < K; k++) {
                x[(int64_t) u * KP + k] = node_weight(ts, qd, u, k);
            }
        };
        for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
            int2 pc = alive[i];
            init_node(pc.x);
            init_node(pc.y);
        }
        // the span also replays the transition into the next span's first tree
        // (its running-sum change belongs to this span's total)
        const int32_t t_end = t1 < ts.num_trees ? t1 + 1 : t1;
        const int32_t ie0 = ts.tree_in[t0 + 1 <= t1 ? t0 + 1 : t1], ie1 = ts.tree_in[t_end];
        for (int32_t i = ie0 + threadIdx.x; i < ie1; i += blockDim.x) {
            init_node(ts.ins_parent[i]);
            init_node(ts.ins_child[i]);
        }
        const int32_t m0 = ts.site_mut[ts.tree_sites[t0]], m1 = ts.site_mut[ts.tree_sites[t1]];
        for (int32_t m = m0 + threadIdx.x; m < m1; m += blockDim.x) {
            init_node(ts.mutation_node[m]);
        }
        __syncthreads();
        // ---- phase 1: link the tree at the span start
        for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
            int2 pc = alive[i];
            if (pc.x >= 0 && pc.x < N && pc.y >= 0 && pc.y < N) {
                parent[pc.y] = pc.x;
                atomicAdd(&nchild[pc.x], 1);
            }
        }
        __syncthreads();
        // ---- phase 2: bottom-up counts; the last child to finish climbs on
        for (int64_t i = a0 + threadIdx.x; i < a1; i += blockDim.x) {
            int32_t v = alive[i].y;
            if (v < 0 || v >= N || nchild[v] != 0) {
                continue;
            }
            for (int64_t iter = 0;; iter++) {
                int32_t p = parent[v];
                if (p < 0) {
                    break;
                }
                if (iter > N) {
                    dev_error(w.err, DEV_PATH_TOO_LONG);
                    break;
                }
                for (int k = 0; k < K; k++) {
                    int32_t xv = __ldcg(&x[(int64_t) v * KP + k]);
                    if (xv != 0) {
                        atomicAdd(&x[(int64_t) p * KP + k], xv);
                    }
                }
                __threadfence();
                if (atomicAdd(&arrive[p], 1) + 1 != nchild[p]) {
                    break;
                }
                __threadfence();
                v = p;
            }
        }
        __syncthreads();

        // ---- phase 3: running sum on the first tree (span 0 only), fixed order
        if (s == 0 && q.branch) {
            double part0 = 0, part1 = 0;
            for (int32_t i = warp; i < ts.tree_in[1]; i += nwarps) {
                int32_t c = ts.ins_child[i], p = ts.ins_parent[i];
                double bl = time[p] - time[c];
                int xc = lane < K ? __ldcg(&x[(int64_t) c * KP + lane]) : 0;
                part0 += bl * eval_branch<double>(q, xc, 0);
                if (q.R > 32) {
                    part1 += bl * eval_branch<double>(q, xc, 1);
                }
            }
            s_red[warp][lane] = part0;
            s_red[warp][lane + 32] = part1;
            __syncthreads();
            if (warp == 0) {
                double a = 0, b = 0;
                for (int j = 0; j < nwarps; j++) {
                    a += s_red[j][lane];
                    b += s_red[j][lane + 32];
                }
                if (lane < q.R) {
                    w.rs0[lane] = a;
                }
                if (lane + 32 < q.R) {
                    w.rs0[lane + 32] = b;
                }
            }
            __syncthreads();
        }

        // ---- phase 4: replay the span (warp 0)
        if (warp == 0) {
            const int R = q.R;
            const int passes = R > 32 ? 2 : 1;
            const int32_t wlo = qd.span_wlo[s];
            const int64_t woff = qd.span_woff[s];
            const int64_t nwin = qd.span_woff[s + 1] - woff;
            const double *win = qd.windows;
            for (int64_t j = lane; j < nwin; j += 32) {
                w.A[woff + j] = 0;
            }
            for (int64_t j = lane; j < nwin * R; j += 32) {
                if (q.branch) {
                    w.B[woff * R + j] = 0;
                }
                if (q.site) {
                    w.SITE[woff * R + j] = 0;
                }
            }
            __syncwarp();
            Acc<F> cum[2];
            cum[0].zero();
            cum[1].zero();
            int32_t wi = wlo;   // branch window cursor
            int32_t ws = wlo;   // site window cursor

            auto walk = [&](int32_t v, int xc, int sign) {
                for (int64_t iter = 0; v >= 0; iter++) {
                    if (iter > N || v >= N) {
                        dev_error(w.err, DEV_PATH_TOO_LONG);
                        break;
                    }
                    int32_t pv = parent[v];
                    int xo = lane < K ? x[(int64_t) v * KP + lane] : 0;
                    int xn = xo + sign * xc;
                    double tv = time[v];
                    double tp = pv >= 0 ? time[pv] : tv;
                    if (q.branch) {
                        F bl = (F) (tp - tv);
                        for (int p = 0; p < passes; p++) {
                            F d = eval_branch<F>(q, xn, p) - eval_branch<F>(q, xo, p);
                            cum[p].add(bl * d);
                        }
                    }
                    if (lane < K) {
                        x[(int64_t) v * KP + lane] = xn;
                    }
                    v = pv;
                }
            };

            // apply the removals (O order) and insertions (I order) entering tree t
            auto transition = [&](int32_t t) {
                for (int32_t i = ts.tree_out[t]; i < ts.tree_out[t + 1]; i++) {
                    int32_t c = ts.rem_child[i], p = ts.rem_parent[i];
                    int xc = lane < K ? x[(int64_t) c * KP + lane] : 0;
                    if (q.branch) {
                        F bl = (F) (time[p] - time[c]);
                        for (int pp = 0; pp < passes; pp++) {
                            cum[pp].add(-bl * eval_branch<F>(q, xc, pp));
                        }
                    }
                    parent[c] = -1;
                    walk(p, xc, -1);
                }
                for (int32_t i = ts.tree_in[t]; i < ts.tree_in[t + 1]; i++) {
                    int32_t c = ts.ins_child[i], p = ts.ins_parent[i];
                    parent[c] = p;
                    int xc = lane < K ? x[(int64_t) c * KP + lane] : 0;
                    if (q.branch) {
                        F bl = (F) (time[p] - time[c]);
                        for (int pp = 0; pp < passes; pp++) {
                            cum[pp].add(bl * eval_branch<F>(q, xc, pp));
                        }
                    }
                    walk(p, xc, +1);
                }
            };

            for (int32_t t = t0; t < t1; t++) {
                if (t > t0) {
                    transition(t);
                }
                const double tl = ts.breakpoints[t], tr = ts.breakpoints[t + 1];
                if (q.branch) {
                    while (wi < q.Wn && win[wi] < tr) {
                        double a = tl > win[wi] ? tl : win[wi];
                        double b = tr < win[wi + 1] ? tr : win[wi + 1];
                        double len = b - a;
                        int64_t li = woff + (wi - wlo);
                        if (lane == 0) {
                            w.A[li] += len;
                        }
                        for (int p = 0; p < passes; p++) {
                            int r = lane + 32 * p;
                            if (r < R) {
                                w.B[li * R + r] += cum[p].value() * len;
                            }
                        }
                        if (win[wi + 1] <= tr) {
                            wi++;
                        } else {
                            break;
                        }
                    }
                }
                if (q.site) {
                    for (int32_t site = ts.tree_sites[t]; site < ts.tree_sites[t + 1]; site++) {
                        const double pos = ts.site_position[site];
                        while (ws + 1 < q.Wn && win[ws + 1] <= pos) {
                            ws++;
                        }
                        const int32_t sm0 = ts.site_mut[site], sm1 = ts.site_mut[site + 1];
                        int32_t A = 1;
                        for (int32_t m = sm0; m < sm1; m++) {
                            A = max(A, ts.mutation_allele[m] + 1);
                        }
                        double val[2] = { 0, 0 };
                        for (int32_t a = q.polarised ? 1 : 0; a < A; a++) {
                            int st = (a == 0 && lane < K) ? (int) q.set_size[lane] : 0;
                            for (int32_t m = sm0; m < sm1; m++) {
                                int32_t u = ts.mutation_node[m];
                                int xm = lane < K ? x[(int64_t) u * KP + lane] : 0;
                                if (ts.mutation_allele[m] == a) {
                                    st += xm;
                                }
                                if (ts.mutation_alt[m] == a) {
                                    st -= xm;
                                }
                            }
                            for (int p = 0; p < passes; p++) {
                                val[p] += eval_f<double>(q, (double) st, p);
                            }
                        }
                        int64_t li = woff + (ws - wlo);
                        for (int p = 0; p < passes; p++) {
                            int r = lane + 32 * p;
                            if (r < R) {
                                w.SITE[li * R + r] += val[p];
                            }
                        }
                    }
                }
            }
            if (q.branch) {
                if (t1 < ts.num_trees) {
                    transition(t1);
                }
                for (int p = 0; p < passes; p++) {
                    int r = lane + 32 * p;
                    if (r < R) {
                        w.D[(int64_t) s * R + r] = cum[p].value();
                    }
                }
            }
        }
        __syncthreads();
    }
}


// Item pipeline forms: node state in shared memory (16-bit counts and ids)
// or in a per-CTA slice of global memory (32-bit counts and ids); the
// replay values its items itself when the query has branch terms.
static void *replay_kernel(int W, int KQ, const QueryParams &p)
{
    const int form = (W == 16 ? 0 : 2) + (KQ == 1 ? 0 : 1);
    if (p.branch) {
        if (p.f32) {
            return p.polarised ? replay_eval_fn_f32_pol(form) : replay_eval_fn_f32_unpol(form);
        }
        return p.polarised ? replay_eval_fn_f64_pol(form) : replay_eval_fn_f64_unpol(form);
    }
    switch (form) {
        case 0: return (void *) k_replay_items<16, 1, uint16_t, float, false, false>;
        case 1: return (void *) k_replay_items<16, 2, uint16_t, float, false, false>;
        case 2: return (void *) k_replay_items<32, 1, int32_t, float, false, false>;
        default: return (void *) k_replay_items<32, 2, int32_t, float, false, false>;
    }
}

// The compact replay (tsg_replay_compact.cuh).
static void *compact_kernel(int KQ)
{
    return KQ == 1 ? (void *) k_replay_compact<1> : (void *) k_replay_compact<2>;
}

// blocks of k_compact_rows: a warp per (span, chunk of rows)
static int64_t compact_rows_blocks(const tsg_treeseq_t *ts)
{
    const int64_t warps = ts->v.c_num_spans * compact_row_chunks(ts->v.num_samples);
    return std::min<int64_t>((warps + TSG_ROWS_THREADS / 32 - 1) / (TSG_ROWS_THREADS / 32),
        1 << 20);
}


// bytes of one span's node state: packed counts and parent ids (node times
// come from the span plan, seek counters from per-CTA scratch)
static int64_t span_state_bytes(int64_t L, int W, int KQ)
{
    return L * 8 * KQ + L * (W == 16 ? 2 : 4);
}

// Dynamic shared memory a block of `kernel` may have: the device's opt-in
// maximum less the kernel's static shared memory.
static int64_t smem_budget(const void *kernel)
{
    return kernel_smem_budget(kernel);
}

static int grid_for(int64_t n, int block = 256)
{
    int64_t g = (n + block - 1) / block;
    return (int) std::max<int64_t>(1, std::min<int64_t>(g, 65535LL * 4));
}

static int64_t align_up(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

// bytes of the item replay's span state (counts and parent entries)
static int64_t replay_state_bytes(int64_t L, int W, int KQ)
{
    return align_up(span_state_bytes(L, W, KQ), 8);
}

}  // namespace tsg

using namespace tsg;

struct tsg_query {
    const tsg_treeseq_t *ts;
    QueryParams p;
    QueryDev d;
    void *dbuf;              // device copy of per-query arrays (owned), or null
    std::vector<char> blob;  // host image of the per-query arrays
    int64_t off[12];         // offsets in the image: mask, windows, wlo, woff, wsl, wsh, wsite,
                             // time windows (allele frequency spectrum)
    cudaEvent_t ev_start, ev_stop;  // optional events around the sweep kernel
    cudaEvent_t ev_rstart = nullptr, ev_rstop = nullptr;  // ... around the replay kernel
    int64_t total_span_windows;
    int64_t total_seg_windows;  // window segments x windows they overlap (item pipeline)
    int64_t num_slots;
    int64_t ws_bytes;
    bool smem;               // item pipeline (either form); else the general sweep
    bool gstate;             // item pipeline with node state in global memory
    bool compact_ok;         // the compact replay serves when the tree sequence has its plan
    int64_t c_rows_cap;      // compact spans and sample-range endpoints the workspace's
    int64_t c_ep_cap;        // arrays hold (the plan's when the query was prepared)
    int W, KQ;               // count field width, 64-bit count words per node
    int64_t smem_bytes, smem_grid, slot_bytes;
    int span_normalise;
    uint32_t options;
    int kind;                // TSG_KIND_STATS, TSG_KIND_AFS or TSG_KIND_MATVEC
    AfsParams afs;           // allele frequency spectrum (device pointers bound at launch)
    int64_t afs_bins;        // windows x time windows x afs_size
    MvParams mv;             // relatedness vector (device pointers bound at launch)
    int64_t mv_grid;
    int64_t mv_pairs;        // (group, window) partial blocks
    const double *weights;   // relatedness vector: device weights (num_samples x W)
};

#define TSG_KIND_STATS 0
#define TSG_KIND_AFS 1
#define TSG_KIND_MATVEC 2

namespace tsg {

// whether the compact replay serves a launch of q: the tree sequence has a
// compact plan and q's row arrays hold its spans (a plan rebuilt with more
// spans after q was prepared leaves q on the general replay)
static bool compact_serves(const tsg_query_t *q)
{
    return q->compact_ok && q->ts->v.c_num_spans > 0 && q->ts->v.c_num_spans <= q->c_rows_cap
        && q->ts->h_compact_endpoints <= q->c_ep_cap;
}

// Check the sample sets (c/tskit/trees.c:2114-2149 and the duplicate check of
// 2174-2220) and build per-sample membership masks.
static int check_sample_sets(const tsg_treeseq_t *ts, uint64_t K, const uint64_t *sizes,
    const int32_t *sets, std::vector<uint32_t> &mask)
{
    if (K == 0) {
        return TSG_ERR_INSUFFICIENT_SAMPLE_SETS;
    }
    if (K > TSG_MAX_SAMPLE_SETS) {
        return TSG_ERR_TOO_MANY_SAMPLE_SETS;
    }
    mask.assign((size_t) ts->v.num_samples, 0u);
    uint64_t j = 0;
    for (uint64_t k = 0; k < K; k++) {
        if (sizes[k] == 0) {
            return TSG_ERR_EMPTY_SAMPLE_SET;
        }
        for (uint64_t l = 0; l < sizes[k]; l++) {
            int32_t u = sets[j++];
            if (u < 0 || u >= ts->v.num_nodes) {
                return TSG_ERR_NODE_OUT_OF_BOUNDS;
            }
            int32_t si = ts->h_sample_index[(size_t) u];
            if (si < 0) {
                return TSG_ERR_BAD_SAMPLES;
            }
            if (mask[(size_t) si] & (1u << k)) {
                return TSG_ERR_DUPLICATE_SAMPLE;
            }
            mask[(size_t) si] |= 1u << k;
        }
    }
    return 0;
}

// trees.c:1244-1286 with TSK_REQUIRE_FULL_SPAN
static int check_windows(const tsg_treeseq_t *ts, uint64_t Wn, const double *windows)
{
    if (Wn < 1) {
        return TSG_ERR_BAD_NUM_WINDOWS;
    }
    if (windows[0] != 0 || windows[Wn] != ts->v.sequence_length) {
        return TSG_ERR_BAD_WINDOWS;
    }
    for (uint64_t j = 0; j < Wn; j++) {
        if (!(windows[j] < windows[j + 1])) {
            return TSG_ERR_BAD_WINDOWS;
        }
    }
    return 0;
}

static int tuple_width(int32_t type)
{
    switch (type) {
        case TSG_DIVERSITY:
        case TSG_SEGREGATING_SITES:
        case TSG_Y1:
            return 1;
        case TSG_DIVERGENCE:
        case TSG_Y2:
        case TSG_F2:
        case TSG_RELATEDNESS:
        case TSG_RELATEDNESS_NONCENTRED:
            return 2;
        case TSG_Y3:
        case TSG_F3:
            return 3;
        case TSG_F4:
            return 4;
        default:
            return 0;
    }
}

}  // namespace tsg

extern "C" {

int tsg_query_free(tsg_query_t *q)
{
    if (q != nullptr) {
        // stream-ordered: no device-wide synchronisation (a serving loop
        // frees queries while other streams run)
        if (q->dbuf != nullptr) {
            cudaFreeAsync(q->dbuf, 0);
        }
        delete q;
    }
    return 0;
}

int64_t tsg_query_workspace_bytes(const tsg_query_t *q) { return q->ws_bytes; }

int64_t tsg_query_result_size(const tsg_query_t *q)
{
    if (q->kind == TSG_KIND_AFS) {
        return q->afs_bins;
    }
    if (q->kind == TSG_KIND_MATVEC) {
        return (int64_t) q->mv.Wn * q->mv.nf * q->mv.W;
    }
    return (int64_t) q->p.Wn * q->p.R * ((q->p.branch ? 1 : 0) + (q->p.site ? 1 : 0));
}

}  // extern "C"

namespace tsg {

static void query_bind(tsg_query_t *q, void *dev)
{
    char *b = (char *) dev;
    q->d.sample_mask = (const uint32_t *) (b + q->off[0]);
    q->d.windows = (const double *) (b + q->off[1]);
    q->d.span_wlo = (const int32_t *) (b + q->off[2]);
    q->d.span_woff = (const int64_t *) (b + q->off[3]);
    q->d.win_span_lo = (const int32_t *) (b + q->off[4]);
    q->d.win_span_hi = (const int32_t *) (b + q->off[5]);
    q->d.win_site_lo = (const int32_t *) (b + q->off[6]);
    q->d.seg_wlo = (const int32_t *) (b + q->off[8]);
    q->d.seg_woff = (const int64_t *) (b + q->off[9]);
    q->d.win_seg_lo = (const int32_t *) (b + q->off[10]);
    q->d.win_seg_hi = (const int32_t *) (b + q->off[11]);
    q->d.node_mask = nullptr;
    if (q->kind == TSG_KIND_AFS) {
        q->afs.windows = q->d.windows;
        q->afs.time_windows = (const double *) (b + q->off[7]);
    }
    if (q->kind == TSG_KIND_MATVEC) {
        // windows, focal, group_span, group_wlo, pair_off, win_glo, win_ghi
        q->mv.windows = (const double *) (b + q->off[1]);
        q->mv.focal = (const int32_t *) (b + q->off[2]);
        q->mv.group_span = (const int32_t *) (b + q->off[3]);
        q->mv.group_wlo = (const int32_t *) (b + q->off[4]);
        q->mv.pair_off = (const int64_t *) (b + q->off[5]);
        q->mv.win_glo = (const int32_t *) (b + q->off[6]);
        q->mv.win_ghi = (const int32_t *) (b + q->off[7]);
    }
}

// Overlap tables of windows and units (runs of consecutive trees
// [ut[u], ut[u + 1])): per unit its first window and its offset into the
// unit-window arrays; per window its first and last overlapping unit.
struct WindowUnits {
    std::vector<int32_t> wlo, wsl, wsh;
    std::vector<int64_t> woff;
};

static void window_units(const std::vector<double> &bp, const int32_t *ut, int64_t NU,
    const double *windows, uint64_t Wn, WindowUnits &o)
{
    std::vector<int32_t> whi((size_t) NU);
    o.wlo.assign((size_t) NU, 0);
    o.woff.assign((size_t) NU + 1, 0);
    // the units' ends and the windows both increase: one merge walk finds
    // every unit's first window (the upper bound of its start) and last
    // window (the lower bound of its end) -- the binary searches they replace
    // cost most of a query's preparation on thousands of units
    const int64_t nw = (int64_t) Wn + 1;
    int64_t ub = 0, lb = 0;
    for (int64_t u = 0; u < NU; u++) {
        double b0 = bp[(size_t) ut[u]], b1 = bp[(size_t) ut[u + 1]];
        while (ub < nw && windows[ub] <= b0) {
            ub++;
        }
        while (lb < nw && windows[lb] < b1) {
            lb++;
        }
        int64_t lo = ub - 1;
        int64_t hi = lb - 1;
        lo = std::max<int64_t>(0, std::min<int64_t>(lo, (int64_t) Wn - 1));
        hi = std::max<int64_t>(lo, std::min<int64_t>(hi, (int64_t) Wn - 1));
        o.wlo[(size_t) u] = (int32_t) lo;
        whi[(size_t) u] = (int32_t) hi;
        o.woff[(size_t) u + 1] = o.woff[(size_t) u] + (hi - lo + 1);
    }
    o.wsl.assign((size_t) Wn, 0);
    o.wsh.assign((size_t) Wn, 0);
    int64_t u = 0;
    for (int64_t wdx = 0; wdx < (int64_t) Wn; wdx++) {
        while (u < NU && whi[(size_t) u] < wdx) {
            u++;
        }
        o.wsl[(size_t) wdx] = (int32_t) u;
        int64_t e = u;
        while (e + 1 < NU && o.wlo[(size_t) e + 1] <= wdx) {
            e++;
        }
        o.wsh[(size_t) wdx] = (int32_t) e;
    }
}

// Validate the query and build its host image; the device copy is made by
// the caller (its own allocation, or the tree sequence's staging buffer).
static int query_build(tsg_query_t **out, const tsg_treeseq_t *ts, uint64_t K,
    const uint64_t *sizes, const int32_t *sets, uint64_t R, const tsg_output_t *outputs,
    uint64_t Wn, const double *windows, uint32_t options)
{
    NvtxRange nvtx("tsg.query_build");
    *out = nullptr;
    int ret;
    const uint32_t modes = options & (TSG_STAT_SITE | TSG_STAT_BRANCH | TSG_STAT_NODE);
    bool site = options & TSG_STAT_SITE, branch = options & TSG_STAT_BRANCH;
    if (options & TSG_STAT_NODE) {
        return TSG_ERR_UNSUPPORTED_STAT_MODE;
    }
    if (options & TSG_STAT_BOTH_MODES) {
        site = branch = true;
    } else {
        if (modes == 0) {
            site = true;  // default mode is site (trees.c:2046-2049)
        }
        if (site && branch) {
            return TSG_ERR_MULTIPLE_STAT_MODES;
        }
    }
    if (R < 1) {
        return TSG_ERR_BAD_RESULT_DIMS;
    }
    if (R > TSG_MAX_OUTPUTS) {
        return TSG_ERR_TOO_MANY_OUTPUTS;
    }
    double default_windows[2] = { 0, ts->v.sequence_length };
    if (windows == nullptr) {
        Wn = 1;
        windows = default_windows;
    } else if ((ret = check_windows(ts, Wn, windows)) != 0) {
        return ret;
    }
    std::vector<uint32_t> mask;
    if ((ret = check_sample_sets(ts, K, sizes, sets, mask)) != 0) {
        return ret;
    }
    // c/tskit/trees.c:1383-1386
    if (branch && (ts->options & TSG_TIME_UNCALIBRATED)
        && !(options & TSG_STAT_ALLOW_TIME_UNCALIBRATED)) {
        return TSG_ERR_TIME_UNCALIBRATED;
    }
    tsg_query_t *q = new tsg_query_t();
    std::memset(&q->p, 0, sizeof(q->p));
    q->kind = TSG_KIND_STATS;
    q->dbuf = nullptr;
    q->ev_start = nullptr;
    q->ev_stop = nullptr;
    q->ts = ts;
    q->options = options;
    q->span_normalise = !!(options & TSG_STAT_SPAN_NORMALISE);
    QueryParams &p = q->p;
    p.K = (int32_t) K;
    p.KP = K <= 1 ? 1 : K <= 2 ? 2 : K <= 4 ? 4 : K <= 8 ? 8 : K <= 16 ? 16 : 32;
    p.R = (int32_t) R;
    p.Wn = (int32_t) Wn;
    p.branch = branch;
    p.site = site;
    p.polarised = !!(options & TSG_STAT_POLARISED);
    p.f32 = !!(options & TSG_PRECISION_F32_KAHAN);
    p.spin_limit = (options & TSG_TEST_WAIT_EXPIRES) ? 0u : (uint32_t) TSG_REPLAY_SPIN_LIMIT;
    for (uint64_t k = 0; k < K; k++) {
        p.set_size[k] = (double) sizes[k];
        p.set_size_i[k] = (int32_t) sizes[k];
        if (sizes[k] >= ((uint64_t) 1 << 23)) {
            p.f32 = 0;  // the FP32 form needs every count exact in FP32
        }
    }
    for (uint64_t r = 0; r < R; r++) {
        int wdt = tuple_width(outputs[r].type);
        if (wdt == 0) {
            delete q;
            return TSG_ERR_BAD_PARAM_VALUE;
        }
        p.term[r].type = outputs[r].type;
        for (int j = 0; j < 4; j++) {
            int32_t ix = j < wdt ? outputs[r].idx[j] : 0;
            if (ix < 0 || ix >= (int32_t) K) {
                delete q;
                return TSG_ERR_BAD_SAMPLE_SET_INDEX;
            }
            p.term[r].idx[j] = ix;
        }
        if (outputs[r].type == TSG_RELATEDNESS) {
            p.need_mean = 1;
        }
        // reciprocal denominators of the terms (the summary functions of
        // c/tskit/trees.c divide by these products of set sizes)
        const int32_t *ix = p.term[r].idx;
        const double ni = (double) sizes[ix[0]], nj = (double) sizes[ix[1]];
        const double nk = (double) sizes[ix[2]], nl = (double) sizes[ix[3]];
        double den = 1;
        switch (outputs[r].type) {
            case TSG_DIVERSITY:
                den = ni * (ni - 1);
                break;
            case TSG_SEGREGATING_SITES:
                den = ni;
                break;
            case TSG_Y1:
                den = ni * (ni - 1) * (ni - 2);
                break;
            case TSG_DIVERGENCE:
                den = ni * (nj - (ix[0] == ix[1] ? 1 : 0));
                break;
            case TSG_Y2:
                den = ni * nj * (nj - 1);
                break;
            case TSG_F2:
                den = ni * (ni - 1) * nj * (nj - 1);
                break;
            case TSG_Y3:
                den = ni * nj * nk;
                break;
            case TSG_F3:
                den = ni * (ni - 1) * nj * nk;
                break;
            case TSG_F4:
                den = ni * nj * nk * nl;
                break;
            case TSG_RELATEDNESS_NONCENTRED:
                den = ni * nj;
                break;
            default:
                den = 1;
        }
        p.inv[r] = 1.0 / den;
    }
    for (uint64_t k = 0; k < K; k++) {
        p.inv_size[k] = 1.0 / (double) sizes[k];
    }
    // integer site summaries when every term is a polynomial and the set
    // sizes keep its products within 64 bits
    p.site_int = 1;
    for (uint64_t k = 0; k < K; k++) {
        p.site_int &= sizes[k] < ((uint64_t) 1 << 15) ? 1 : 0;
    }
    for (uint64_t r = 0; r < R; r++) {
        p.site_int &= outputs[r].type != TSG_RELATEDNESS ? 1 : 0;
    }
    // terms grouped by type, in term order within a group
    p.ngroups = 0;
    {
        int32_t at = 0;
        std::vector<bool> used((size_t) R, false);
        for (uint64_t r = 0; r < R; r++) {
            if (used[(size_t) r]) {
                continue;
            }
            p.gfirst[p.ngroups++] = at;
            for (uint64_t u = r; u < R; u++) {
                if (!used[(size_t) u] && outputs[u].type == outputs[r].type) {
                    used[(size_t) u] = true;
                    p.gterm[at++] = (int32_t) u;
                }
            }
        }
        p.gfirst[p.ngroups] = at;
        p.gwpb = 0;
        for (int g = 0; g < p.ngroups; g++) {
            const int gs = p.gfirst[g + 1] - p.gfirst[g];
            const int nw = (TSG_EVAL_BLOCK * gs + 31) / 32;
            for (int k = 0; k < nw && p.gwpb < TSG_MAX_OUTPUTS; k++) {
                p.gw_group[p.gwpb] = g;
                p.gw_k[p.gwpb] = k;
                p.gwpb++;
            }
        }
    }
    p.inv_K = 1.0 / (double) K;
    for (uint64_t k = 0; k < K; k++) {
        p.set_size_f[k] = (float) p.set_size[k];
        p.inv_size_f[k] = (float) p.inv_size[k];
    }
    for (uint64_t r = 0; r < R; r++) {
        p.inv_f[r] = (float) p.inv[r];
    }
    p.inv_K_f = (float) p.inv_K;

    // span <-> window and segment <-> window overlap tables (host; spans,
    // segments and windows are few)
    const int64_t NS = ts->v.num_spans, NG = ts->v.num_segs;
    WindowUnits su, gu;
    window_units(ts->h_breakpoints, ts->h_span_tree.data(), NS, windows, Wn, su);
    window_units(ts->h_breakpoints, ts->h_seg_tree.data(), NG, windows, Wn, gu);
    q->total_span_windows = su.woff[(size_t) NS];
    q->total_seg_windows = gu.woff[(size_t) NG];

    // device copy of the per-query arrays, one allocation
    const int64_t n = ts->v.num_samples;
    int64_t off_mask = 0;
    int64_t off_win = align_up(off_mask + std::max<int64_t>(n, 1) * 4, 256);
    int64_t off_wlo = align_up(off_win + ((int64_t) Wn + 1) * 8, 256);
    int64_t off_woff = align_up(off_wlo + NS * 4, 256);
    int64_t off_wsl = align_up(off_woff + (NS + 1) * 8, 256);
    int64_t off_wsh = align_up(off_wsl + (int64_t) Wn * 4, 256);
    int64_t off_wsite = align_up(off_wsh + (int64_t) Wn * 4, 256);
    int64_t off_gwlo = align_up(off_wsite + ((int64_t) Wn + 1) * 4, 256);
    int64_t off_gwoff = align_up(off_gwlo + NG * 4, 256);
    int64_t off_gwsl = align_up(off_gwoff + (NG + 1) * 8, 256);
    int64_t off_gwsh = align_up(off_gwsl + (int64_t) Wn * 4, 256);
    int64_t total = align_up(off_gwsh + (int64_t) Wn * 4, 256);
    std::vector<int32_t> wsite((size_t) Wn + 1);
    {
        // each window's first site: a branch-free binary search per window
        // (conditional moves instead of unpredictable branches)
        const auto &sp = ts->h_site_position;
        const int64_t S = (int64_t) sp.size();
        for (uint64_t wdx = 0; wdx <= Wn; wdx++) {
            const double x = windows[wdx];
            int64_t base = 0, len = S;
            while (len > 1) {
                const int64_t half = len >> 1;
                base = sp[(size_t) (base + half - 1)] < x ? base + half : base;
                len -= half;
            }
            wsite[(size_t) wdx] = (int32_t) (base + (len == 1 && sp[(size_t) base] < x ? 1 : 0));
        }
    }
    q->blob.assign((size_t) total, 0);
    char *h = q->blob.data();
    std::memcpy(h + off_mask, mask.data(), (size_t) n * 4);
    std::memcpy(h + off_win, windows, ((size_t) Wn + 1) * 8);
    std::memcpy(h + off_wlo, su.wlo.data(), (size_t) NS * 4);
    std::memcpy(h + off_woff, su.woff.data(), ((size_t) NS + 1) * 8);
    std::memcpy(h + off_wsl, su.wsl.data(), (size_t) Wn * 4);
    std::memcpy(h + off_wsh, su.wsh.data(), (size_t) Wn * 4);
    std::memcpy(h + off_wsite, wsite.data(), ((size_t) Wn + 1) * 4);
    std::memcpy(h + off_gwlo, gu.wlo.data(), (size_t) NG * 4);
    std::memcpy(h + off_gwoff, gu.woff.data(), ((size_t) NG + 1) * 8);
    std::memcpy(h + off_gwsl, gu.wsl.data(), (size_t) Wn * 4);
    std::memcpy(h + off_gwsh, gu.wsh.data(), (size_t) Wn * 4);
    q->off[8] = off_gwlo;
    q->off[9] = off_gwoff;
    q->off[10] = off_gwsl;
    q->off[11] = off_gwsh;
    q->off[6] = off_wsite;
    q->off[0] = off_mask;
    q->off[1] = off_win;
    q->off[2] = off_wlo;
    q->off[3] = off_woff;
    q->off[4] = off_wsl;
    q->off[5] = off_wsh;

    // workspace: per-slot node state + per-span accumulators
    int blocks_per_sm = 0;
    if (p.f32) {
        blocks_per_sm = occupancy_blocks((const void *) k_sweep<float>, 256, (size_t) (0));
    } else {
        blocks_per_sm = occupancy_blocks((const void *) k_sweep<double>, 256, (size_t) (0));
    }
    int64_t slots = (int64_t) std::max(1, blocks_per_sm) * std::max(1, device_count_sms());
    const int64_t per_slot = align_up(ts->v.num_nodes * (12 + 4 * (int64_t) p.KP), 256);
    const int64_t budget = (int64_t) 24 << 30;  // node state at most 24 GiB
    slots = std::min<int64_t>(slots, std::max<int64_t>(1, budget / std::max<int64_t>(per_slot, 1)));
    slots = std::min<int64_t>(slots, std::max<int64_t>(NS, 1));
    q->num_slots = slots;
    p.num_slots = (int32_t) slots;

    // item pipeline when the terms fit its accumulators: node state in shared
    // memory when it fits (16-bit counts and ids, up to 8 sets), else in
    // global memory (32-bit counts and ids, up to 4 sets)
    uint64_t max_size = 0;
    for (uint64_t k = 0; k < K; k++) {
        max_size = std::max<uint64_t>(max_size, sizes[k]);
    }
    const int64_t L = std::max<int64_t>(ts->v.max_local, 1);
    const bool forced = (options & TSG_FORCE_GLOBAL_SWEEP) != 0;
    const bool items_ok = !forced && (int64_t) R <= TSG_ITEM_RMAX && ts->max_children < 65535;
    q->smem = false;
    q->gstate = false;
    q->W = 16;
    q->KQ = (int) (((int64_t) K + 3) / 4);
    q->smem_bytes = align_up(replay_state_bytes(L, 16, q->KQ), 16);
    q->slot_bytes = 0;
    if (items_ok && K <= 8 && max_size <= 65535 && ts->v.max_local <= 32766
        && q->smem_bytes <= smem_budget(replay_kernel(16, q->KQ, p))
        && !(options & TSG_FORCE_GLOBAL_STATE)) {
        q->smem = true;
    } else if (items_ok && K <= 4 && ts->v.max_local < INT32_MAX) {
        q->smem = true;
        q->gstate = true;
        q->W = 32;
        q->KQ = K <= 2 ? 1 : 2;
        q->smem_bytes = 0;
        q->slot_bytes = align_up(replay_state_bytes(L, 32, q->KQ), 256);
    }
    const int64_t KQ = q->KQ;
    if (q->smem) {
        int per_sm = 0;
        void *fn = replay_kernel(q->W, q->KQ, p);
        if (!q->gstate) {
            // a cap, not a reservation: every query of every tree sequence fits
            // (the replay without evaluation serves general_stat's prepare step)
            QueryParams plain;
            std::memset(&plain, 0, sizeof(plain));
            void *fn0 = replay_kernel(q->W, q->KQ, plain);
            allow_max_dynamic_smem(fn);
            allow_max_dynamic_smem(fn0);
        }
        per_sm = occupancy_blocks((const void *) fn, 512, (size_t) ((size_t) q->smem_bytes));
        int64_t grid = (int64_t) std::max(per_sm, 1) * std::max(1, device_count_sms());
        if (q->gstate) {
            // node state of every resident CTA at most 8 GiB
            grid = std::min<int64_t>(grid, std::max<int64_t>(1, ((int64_t) 8 << 30) / q->slot_bytes));
        }
        q->smem_grid = std::min<int64_t>(grid, std::max<int64_t>(NS, 1));
        slots = 0;  // no per-slot node arrays of the general sweep
        q->num_slots = 0;
    }
    q->compact_ok = q->smem && !q->gstate && q->W == 16 && q->KQ <= 2;
    q->c_rows_cap = q->compact_ok ? ts->v.c_num_spans : 0;
    q->c_ep_cap = q->compact_ok ? ts->h_compact_endpoints : 0;
    if (q->compact_ok) {
        void *fn = compact_kernel(q->KQ);
        allow_max_dynamic_smem(fn);
    }
    // window accumulators: per span (general sweep) or per segment (item
    // pipeline)
    const int64_t TSW = std::max(q->total_span_windows, q->total_seg_windows);
    const int64_t NU = std::max(NS, NG);
    int64_t bytes = 0;
    bytes += align_up(slots * ts->v.num_nodes * 4, 256) * 3;          // parent, nchild, arrive
    bytes += align_up(slots * ts->v.num_nodes * 4 * p.KP, 256);       // x
    bytes += align_up(TSW * 8, 256);                                  // A
    bytes += align_up(TSW * R * 8, 256) * 2;                          // B, SITE
    bytes += align_up(NU * R * 8, 256) * 2;                           // D, RS
    bytes += align_up((int64_t) R * 8, 256);                          // rs0
    if (q->smem) {
        const int64_t item_bytes = KQ == 1 ? (int64_t) sizeof(Item<1>) : (int64_t) sizeof(Item<2>);
        bytes += align_up((p.branch ? ts->v.num_items : 0) * item_bytes, 256);  // items
        bytes += align_up((p.branch ? ts->v.num_items : 0) * (p.f32 ? 8 : 16), 256);  // bl
        bytes += align_up(ts->v.num_mutations * 8 * KQ, 256);                   // mcnt
        bytes += align_up(ts->v.num_chunks * R * 8, 256);                        // dD (per chunk)
        bytes += align_up(ts->v.num_nodes * 4, 256);                             // node_mask
        bytes += align_up((p.site ? ts->v.num_sites : 0) * R * 8, 256);          // site_val
        bytes += align_up((p.site && p.site_int ? (int64_t) Wn : 0) * R * 16, 256);    // site_acc
        bytes += align_up((int64_t) Wn * R * 8, 256);                            // site_win
        bytes += align_up(q->gstate ? q->smem_grid * q->slot_bytes : 0, 256);    // node state
        bytes += align_up(q->smem_grid * L * 4, 256);                            // seek counters
        bytes += align_up((p.branch ? (int64_t) Wn << K : 0) * TSG_FX_LIMBS * 8 * 3, 256);  // leaf areas
        bytes += align_up((p.branch ? (int64_t) Wn << K : 0) * 8, 256);          // leaf_dbl
        bytes += align_up((int64_t) Wn * R * 8, 256);                            // leaf_win
        bytes += align_up(q->compact_ok ? (ts->v.num_samples + 1) * 16 : 0, 256); // cp0
        bytes += align_up(q->c_ep_cap * 8 * KQ, 256);                                  // c_pep
        bytes += align_up(q->c_rows_cap * compact_row_chunks(ts->v.num_samples) * 8 * KQ, 256);
    }
    bytes += 256;                                                     // err, counter
    q->ws_bytes = bytes;
    *out = q;
    return 0;
}

// trees.c:1289-1313
static int check_time_windows(uint64_t TW, const double *tw)
{
    if (TW < 1) {
        return TSG_ERR_BAD_TIME_WINDOWS_DIM;
    }
    if (tw[0] != 0.0) {
        return TSG_ERR_BAD_TIME_WINDOWS;
    }
    for (uint64_t j = 0; j < TW; j++) {
        if (tw[j] >= tw[j + 1]) {
            return TSG_ERR_BAD_TIME_WINDOWS;
        }
    }
    return 0;
}

// Workspace layout of an allele frequency spectrum query.
struct AfsLayout {
    int64_t node_mask, mcnt, state, seekcnt, acc, err, total;
};

static AfsLayout afs_layout(const tsg_query_t *q)
{
    const TSView &v = q->ts->v;
    AfsLayout l;
    int64_t off = 0;
    l.node_mask = off;
    off += align_up(v.num_nodes * 4, 256);
    l.mcnt = off;
    off += align_up(q->p.site ? v.num_mutations * 8 * q->KQ : 0, 256);
    l.state = off;
    off += align_up(q->gstate ? q->smem_grid * q->slot_bytes : 0, 256);
    l.seekcnt = off;
    off += align_up(q->smem_grid * std::max<int64_t>(v.max_local, 1) * 4, 256);
    l.acc = off;
    off += align_up(q->p.branch ? q->afs_bins * TSG_FX_LIMBS * 8 : 0, 256);
    l.err = off;
    off += 256;
    l.total = off;
    return l;
}

// Validate an allele frequency spectrum query (the checks and their order
// of c/tskit/trees.c:3830-3900) and build its host image.
static int afs_build(tsg_query_t **out, const tsg_treeseq_t *ts, uint64_t K,
    const uint64_t *sizes, const int32_t *sets, uint64_t Wn, const double *windows,
    uint64_t TW, const double *time_windows, uint32_t options)
{
    *out = nullptr;
    int ret;
    if (options & TSG_STAT_NODE) {
        return TSG_ERR_UNSUPPORTED_STAT_MODE;
    }
    bool site = options & TSG_STAT_SITE, branch = options & TSG_STAT_BRANCH;
    if (!site && !branch) {
        site = true;
    }
    if (site && branch) {
        return TSG_ERR_MULTIPLE_STAT_MODES;
    }
    double default_windows[2] = { 0, ts->v.sequence_length };
    if (windows == nullptr) {
        Wn = 1;
        windows = default_windows;
    } else if ((ret = check_windows(ts, Wn, windows)) != 0) {
        return ret;
    }
    double default_tw[2] = { 0, INFINITY };
    if (time_windows == nullptr) {
        TW = 1;
        time_windows = default_tw;
    } else {
        if ((ret = check_time_windows(TW, time_windows)) != 0) {
            return ret;
        }
        if (site && !(time_windows[0] == 0.0 && std::isinf((float) time_windows[1]))) {
            return TSG_ERR_UNSUPPORTED_STAT_MODE;
        }
    }
    std::vector<uint32_t> mask;
    if ((ret = check_sample_sets(ts, K, sizes, sets, mask)) != 0) {
        return ret;
    }
    // c/tskit/trees.c:3723-3726
    if (branch && (ts->options & TSG_TIME_UNCALIBRATED)
        && !(options & TSG_STAT_ALLOW_TIME_UNCALIBRATED)) {
        return TSG_ERR_TIME_UNCALIBRATED;
    }
    if (K > TSG_AFS_KMAX) {
        return TSG_ERR_TOO_MANY_SAMPLE_SETS;
    }
    // the last count field: every sample of the tree sequence
    for (auto &m : mask) {
        m |= 1u << K;
    }
    const int64_t n = ts->v.num_samples;
    int64_t afs_size = 1;
    for (uint64_t k = 0; k < K; k++) {
        if (afs_size > ((int64_t) 1 << 40) / (int64_t) (sizes[k] + 1)) {
            return TSG_ERR_NO_MEMORY;
        }
        afs_size *= (int64_t) (sizes[k] + 1);
    }
    const int64_t bins = (int64_t) Wn * (int64_t) TW * afs_size;

    tsg_query_t *q = new tsg_query_t();
    std::memset(&q->p, 0, sizeof(q->p));
    std::memset(&q->afs, 0, sizeof(q->afs));
    q->kind = TSG_KIND_AFS;
    q->dbuf = nullptr;
    q->ev_start = nullptr;
    q->ev_stop = nullptr;
    q->ts = ts;
    q->options = options;
    q->span_normalise = !!(options & TSG_STAT_SPAN_NORMALISE);
    q->total_span_windows = 0;
    q->total_seg_windows = 0;
    q->num_slots = 0;
    q->afs_bins = bins;
    QueryParams &p = q->p;
    const int KC = (int) K + 1;
    p.K = KC;  // count fields of the replay
    p.Wn = (int32_t) Wn;
    p.branch = branch;
    p.site = site;
    p.polarised = !!(options & TSG_STAT_POLARISED);
    AfsParams &a = q->afs;
    a.K = (int32_t) K;
    a.Wn = (int32_t) Wn;
    a.TW = (int32_t) TW;
    a.polarised = p.polarised;
    a.num_samples = n;
    a.afs_size = afs_size;
    {
        int64_t stride = 1;
        for (int k = (int) K - 1; k >= 0; k--) {
            a.dims[k] = (int64_t) sizes[k] + 1;
            a.stride[k] = stride;
            stride *= a.dims[k];
        }
    }

    // node state form: shared memory (16-bit counts) or global memory
    // (32-bit counts, up to 3 sets); the branch replay adds a last-touch
    // position per node
    const int64_t L = std::max<int64_t>(ts->v.max_local, 1);
    q->W = 16;
    q->KQ = (KC + 3) / 4;
    q->smem_bytes = align_up(span_state_bytes(L, 16, q->KQ), 8) + (branch ? L * 8 : 0);
    q->smem_bytes = align_up(q->smem_bytes, 16);
    q->gstate = false;
    q->smem = true;
    q->slot_bytes = 0;
    // (the site replay's 16-bit parent entries keep their top bit for a flag)
    if (!(n <= 65535 && ts->v.max_local <= (branch ? 65534 : 32766)
            && q->smem_bytes <= smem_budget(branch ? afs_replay_kernel((KC + 3) / 4 == 1 ? 0 : 1)
                                                   : replay_kernel(16, (KC + 3) / 4, p)))) {
        if (KC > 4 || ts->v.max_local >= INT32_MAX) {
            delete q;
            return TSG_ERR_TOO_MANY_SAMPLE_SETS;
        }
        q->gstate = true;
        q->W = 32;
        q->KQ = KC <= 2 ? 1 : 2;
        q->smem_bytes = 0;
        q->slot_bytes = align_up(align_up(span_state_bytes(L, 32, q->KQ), 8) + (branch ? L * 8 : 0), 256);
    }
    if (ts->max_children >= 65535) {
        delete q;
        return TSG_ERR_BAD_TREE_SEQUENCE;
    }
    if (branch && ts->v.num_items + ts->v.num_edges >= ((int64_t) 1 << 31)) {
        // each bin's limb counters take at most 2^31 adds
        delete q;
        return TSG_ERR_NO_MEMORY;
    }
    const int form = (q->W == 16 ? 0 : 2) + (q->KQ == 1 ? 0 : 1);
    {
        void *fn = branch ? afs_replay_kernel(form) : replay_kernel(q->W, q->KQ, p);
        if (!q->gstate) {
            // a cap, not a reservation: every query of every tree sequence fits
            allow_max_dynamic_smem(fn);
        }
        int per_sm = 0;
        per_sm = occupancy_blocks((const void *) fn, 512, (size_t) ((size_t) q->smem_bytes));
        cudaGetLastError();
        int64_t grid = (int64_t) std::max(per_sm, 1) * std::max(1, device_count_sms());
        if (q->gstate) {
            grid = std::min<int64_t>(grid, std::max<int64_t>(1, ((int64_t) 8 << 30) / q->slot_bytes));
        }
        q->smem_grid = std::min<int64_t>(grid, std::max<int64_t>(ts->v.num_spans, 1));
    }

    // per-query arrays: sample masks, windows, time windows
    int64_t off_mask = 0;
    int64_t off_win = align_up(off_mask + std::max<int64_t>(n, 1) * 4, 256);
    int64_t off_tw = align_up(off_win + ((int64_t) Wn + 1) * 8, 256);
    int64_t total = align_up(off_tw + ((int64_t) TW + 1) * 8, 256);
    q->blob.assign((size_t) total, 0);
    char *h = q->blob.data();
    std::memcpy(h + off_mask, mask.data(), (size_t) n * 4);
    std::memcpy(h + off_win, windows, ((size_t) Wn + 1) * 8);
    std::memcpy(h + off_tw, time_windows, ((size_t) TW + 1) * 8);
    for (int j = 0; j < 12; j++) {
        q->off[j] = off_win;  // unused span tables point at valid memory
    }
    q->off[0] = off_mask;
    q->off[1] = off_win;
    q->off[7] = off_tw;
    q->ws_bytes = afs_layout(q).total;
    *out = q;
    return 0;
}

// Workspace layout of a relatedness-vector query.
struct MvLayout {
    int64_t wc, partial, slots, err, total;
};

static MvLayout mv_layout_ws(const tsg_query_t *q)
{
    MvLayout l;
    int64_t off = 0;
    l.wc = off;
    off += align_up(q->ts->v.num_samples * (int64_t) q->mv.W * 8, 256);
    l.partial = off;
    off += align_up(q->mv_pairs * q->mv.nf * (int64_t) q->mv.W * 8, 256);
    l.slots = off;
    off += align_up(q->mv_grid * q->mv.slot_bytes, 256);
    l.err = off;
    off += 256;
    l.total = off;
    return l;
}

// Validate a relatedness-vector query (c/tskit/trees.c:10782-10816, windows
// checked without requiring the full span, trees.c:1244-1286) and plan it:
// span groups, their (group, window) partial blocks, per-CTA slots.
static int matvec_build(tsg_query_t **out, const tsg_treeseq_t *ts, uint64_t W, uint64_t Wn,
    const double *windows, uint64_t nf, const int32_t *focal, uint32_t options)
{
    *out = nullptr;
    if (options & (TSG_STAT_NODE | TSG_STAT_SITE)) {
        return TSG_ERR_UNSUPPORTED_STAT_MODE;
    }
    const double Lg = ts->v.sequence_length;
    double default_windows[2] = { 0, Lg };
    if (windows == nullptr) {
        Wn = 1;
        windows = default_windows;
    }
    if (Wn < 1) {
        return TSG_ERR_BAD_NUM_WINDOWS;
    }
    if (windows[0] < 0 || windows[Wn] > Lg) {
        return TSG_ERR_BAD_WINDOWS;
    }
    for (uint64_t j = 0; j < Wn; j++) {
        if (windows[j] >= windows[j + 1]) {
            return TSG_ERR_BAD_WINDOWS;
        }
    }
    for (uint64_t j = 0; j < nf; j++) {
        if (focal[j] < 0 || focal[j] >= ts->v.num_nodes) {
            return TSG_ERR_NODE_OUT_OF_BOUNDS;
        }
    }
    tsg_query_t *q = new tsg_query_t();
    std::memset(&q->p, 0, sizeof(q->p));
    std::memset(&q->afs, 0, sizeof(q->afs));
    std::memset(&q->mv, 0, sizeof(q->mv));
    q->kind = TSG_KIND_MATVEC;
    q->dbuf = nullptr;
    q->ev_start = nullptr;
    q->ev_stop = nullptr;
    q->ts = ts;
    q->options = options;
    q->span_normalise = !!(options & TSG_STAT_SPAN_NORMALISE);
    q->weights = nullptr;
    q->smem = false;
    MvParams &m = q->mv;
    m.W = (int32_t) W;
    m.ncb = (int32_t) ((W + 31) / 32);
    m.Wn = (int32_t) Wn;
    m.nf = (int64_t) nf;
    m.centre = !(options & TSG_STAT_NONCENTRED);
    m.L = std::max<int64_t>(ts->v.max_local, 1);
    m.slot_bytes = align_up(matvec_slot_bytes(ts->v, m.L), 256);

    // resident CTAs, bounded by 64 GiB of node state
    int per_sm = 0;
    per_sm = occupancy_blocks((const void *) k_matvec_ptr(), TSG_MV_WARPS * 32, (size_t) (0));
    cudaGetLastError();
    int64_t slots = (int64_t) std::max(per_sm, 1) * std::max(1, device_count_sms());
    slots = std::min<int64_t>(slots, std::max<int64_t>(1, ((int64_t) 64 << 30) / m.slot_bytes));
    const int64_t NS = ts->v.num_spans;
    const auto &bp = ts->h_breakpoints;
    const auto &st = ts->h_span_tree;
    const double W0 = windows[0], WE = windows[Wn];
    int64_t G = std::max<int64_t>(1, std::min<int64_t>(NS, slots / std::max(1, m.ncb)));
    std::vector<int32_t> gspan, gwlo, gwhi;
    std::vector<int64_t> poff;
    for (;;) {
        gspan.assign((size_t) G + 1, 0);
        gwlo.assign((size_t) G, -1);
        gwhi.assign((size_t) G, -2);
        poff.assign((size_t) G + 1, 0);
        for (int64_t g = 0; g <= G; g++) {
            gspan[(size_t) g] = (int32_t) (g * NS / G);
        }
        for (int64_t g = 0; g < G; g++) {
            const double xs = bp[(size_t) st[(size_t) gspan[(size_t) g]]];
            const double xe = bp[(size_t) st[(size_t) gspan[(size_t) g + 1]]];
            int64_t np = 0;
            if (gspan[(size_t) g] < gspan[(size_t) g + 1] && xe > W0 && xs < WE) {
                const double a = std::max(xs, W0), b = std::min(xe, WE);
                const int64_t lo = upper_bound(windows, (int64_t) Wn + 1, a) - 1;
                const int64_t hi = lower_bound(windows, (int64_t) Wn + 1, b) - 1;
                gwlo[(size_t) g] = (int32_t) lo;
                gwhi[(size_t) g] = (int32_t) hi;
                np = hi - lo + 1;
            }
            poff[(size_t) g + 1] = poff[(size_t) g] + np;
        }
        const int64_t bytes = poff[(size_t) G] * (int64_t) nf * (int64_t) W * 8;
        if (bytes <= ((int64_t) 24 << 30) || G == 1) {
            if (bytes > ((int64_t) 48 << 30)) {
                delete q;
                return TSG_ERR_NO_MEMORY;
            }
            break;
        }
        G = std::max<int64_t>(1, G / 2);
    }
    std::vector<int32_t> wglo((size_t) Wn, 0), wghi((size_t) Wn, -1);
    for (int64_t mw = 0; mw < (int64_t) Wn; mw++) {
        int32_t lo = -1, hi = -2;
        for (int64_t g = 0; g < G; g++) {
            if (gwlo[(size_t) g] >= 0 && gwlo[(size_t) g] <= mw && mw <= gwhi[(size_t) g]) {
                if (lo < 0) {
                    lo = (int32_t) g;
                }
                hi = (int32_t) g;
            }
        }
        wglo[(size_t) mw] = lo < 0 ? 0 : lo;
        wghi[(size_t) mw] = hi;
    }
    m.G = (int32_t) G;
    q->mv_pairs = poff[(size_t) G];
    q->mv_grid = std::min<int64_t>(G * m.ncb, slots);

    int64_t off_win = 0;
    int64_t off_focal = align_up(off_win + ((int64_t) Wn + 1) * 8, 256);
    int64_t off_gspan = align_up(off_focal + std::max<int64_t>((int64_t) nf, 1) * 4, 256);
    int64_t off_gwlo = align_up(off_gspan + (G + 1) * 4, 256);
    int64_t off_poff = align_up(off_gwlo + G * 4, 256);
    int64_t off_wglo = align_up(off_poff + (G + 1) * 8, 256);
    int64_t off_wghi = align_up(off_wglo + (int64_t) Wn * 4, 256);
    int64_t total = align_up(off_wghi + (int64_t) Wn * 4, 256);
    q->blob.assign((size_t) total, 0);
    char *h = q->blob.data();
    std::memcpy(h + off_win, windows, ((size_t) Wn + 1) * 8);
    if (nf > 0) {
        std::memcpy(h + off_focal, focal, (size_t) nf * 4);
    }
    std::memcpy(h + off_gspan, gspan.data(), (size_t) (G + 1) * 4);
    std::memcpy(h + off_gwlo, gwlo.data(), (size_t) G * 4);
    std::memcpy(h + off_poff, poff.data(), (size_t) (G + 1) * 8);
    std::memcpy(h + off_wglo, wglo.data(), (size_t) Wn * 4);
    std::memcpy(h + off_wghi, wghi.data(), (size_t) Wn * 4);
    for (int j = 8; j < 12; j++) {
        q->off[j] = off_win;  // unused window tables point at valid memory
    }
    q->off[0] = off_win;
    q->off[1] = off_win;
    q->off[2] = off_focal;
    q->off[3] = off_gspan;
    q->off[4] = off_gwlo;
    q->off[5] = off_poff;
    q->off[6] = off_wglo;
    q->off[7] = off_wghi;
    q->ws_bytes = mv_layout_ws(q).total;
    *out = q;
    return 0;
}

static int matvec_launch(const tsg_query_t *q, tsg_workspace_t *ws, double *result,
    cudaStream_t st)
{
    NvtxRange nvtx("tsg.relatedness_vector");
    const int64_t nres = tsg_query_result_size(q);
    if (q->mv.W == 0 || q->mv.nf == 0) {
        return 0;
    }
    if (q->weights == nullptr) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    const MvLayout l = mv_layout_ws(q);
    char *b = (char *) ws->ptr;
    MvParams m = q->mv;
    m.weights = q->weights;
    m.wc = (double *) (b + l.wc);
    m.partial = (double *) (b + l.partial);
    m.slots = (unsigned char *) (b + l.slots);
    m.err = (int32_t *) (b + l.err);
    m.counter = m.err + 1;
    TSG_CUDA(cudaMemsetAsync(m.err, 0, 2 * sizeof(int32_t), st));
    if (q->ev_start != nullptr) {
        TSG_CUDA(cudaEventRecord(q->ev_start, st));
    }
    int ret = launch_matvec((unsigned) q->mv_grid, st, q->ts->v, m, q->span_normalise, result);
    if (ret == 0 && q->ev_stop != nullptr) {
        TSG_CUDA(cudaEventRecord(q->ev_stop, st));
    }
    (void) nres;
    return ret;
}

static int afs_launch(const tsg_query_t *q, tsg_workspace_t *ws, double *result, cudaStream_t st)
{
    NvtxRange nvtx("tsg.afs");
    const tsg_treeseq_t *ts = q->ts;
    const AfsLayout l = afs_layout(q);
    char *b = (char *) ws->ptr;
    WsDev w;
    std::memset(&w, 0, sizeof(w));
    w.node_mask = (uint32_t *) (b + l.node_mask);
    w.mcnt = (uint64_t *) (b + l.mcnt);
    w.state = b + l.state;
    w.seekcnt = (uint32_t *) (b + l.seekcnt);
    w.err = (int32_t *) (b + l.err);
    w.counter = w.err + 1;
    AfsParams a = q->afs;
    a.acc = (unsigned long long *) (b + l.acc);
    a.out = result;
    a.err = w.err;
    a.counter = w.counter;
    a.seekcnt = w.seekcnt;
    QueryDev d = q->d;
    d.node_mask = w.node_mask;
    const QueryParams &p = q->p;
    const int form = (q->W == 16 ? 0 : 2) + (q->KQ == 1 ? 0 : 1);
    int ret;
    TSG_CUDA(cudaMemsetAsync(w.err, 0, 2 * sizeof(int32_t), st));
    if (q->ev_start != nullptr) {
        TSG_CUDA(cudaEventRecord(q->ev_start, st));
    }
    k_node_mask<<<grid_for(ts->v.num_nodes), 256, 0, st>>>(ts->v, d, w.node_mask);
    TSG_LAUNCHED();
    const unsigned g = (unsigned) q->smem_grid;
    if (p.site) {
        TSG_CUDA(cudaMemsetAsync(result, 0, (size_t) q->afs_bins * 8, st));
        const size_t sb = (size_t) q->smem_bytes;
        switch (form) {
            case 0: k_replay_items<16, 1, uint16_t, float, false, false><<<g, 512, sb, st>>>(ts->v, p, d, w, 0); break;
            case 1: k_replay_items<16, 2, uint16_t, float, false, false><<<g, 512, sb, st>>>(ts->v, p, d, w, 0); break;
            case 2: k_replay_items<32, 1, int32_t, float, false, false><<<g, 512, 0, st>>>(ts->v, p, d, w, q->slot_bytes); break;
            default: k_replay_items<32, 2, int32_t, float, false, false><<<g, 512, 0, st>>>(ts->v, p, d, w, q->slot_bytes); break;
        }
        TSG_LAUNCHED();
        if ((ret = launch_afs_site(form, st, ts->v, a, w.mcnt)) != 0) {
            return ret;
        }
    } else {
        TSG_CUDA(cudaMemsetAsync(a.acc, 0, (size_t) q->afs_bins * TSG_FX_LIMBS * 8, st));
        if ((ret = launch_afs_branch(form, g, (size_t) q->smem_bytes, q->slot_bytes, w.state, st,
                 ts->v, d, a)) != 0) {
            return ret;
        }
    }
    if (q->ev_stop != nullptr) {
        TSG_CUDA(cudaEventRecord(q->ev_stop, st));
    }
    return launch_afs_finish(st, a, q->span_normalise, p.branch, result);
}

}  // namespace tsg

extern "C" {

}  // extern "C"

namespace tsg {

// Views of a sample-count query's workspace (layout of query_build).
static WsDev ws_bind(const tsg_query_t *q, tsg_workspace_t *ws)
{
    const tsg_treeseq_t *ts = q->ts;
    const QueryParams &p = q->p;
    const int64_t N = ts->v.num_nodes;
    const int64_t NS = std::max(ts->v.num_spans, ts->v.num_segs);
    const int64_t TSW = std::max(q->total_span_windows, q->total_seg_windows);
    const int64_t R = p.R, slots = q->num_slots;
    char *b = (char *) ws->ptr;
    WsDev w;
    int64_t off = 0;
    w.parent = (int32_t *) (b + off);
    off += align_up(slots * N * 4, 256);
    w.nchild = (int32_t *) (b + off);
    off += align_up(slots * N * 4, 256);
    w.arrive = (int32_t *) (b + off);
    off += align_up(slots * N * 4, 256);
    w.x = (int32_t *) (b + off);
    off += align_up(slots * N * 4 * p.KP, 256);
    w.A = (double *) (b + off);
    off += align_up(TSW * 8, 256);
    w.B = (double *) (b + off);
    off += align_up(TSW * R * 8, 256);
    w.SITE = (double *) (b + off);
    off += align_up(TSW * R * 8, 256);
    w.D = (double *) (b + off);
    off += align_up(NS * R * 8, 256);
    w.RS = (double *) (b + off);
    off += align_up(NS * R * 8, 256);
    w.rs0 = (double *) (b + off);
    off += align_up(R * 8, 256);
    w.items = nullptr;
    w.bl = nullptr;
    w.state = nullptr;
    w.seekcnt = nullptr;
    w.leaf_area = nullptr;
    w.leaf_dbl = nullptr;
    w.leaf_win = nullptr;
    w.mcnt = nullptr;
    w.dD = nullptr;
    w.node_mask = nullptr;
    w.site_val = nullptr;
    w.site_win = nullptr;
    w.cp0 = nullptr;
    w.c_pep = nullptr;
    w.c_ctot = nullptr;
    w.site_acc = nullptr;
    if (q->smem) {
        const int64_t item_bytes = q->KQ == 1 ? (int64_t) sizeof(Item<1>) : (int64_t) sizeof(Item<2>);
        w.items = b + off;
        off += align_up((p.branch ? ts->v.num_items : 0) * item_bytes, 256);
        w.bl = b + off;
        off += align_up((p.branch ? ts->v.num_items : 0) * (p.f32 ? 8 : 16), 256);
        w.mcnt = (uint64_t *) (b + off);
        off += align_up(ts->v.num_mutations * 8 * q->KQ, 256);
        w.dD = (double *) (b + off);
        off += align_up(ts->v.num_chunks * R * 8, 256);
        w.node_mask = (uint32_t *) (b + off);
        off += align_up(ts->v.num_nodes * 4, 256);
        w.site_val = (double *) (b + off);
        off += align_up((p.site ? ts->v.num_sites : 0) * R * 8, 256);
        w.site_acc = (unsigned long long *) (b + off);
        off += align_up((p.site && p.site_int ? (int64_t) p.Wn : 0) * R * 16, 256);
        w.site_win = (double *) (b + off);
        off += align_up((int64_t) p.Wn * R * 8, 256);
        w.state = b + off;
        off += align_up(q->gstate ? q->smem_grid * q->slot_bytes : 0, 256);
        w.seekcnt = (uint32_t *) (b + off);
        off += align_up(q->smem_grid * std::max<int64_t>(ts->v.max_local, 1) * 4, 256);
        w.leaf_area = (unsigned long long *) (b + off);
        off += align_up((p.branch ? (int64_t) p.Wn << p.K : 0) * TSG_FX_LIMBS * 8 * 3, 256);
        w.leaf_dbl = (double *) (b + off);
        off += align_up((p.branch ? (int64_t) p.Wn << p.K : 0) * 8, 256);
        w.leaf_win = (double *) (b + off);
        off += align_up((int64_t) p.Wn * R * 8, 256);
        w.cp0 = (uint64_t *) (b + off);
        off += align_up(q->compact_ok ? (ts->v.num_samples + 1) * 16 : 0, 256);
        w.c_pep = (uint64_t *) (b + off);
        off += align_up(q->c_ep_cap * 8 * q->KQ, 256);
        w.c_ctot = (uint64_t *) (b + off);
        off += align_up(q->c_rows_cap * compact_row_chunks(ts->v.num_samples) * 8 * q->KQ, 256);
    }
    w.err = (int32_t *) (b + off);
    w.counter = w.err + 1;
    return w;
}

}  // namespace tsg

extern "C" {

static int query_upload(tsg_query_t *q, tsg_query_t **out)
{
    if (cudaMallocAsync(&q->dbuf, q->blob.size(), 0) != cudaSuccess) {
        cudaGetLastError();
        q->dbuf = nullptr;
        delete q;
        return TSG_ERR_NO_MEMORY;
    }
    if (cudaMemcpy(q->dbuf, q->blob.data(), q->blob.size(), cudaMemcpyHostToDevice)
        != cudaSuccess) {
        tsg_query_free(q);
        return TSG_ERR_CUDA;
    }
    query_bind(q, q->dbuf);
    *out = q;
    return 0;
}

int tsg_query_create(tsg_query_t **out, const tsg_treeseq_t *ts, uint64_t K,
    const uint64_t *sizes, const int32_t *sets, uint64_t R, const tsg_output_t *outputs,
    uint64_t Wn, const double *windows, uint32_t options)
{
    tsg_query_t *q = nullptr;
    int ret = query_build(&q, ts, K, sizes, sets, R, outputs, Wn, windows, options);
    if (ret != 0) {
        return ret;
    }
    return query_upload(q, out);
}

int tsg_query_create_afs(tsg_query_t **out, const tsg_treeseq_t *ts, uint64_t K,
    const uint64_t *sizes, const int32_t *sets, uint64_t Wn, const double *windows, uint64_t TW,
    const double *time_windows, uint32_t options)
{
    tsg_query_t *q = nullptr;
    int ret = afs_build(&q, ts, K, sizes, sets, Wn, windows, TW, time_windows, options);
    if (ret != 0) {
        return ret;
    }
    return query_upload(q, out);
}

int tsg_query_create_relatedness_vector(tsg_query_t **out, const tsg_treeseq_t *ts,
    uint64_t num_weights, uint64_t num_windows, const double *windows, uint64_t num_focal,
    const int32_t *focal, uint32_t options)
{
    tsg_query_t *q = nullptr;
    int ret = matvec_build(&q, ts, num_weights, num_windows, windows, num_focal, focal, options);
    if (ret != 0) {
        return ret;
    }
    return query_upload(q, out);
}

int tsg_query_set_weights(tsg_query_t *q, const double *weights_device)
{
    if (q->kind != TSG_KIND_MATVEC) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    q->weights = weights_device;
    return 0;
}

int tsg_query_set_sweep_events(tsg_query_t *q, void *start_event, void *stop_event)
{
    q->ev_start = (cudaEvent_t) start_event;
    q->ev_stop = (cudaEvent_t) stop_event;
    return 0;
}

int tsg_query_set_replay_events(tsg_query_t *q, void *start_event, void *stop_event)
{
    q->ev_rstart = (cudaEvent_t) start_event;
    q->ev_rstop = (cudaEvent_t) stop_event;
    return 0;
}

int tsg_workspace_create(tsg_workspace_t **ws)
{
    tsg_workspace_t *w = new tsg_workspace_t();
    w->ptr = nullptr;
    w->bytes = 0;
    // the launch forks independent stages onto these (optional: without
    // them everything runs on the caller's stream)
    bool ok = true;
    for (int i = 0; i < 2; i++) {
        ok = ok && cudaStreamCreateWithFlags(&w->aux[i], cudaStreamNonBlocking) == cudaSuccess;
    }
    for (int i = 0; i < 6; i++) {
        ok = ok && cudaEventCreateWithFlags(&w->ev[i], cudaEventDisableTiming) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        for (int i = 0; i < 2; i++) {
            if (w->aux[i] != nullptr) {
                cudaStreamDestroy(w->aux[i]);
                w->aux[i] = nullptr;
            }
        }
        for (int i = 0; i < 6; i++) {
            if (w->ev[i] != nullptr) {
                cudaEventDestroy(w->ev[i]);
                w->ev[i] = nullptr;
            }
        }
    }
    *ws = w;
    return 0;
}

int tsg_workspace_reserve(tsg_workspace_t *ws, int64_t bytes)
{
    if (bytes <= ws->bytes) {
        return 0;
    }
    if (ws->ptr != nullptr) {
        TSG_CUDA(cudaFree(ws->ptr));
        ws->ptr = nullptr;
        ws->bytes = 0;
    }
    if (cudaMalloc(&ws->ptr, (size_t) bytes) != cudaSuccess) {
        cudaGetLastError();
        return TSG_ERR_NO_MEMORY;
    }
    ws->bytes = bytes;
    return 0;
}

int64_t tsg_workspace_bytes(const tsg_workspace_t *ws) { return ws->bytes; }

int tsg_workspace_free(tsg_workspace_t *ws)
{
    if (ws != nullptr) {
        for (int i = 0; i < 2; i++) {
            if (ws->aux[i] != nullptr) {
                cudaStreamDestroy(ws->aux[i]);
            }
        }
        for (int i = 0; i < 6; i++) {
            if (ws->ev[i] != nullptr) {
                cudaEventDestroy(ws->ev[i]);
            }
        }
        cudaFree(ws->ptr);
        delete ws;
    }
    return 0;
}

int tsg_query_launch(const tsg_query_t *q, tsg_workspace_t *ws, double *result,
    void *cuda_stream)
{
    if (ws == nullptr || ws->bytes < q->ws_bytes) {
        return TSG_ERR_WORKSPACE_TOO_SMALL;
    }
    cudaStream_t st = (cudaStream_t) cuda_stream;
    if (q->kind == TSG_KIND_AFS) {
        return afs_launch(q, ws, result, st);
    }
    if (q->kind == TSG_KIND_MATVEC) {
        return matvec_launch(q, ws, result, st);
    }
    NvtxRange nvtx("tsg.query_launch");
    const tsg_treeseq_t *ts = q->ts;
    const QueryParams &p = q->p;
    const int64_t N = ts->v.num_nodes, NS = ts->v.num_spans;
    const int64_t R = p.R, slots = q->num_slots;
    const WsDev w = ws_bind(q, ws);
    TSG_CUDA(cudaMemsetAsync(w.err, 0, 2 * sizeof(int32_t), st));
    TSG_CUDA(cudaMemsetAsync(w.rs0, 0, (size_t) R * 8, st));
    if (q->ev_start != nullptr) {
        TSG_CUDA(cudaEventRecord(q->ev_start, st));
    }
    const bool item_pipeline = q->smem;
    QueryDev d = q->d;
    d.node_mask = w.node_mask;
    // independent stages of the item pipeline run on the workspace's side
    // streams, joined before the window reduction: the leaves' areas (after
    // the node masks) beside the replay, the exact site sums (after the
    // replay) beside the item evaluation
    const bool fork = item_pipeline && ws->aux[0] != nullptr && ws->aux[1] != nullptr;
    const bool site_sums = p.site && p.site_int && ts->v.num_sites > 0;
    const int form = (q->W == 16 ? 0 : 2) + (q->KQ == 1 ? 0 : 1);
    auto leaf_stage = [&](cudaStream_t s) -> int {
        NvtxRange r("tsg.leaves");
        TSG_CUDA(cudaMemsetAsync(w.leaf_area, 0,
            (size_t) ((int64_t) p.Wn << p.K) * TSG_FX_LIMBS * 8 * 3, s));
        if (ts->v.num_edges > 0) {
            k_leaf_areas<<<grid_for(ts->v.num_edges), 256, 0, s>>>(ts->v, p, d, w);
            TSG_LAUNCHED();
        }
        k_leaf_prefix<<<(unsigned) (1 << p.K), 256, 0, s>>>(p, d, w);
        TSG_LAUNCHED();
        if (q->W == 16) {
            k_leaf_terms<16><<<grid_for((int64_t) p.Wn * R), 256, 0, s>>>(p, w);
        } else {
            k_leaf_terms<32><<<grid_for((int64_t) p.Wn * R), 256, 0, s>>>(p, w);
        }
        TSG_LAUNCHED();
        return 0;
    };
    auto site_stage = [&](cudaStream_t s) -> int {
        NvtxRange r("tsg.site_sums");
        // integer numerators summed exactly per window in one pass
        TSG_CUDA(cudaMemsetAsync(w.site_acc, 0, (size_t) p.Wn * R * 16, s));
        const unsigned gsite = (unsigned) ((ts->v.num_sites + 255) / 256);
        switch (form) {
            case 0: k_site_sums<16, 1><<<gsite, 256, 0, s>>>(ts->v, p, d, w); break;
            case 1: k_site_sums<16, 2><<<gsite, 256, 0, s>>>(ts->v, p, d, w); break;
            case 2: k_site_sums<32, 1><<<gsite, 256, 0, s>>>(ts->v, p, d, w); break;
            default: k_site_sums<32, 2><<<gsite, 256, 0, s>>>(ts->v, p, d, w); break;
        }
        TSG_LAUNCHED();
        k_site_sums_finish<<<grid_for((int64_t) p.Wn * R), 256, 0, s>>>(p, w);
        TSG_LAUNCHED();
        return 0;
    };
    bool forked_leaf = false, forked_site = false;
    if (q->smem) {
        k_node_mask<<<grid_for(N), 256, 0, st>>>(ts->v, d, w.node_mask);
        TSG_LAUNCHED();
        // the leaves' stage on side stream 0 from this point of the main
        // stream: right after the node masks for the general replay; after
        // the order rows for the compact one, so that the replay's blocks,
        // launched first, are spread over every SM before the leaves' blocks
        // take some
        auto fork_leaf = [&](bool record) -> int {
            if (fork && p.branch) {
                if (record) {
                    TSG_CUDA(cudaEventRecord(ws->ev[0], st));
                }
                TSG_CUDA(cudaStreamWaitEvent(ws->aux[0], ws->ev[0], 0));
                int r = leaf_stage(ws->aux[0]);
                if (r != 0) {
                    return r;
                }
                TSG_CUDA(cudaEventRecord(ws->ev[1], ws->aux[0]));
                forked_leaf = true;
            }
            return 0;
        };
        if (!compact_serves(q)) {
            int r = fork_leaf(true);
            if (r != 0) {
                return r;
            }
        }
        const unsigned g = (unsigned) q->smem_grid;
        const size_t sb = (size_t) q->smem_bytes;
        auto fork_site = [&]() -> int {
            if (fork && site_sums) {
                TSG_CUDA(cudaEventRecord(ws->ev[2], st));
                TSG_CUDA(cudaStreamWaitEvent(ws->aux[1], ws->ev[2], 0));
                int r = site_stage(ws->aux[1]);
                if (r != 0) {
                    return r;
                }
                TSG_CUDA(cudaEventRecord(ws->ev[3], ws->aux[1]));
                forked_site = true;
            }
            return 0;
        };
        if (compact_serves(q)) {
            // the compact replay: every span's order rows, then one block per
            // span at a time (seek and replay); the first tree's items and
            // the leaves' stage beside it on the side streams, forked after
            // the rows and submitted after the replay so that the replay's
            // blocks are spread over every SM first; then every chunk's item
            // values
            const int kq = q->KQ;
            const unsigned gr = (unsigned) compact_rows_blocks(ts);
            if (kq == 1) {
                k_compact_rows<1><<<gr, TSG_ROWS_THREADS, 0, st>>>(ts->v, p, d, w);
            } else {
                k_compact_rows<2><<<gr, TSG_ROWS_THREADS, 0, st>>>(ts->v, p, d, w);
            }
            TSG_LAUNCHED();
            const bool anchors = p.branch && ts->v.c_num_anchors > 0;
            // the first tree's items are read only by the evaluation
            auto anchor_stage = [&](cudaStream_t sa) -> int {
                const unsigned gp = (unsigned) ((ts->v.num_samples + 1023) / 1024);
                if (kq == 1) {
                    k_compact_prefix<1><<<gp, 1024, 0, sa>>>(ts->v, p, d, w.cp0);
                } else {
                    k_compact_prefix<2><<<gp, 1024, 0, sa>>>(ts->v, p, d, w.cp0);
                }
                TSG_LAUNCHED();
                const unsigned ga = (unsigned) grid_for(ts->v.c_num_anchors);
                if (kq == 1) {
                    k_compact_anchors<1><<<ga, 256, 0, sa>>>(ts->v, p, w.cp0, w);
                } else {
                    k_compact_anchors<2><<<ga, 256, 0, sa>>>(ts->v, p, w.cp0, w);
                }
                TSG_LAUNCHED();
                return 0;
            };
            bool forked_anchors = false;
            if (fork) {
                TSG_CUDA(cudaEventRecord(ws->ev[0], st));
            } else if (anchors) {
                anchor_stage(st);
            }
            const size_t csb = (size_t) align_up(replay_state_bytes(ts->v.c_max_local, 16, kq), 16);
            void *fn = compact_kernel(kq);
            int per_sm = 0;
            per_sm = occupancy_blocks((const void *) fn, TSG_COMPACT_THREADS, (size_t) (csb));
            const unsigned cg = (unsigned) std::min<int64_t>(
                (int64_t) std::max(per_sm, 1) * std::max(1, device_count_sms()), ts->v.c_num_spans);
            if (q->ev_rstart != nullptr) {
                TSG_CUDA(cudaEventRecord(q->ev_rstart, st));
            }
            NvtxRange nvtx_replay("tsg.seek_replay");
            if (kq == 1) {
                k_replay_compact<1><<<cg, TSG_COMPACT_THREADS, csb, st>>>(ts->v, p, d, w);
            } else {
                k_replay_compact<2><<<cg, TSG_COMPACT_THREADS, csb, st>>>(ts->v, p, d, w);
            }
            if (fork) {
                int r = fork_leaf(false);
                if (r != 0) {
                    return r;
                }
                if (anchors) {
                    TSG_CUDA(cudaStreamWaitEvent(ws->aux[1], ws->ev[0], 0));
                    anchor_stage(ws->aux[1]);
                    TSG_CUDA(cudaEventRecord(ws->ev[5], ws->aux[1]));
                    forked_anchors = true;
                }
            }
            if (q->ev_rstop != nullptr) {
                TSG_CUDA(cudaEventRecord(q->ev_rstop, st));
            }
            TSG_LAUNCHED();
            int r = fork_site();
            if (r != 0) {
                return r;
            }
            if (p.branch) {
                if (forked_anchors) {
                    TSG_CUDA(cudaStreamWaitEvent(st, ws->ev[5], 0));
                }
                NvtxRange nvtx_eval("tsg.evaluate");
                // the items' values (the replay wrote their branch lengths)
                if (p.f32) {
                    (p.polarised ? launch_eval_chunks_f32_pol : launch_eval_chunks_f32_unpol)(kq, st,
                        ts->v, p, w);
                } else {
                    (p.polarised ? launch_eval_chunks_f64_pol : launch_eval_chunks_f64_unpol)(kq, st,
                        ts->v, p, w);
                }
                TSG_LAUNCHED();
            }
        } else if (p.branch) {
            // replay and item values in one kernel
            if (q->ev_rstart != nullptr) {
                TSG_CUDA(cudaEventRecord(q->ev_rstart, st));
            }
            if (p.f32) {
                (p.polarised ? launch_replay_eval_f32_pol : launch_replay_eval_f32_unpol)(form, g, sb,
                    q->slot_bytes, st, ts->v, p, d, w);
            } else {
                (p.polarised ? launch_replay_eval_f64_pol : launch_replay_eval_f64_unpol)(form, g, sb,
                    q->slot_bytes, st, ts->v, p, d, w);
            }
            if (q->ev_rstop != nullptr) {
                TSG_CUDA(cudaEventRecord(q->ev_rstop, st));
            }
            TSG_LAUNCHED();
            int r = fork_site();
            if (r != 0) {
                return r;
            }
        } else {
            switch (form) {
                case 0: k_replay_items<16, 1, uint16_t, float, false, false><<<g, 512, sb, st>>>(ts->v, p, d, w, 0); break;
                case 1: k_replay_items<16, 2, uint16_t, float, false, false><<<g, 512, sb, st>>>(ts->v, p, d, w, 0); break;
                case 2: k_replay_items<32, 1, int32_t, float, false, false><<<g, 512, 0, st>>>(ts->v, p, d, w, q->slot_bytes); break;
                default: k_replay_items<32, 2, int32_t, float, false, false><<<g, 512, 0, st>>>(ts->v, p, d, w, q->slot_bytes); break;
            }
            TSG_LAUNCHED();
            int r = fork_site();
            if (r != 0) {
                return r;
            }
        }
        if (p.branch) {
            NvtxRange nvtx_win("tsg.windows");
            k_span_windows<<<(unsigned) ((ts->v.num_segs + 3) / 4), 128, 0, st>>>(ts->v, p, d, w);
            TSG_LAUNCHED();
            if (!forked_leaf) {
                int r = leaf_stage(st);
                if (r != 0) {
                    return r;
                }
            }
        }
        if (site_sums) {
            if (!forked_site) {
                int r = site_stage(st);
                if (r != 0) {
                    return r;
                }
            }
        } else if (p.site && ts->v.num_sites > 0) {
            const unsigned gsite = (unsigned) ((ts->v.num_sites + 255) / 256);
            switch (form) {
                case 0: k_site_eval<TSG_ITEM_RMAX, 16, 1><<<gsite, 256, 0, st>>>(ts->v, p, w); break;
                case 1: k_site_eval<TSG_ITEM_RMAX, 16, 2><<<gsite, 256, 0, st>>>(ts->v, p, w); break;
                case 2: k_site_eval<TSG_ITEM_RMAX, 32, 1><<<gsite, 256, 0, st>>>(ts->v, p, w); break;
                default: k_site_eval<TSG_ITEM_RMAX, 32, 2><<<gsite, 256, 0, st>>>(ts->v, p, w); break;
            }
            TSG_LAUNCHED();
        }
        if (p.site && !(p.site_int && ts->v.num_sites > 0)) {
            if (ts->v.num_sites > 0) {
                k_site_windows<<<(unsigned) p.Wn, 1024, 0, st>>>(p, d, w,
                    ts->v.num_sites, p.site_int);
                TSG_LAUNCHED();
            } else {
                TSG_CUDA(cudaMemsetAsync(w.site_win, 0, (size_t) p.Wn * R * 8, st));
            }
        }
    } else {
        if (p.f32) {
            k_sweep<float><<<(unsigned) slots, 256, 0, st>>>(ts->v, p, q->d, w);
        } else {
            k_sweep<double><<<(unsigned) slots, 256, 0, st>>>(ts->v, p, q->d, w);
        }
        TSG_LAUNCHED();
    }
    if (q->ev_stop != nullptr) {
        TSG_CUDA(cudaEventRecord(q->ev_stop, st));
    }
    if (p.branch) {
        k_span_scan<<<(unsigned) R, 512, 0, st>>>(w.D, w.rs0, w.RS,
            item_pipeline ? ts->v.num_segs : NS, (int) R);
        TSG_LAUNCHED();
    }
    NvtxRange nvtx_reduce("tsg.reduce");
    if (forked_leaf) {
        TSG_CUDA(cudaStreamWaitEvent(st, ws->ev[1], 0));
    }
    if (forked_site) {
        TSG_CUDA(cudaStreamWaitEvent(st, ws->ev[3], 0));
    }
    k_window_reduce<<<grid_for((int64_t) p.Wn * R), 256, 0, st>>>(p, d, w, q->span_normalise,
        item_pipeline ? 1 : 0, result);
    TSG_LAUNCHED();
    return 0;
}

// ------------------------------------------------------------ batched launch
// A batch fuses prepared queries on any resident tree sequences into one
// launch per pipeline stage.  Sample-count queries on the compact replay are
// grouped by count words and arithmetic (the kernels' template forms); every
// group runs each stage as one kernel over its queries (tsg_batch.cu), the
// replay as one persistent kernel over all the group's spans.  Other queries
// (allele frequency spectrum, relatedness vector, the general replay) run
// their own launches in the same stream.  Each query keeps its own region of
// the batch workspace, bound when the batch is made.
struct tsg_batch {
    struct Group {
        int kq = 1, f32 = 0, pol = 0;
        std::vector<int> idx;           // queries of the group
        int64_t blocks[BS_COUNT] = {};  // blocks of each stage over the group
        int64_t stage_off = 0;          // offset of the group's stage arrays in dbuf
        int64_t span_off = 0;           // ... of its span prefix
        int64_t desc_off = 0;           // ... of its descriptors
        int64_t spans = 0;
        int64_t max_local = 0;
        bool branch = false, site = false;
        int32_t *counter = nullptr;     // the replay's span counter (workspace)
    };
    std::vector<const tsg_query_t *> q;
    std::vector<double *> results;
    std::vector<int64_t> ws_off;
    std::vector<Group> groups;
    std::vector<int> single;
    char *ws_base = nullptr;
    void *dbuf = nullptr;
};

namespace tsg {

static bool batch_fusable(const tsg_query_t *q)
{
    const tsg_treeseq_t *ts = q->ts;
    return q->kind == TSG_KIND_STATS && q->smem && compact_serves(q)
        && q->W == 16 && (!q->p.site || (q->p.site_int && ts->v.num_sites > 0));
}

// Blocks of each stage for one fusable query, as its own launch sizes them.
static void batch_stage_blocks(const tsg_query_t *q, int64_t *nb)
{
    const tsg_treeseq_t *ts = q->ts;
    const QueryParams &p = q->p;
    const int64_t R = p.R;
    for (int k = 0; k < BS_COUNT; k++) {
        nb[k] = 0;
    }
    const int64_t leaf = p.branch ? ((int64_t) p.Wn << p.K) * TSG_FX_LIMBS * 3 : 0;
    const int64_t site = p.site && p.site_int ? (int64_t) p.Wn * R * 2 : 0;
    nb[BS_ZERO] = std::min<int64_t>((1 + R + leaf + site + 255) / 256, 4096);
    nb[BS_NODE_MASK] = grid_for(ts->v.num_nodes);
    nb[BS_ROWS] = compact_rows_blocks(ts);
    if (p.branch) {
        if (ts->v.c_num_anchors > 0) {
            nb[BS_PREFIX] = (ts->v.num_samples + 1023) / 1024;
            nb[BS_ANCHORS] = grid_for(ts->v.c_num_anchors);
        }
        const int64_t C = ts->v.num_chunks;
        const int64_t total = (C + TSG_EVAL_BLOCK - 1) / TSG_EVAL_BLOCK * p.gwpb;
        nb[BS_EVAL] = std::min<int64_t>((total + 7) / 8, 1 << 20);
        nb[BS_SPAN_WINDOWS] = (ts->v.num_segs + 7) / 8;
        nb[BS_LEAF_AREAS] = ts->v.num_edges > 0 ? grid_for(ts->v.num_edges) : 0;
        nb[BS_LEAF_PREFIX] = (int64_t) 1 << p.K;
        nb[BS_LEAF_TERMS] = grid_for((int64_t) p.Wn * R);
        nb[BS_SPAN_SCAN] = R;
    }
    if (p.site) {
        nb[BS_SITE_SUMS] = (ts->v.num_sites + 255) / 256;
        nb[BS_SITE_FINISH] = grid_for((int64_t) p.Wn * R);
    }
    nb[BS_REDUCE] = grid_for((int64_t) p.Wn * R);
}

}  // namespace tsg

int tsg_batch_workspace_bytes(uint64_t num_queries, const tsg_query_t *const *queries,
    int64_t *bytes)
{
    if (queries == nullptr || bytes == nullptr) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    int64_t off = 0;
    for (uint64_t i = 0; i < num_queries; i++) {
        if (queries[i] == nullptr) {
            return TSG_ERR_BAD_PARAM_VALUE;
        }
        off += align_up(queries[i]->ws_bytes, 256);
    }
    *bytes = off + 256 * 8;  // the groups' span counters
    return 0;
}

int tsg_batch_create(tsg_batch_t **out, uint64_t num_queries, const tsg_query_t *const *queries,
    double *const *results, tsg_workspace_t *ws)
{
    if (out == nullptr || results == nullptr || ws == nullptr || num_queries == 0) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    int64_t need = 0;
    int ret = tsg_batch_workspace_bytes(num_queries, queries, &need);
    if (ret != 0) {
        return ret;
    }
    if (ws->bytes < need) {
        return TSG_ERR_WORKSPACE_TOO_SMALL;
    }
    tsg_batch_t *b = new tsg_batch_t();
    b->ws_base = (char *) ws->ptr;
    int64_t off = 0;
    for (uint64_t i = 0; i < num_queries; i++) {
        b->q.push_back(queries[i]);
        b->results.push_back(results[i]);
        b->ws_off.push_back(off);
        off += align_up(queries[i]->ws_bytes, 256);
    }
    // groups by the kernels' template forms (at most eight of them share
    // the span-counter words at the workspace's end)
    for (uint64_t i = 0; i < num_queries; i++) {
        const tsg_query_t *q = queries[i];
        if (!batch_fusable(q)) {
            b->single.push_back((int) i);
            continue;
        }
        tsg_batch_t::Group *g = nullptr;
        for (auto &h : b->groups) {
            if (h.kq == q->KQ && h.f32 == q->p.f32 && h.pol == q->p.polarised) {
                g = &h;
            }
        }
        if (g == nullptr) {
            b->groups.emplace_back();
            g = &b->groups.back();
            g->kq = q->KQ;
            g->f32 = q->p.f32;
            g->pol = q->p.polarised;
        }
        g->idx.push_back((int) i);
    }
    // device image: per group its descriptors, stage prefix arrays and span
    // prefix
    std::vector<char> img;
    auto grow = [&](int64_t bytes) {
        const int64_t at = align_up((int64_t) img.size(), 256);
        img.resize((size_t) (at + bytes), 0);
        return at;
    };
    for (size_t gi = 0; gi < b->groups.size(); gi++) {
        auto &g = b->groups[gi];
        const int nq = (int) g.idx.size();
        g.counter = (int32_t *) (b->ws_base + off + 256 * (int64_t) gi);
        g.desc_off = grow((int64_t) nq * (int64_t) sizeof(BatchQuery));
        g.stage_off = grow((int64_t) BS_COUNT * (nq + 1) * 8);
        g.span_off = grow((int64_t) (nq + 1) * 8);
        for (int j = 0; j < nq; j++) {
            const tsg_query_t *q = queries[g.idx[(size_t) j]];
            tsg_workspace_t region{b->ws_base + b->ws_off[(size_t) g.idx[(size_t) j]], q->ws_bytes};
            BatchQuery d;
            memset(&d, 0, sizeof(d));
            d.v = q->ts->v;
            d.p = q->p;
            d.w = ws_bind(q, &region);
            d.d = q->d;
            d.d.node_mask = d.w.node_mask;
            d.result = results[g.idx[(size_t) j]];
            d.span_normalise = q->span_normalise;
            memcpy(img.data() + g.desc_off + (int64_t) j * (int64_t) sizeof(BatchQuery), &d,
                sizeof(d));
            int64_t nb[BS_COUNT];
            batch_stage_blocks(q, nb);
            int64_t *so = (int64_t *) (img.data() + g.stage_off);
            for (int k = 0; k < BS_COUNT; k++) {
                so[(int64_t) k * (nq + 1) + j + 1] = so[(int64_t) k * (nq + 1) + j] + nb[k];
            }
            int64_t *sp = (int64_t *) (img.data() + g.span_off);
            sp[j + 1] = sp[j] + q->ts->v.c_num_spans;
            g.branch = g.branch || q->p.branch;
            g.site = g.site || q->p.site;
            g.max_local = std::max<int64_t>(g.max_local, q->ts->v.c_max_local);
        }
        const int64_t *so = (const int64_t *) (img.data() + g.stage_off);
        for (int k = 0; k < BS_COUNT; k++) {
            g.blocks[k] = so[(int64_t) k * (nq + 1) + nq];
        }
        g.spans = ((const int64_t *) (img.data() + g.span_off))[nq];
    }
    if (!img.empty()) {
        if (cudaMallocAsync(&b->dbuf, img.size(), 0) != cudaSuccess) {
            cudaGetLastError();
            b->dbuf = nullptr;
            delete b;
            return TSG_ERR_NO_MEMORY;
        }
        if (cudaMemcpy(b->dbuf, img.data(), img.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaFreeAsync(b->dbuf, 0);
            delete b;
            return TSG_ERR_CUDA;
        }
    }
    *out = b;
    return 0;
}

int tsg_batch_launch(const tsg_batch_t *b, void *cuda_stream)
{
    if (b == nullptr) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    NvtxRange nvtx("tsg.batch_launch");
    cudaStream_t st = (cudaStream_t) cuda_stream;
    const char *base = (const char *) b->dbuf;
    for (const auto &g : b->groups) {
        const int nq = (int) g.idx.size();
        const BatchQuery *bq = (const BatchQuery *) (base + g.desc_off);
        auto off = [&](int k) { return (const int64_t *) (base + g.stage_off) + (int64_t) k * (nq + 1); };
        auto stage = [&](int k) {
            int r = batch_launch_stage(k, g.kq, g.blocks[k], st, bq, nq, off(k));
            if (r == 0 && g.blocks[k] > 0) {
                TSG_LAUNCHED();
            }
            return r;
        };
        int ret = 0;
        TSG_CUDA(cudaMemsetAsync(g.counter, 0, sizeof(int32_t), st));
        if ((ret = stage(BS_ZERO)) != 0 || (ret = stage(BS_NODE_MASK)) != 0
            || (ret = stage(BS_PREFIX)) != 0 || (ret = stage(BS_ANCHORS)) != 0
            || (ret = stage(BS_ROWS)) != 0) {
            return ret;
        }
        const size_t csb = (size_t) align_up(replay_state_bytes(g.max_local, 16, g.kq), 16);
        int per_sm = 0;
        per_sm = occupancy_blocks((const void *) batch_replay_kernel(g.kq), TSG_COMPACT_THREADS, (size_t) (csb));
        const unsigned grid = (unsigned) std::min<int64_t>(
            (int64_t) std::max(per_sm, 1) * std::max(1, device_count_sms()), g.spans);
        if ((ret = batch_launch_replay(g.kq, grid, csb, st, bq, nq,
                 (const int64_t *) (base + g.span_off), g.counter)) != 0) {
            return ret;
        }
        TSG_LAUNCHED();
        if (g.branch) {
            if (g.f32) {
                (g.pol ? launch_eval_chunks_batch_f32_pol : launch_eval_chunks_batch_f32_unpol)(
                    g.kq, st, bq, nq, off(BS_EVAL), g.blocks[BS_EVAL]);
            } else {
                (g.pol ? launch_eval_chunks_batch_f64_pol : launch_eval_chunks_batch_f64_unpol)(
                    g.kq, st, bq, nq, off(BS_EVAL), g.blocks[BS_EVAL]);
            }
            TSG_LAUNCHED();
            if (cudaGetLastError() != cudaSuccess) {
                return TSG_ERR_CUDA;
            }
        }
        const int rest[] = {BS_SPAN_WINDOWS, BS_LEAF_AREAS, BS_LEAF_PREFIX, BS_LEAF_TERMS,
            BS_SITE_SUMS, BS_SITE_FINISH, BS_SPAN_SCAN, BS_REDUCE};
        for (int k : rest) {
            if ((ret = stage(k)) != 0) {
                return ret;
            }
        }
    }
    for (int i : b->single) {
        const tsg_query_t *q = b->q[(size_t) i];
        tsg_workspace_t region{b->ws_base + b->ws_off[(size_t) i], q->ws_bytes};
        int ret = tsg_query_launch(q, &region, b->results[(size_t) i], cuda_stream);
        if (ret != 0) {
            return ret;
        }
    }
    return 0;
}

int tsg_batch_num_fused(const tsg_batch_t *b)
{
    int n = 0;
    for (const auto &g : b->groups) {
        n += (int) g.idx.size();
    }
    return n;
}

int tsg_batch_check(const tsg_batch_t *b, uint64_t *failed)
{
    for (size_t i = 0; i < b->q.size(); i++) {
        tsg_workspace_t region{b->ws_base + b->ws_off[i], b->q[i]->ws_bytes};
        const int ret = tsg_workspace_check(&region, b->q[i]);
        if (ret != 0) {
            if (failed != nullptr) {
                *failed = (uint64_t) i;
            }
            return ret;
        }
    }
    return 0;
}

void tsg_batch_free(tsg_batch_t *b)
{
    if (b != nullptr) {
        if (b->dbuf != nullptr) {
            cudaFreeAsync(b->dbuf, 0);
        }
        delete b;
    }
}

// Error word of the last launch on this workspace (synchronous read).
int tsg_workspace_check(const tsg_workspace_t *ws, const tsg_query_t *q)
{
    // the error word sits at the tail of the query's layout
    int32_t h = 0;
    const char *b = (const char *) ws->ptr;
    const int64_t off = q->ws_bytes - 256;
    TSG_CUDA(cudaMemcpy(&h, b + off, sizeof(int32_t), cudaMemcpyDeviceToHost));
    return h == 0 ? 0 : TSG_ERR_DEVICE_CHECK;
}

}  // extern "C"

// ------------------------------------------------- arbitrary summary functions
struct tsg_general {
    tsg_query_t *q = nullptr;
    tsg_workspace_t *ws = nullptr;
    cudaStream_t st = nullptr;
    int form = 0;
    int32_t R = 0, K = 0;
    int64_t U = 0, num_site_keys = 0;
    void *buf = nullptr;
    uint64_t *ulo = nullptr, *uhi = nullptr;
    int64_t *site_off = nullptr;
    WsDev w;
    QueryDev d;
    // real-valued weights: states are listed, not deduplicated
    bool weighted = false;
    void *wbuf = nullptr;
    double *states = nullptr;
    int4 *ids = nullptr;
    unsigned long long *leaf_acc = nullptr;
    int64_t sbase = 0, lbase = 0;
    // node mode: items sorted by (node, tree); states are the items' states
    // after their transitions, then every node's initial state
    bool node = false;
    uint64_t *node_keys = nullptr;
    int32_t *node_idx = nullptr;
};

namespace tsg {

static void general_release(tsg_general *g)
{
    if (g == nullptr) {
        return;
    }
    if (g->st != nullptr) {
        cudaStreamSynchronize(g->st);
    }
    cudaFree(g->buf);
    cudaFree(g->wbuf);
    if (g->ws != nullptr) {
        tsg_workspace_free(g->ws);
    }
    if (g->q != nullptr) {
        tsg_query_free(g->q);
    }
    if (g->st != nullptr) {
        cudaStreamDestroy(g->st);
    }
    delete g;
}

}  // namespace tsg

extern "C" {

int tsg_general_stat_prepare(tsg_general_t **out, const tsg_treeseq_t *ts, uint64_t K,
    const uint64_t *sizes, const int32_t *sets, uint64_t R, uint64_t Wn, const double *windows,
    uint32_t options, int64_t *num_states)
{
    *out = nullptr;
    if (R < 1) {
        return TSG_ERR_BAD_RESULT_DIMS;
    }
    if (options & TSG_STAT_BOTH_MODES) {
        return TSG_ERR_MULTIPLE_STAT_MODES;
    }
    // the replay of a query with (up to 32) placeholder terms
    const uint64_t Rb = std::min<uint64_t>(R, TSG_ITEM_RMAX);
    std::vector<tsg_output_t> outs((size_t) Rb);
    for (auto &o : outs) {
        o.type = TSG_DIVERSITY;
        o.idx[0] = o.idx[1] = o.idx[2] = o.idx[3] = 0;
    }
    tsg_general *g = new tsg_general();
    g->R = (int32_t) R;
    g->K = (int32_t) K;
    int ret = tsg_query_create(&g->q, ts, K, sizes, sets, Rb, outs.data(), Wn, windows,
        options & ~(uint32_t) (TSG_PRECISION_F32_KAHAN | TSG_FORCE_GLOBAL_SWEEP));
    if (ret != 0) {
        delete g;
        return ret;
    }
    tsg_query_t *q = g->q;
    if (!q->smem) {
        general_release(g);
        return TSG_ERR_TOO_MANY_SAMPLE_SETS;
    }
    g->form = (q->W == 16 ? 0 : 2) + (q->KQ == 1 ? 0 : 1);
    if (cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking) != cudaSuccess
        || tsg_workspace_create(&g->ws) != 0
        || (ret = tsg_workspace_reserve(g->ws, q->ws_bytes)) != 0) {
        cudaGetLastError();
        general_release(g);
        return ret != 0 ? ret : TSG_ERR_CUDA;
    }
    const TSView &v = ts->v;
    const QueryParams &p = q->p;
    g->w = ws_bind(q, g->ws);
    g->d = q->d;
    g->d.node_mask = g->w.node_mask;
    // allele count of every site
    std::vector<int64_t> site_off((size_t) v.num_sites + 1, 0);
    for (int64_t s = 0; s < v.num_sites; s++) {
        int32_t mx = 0;
        for (int32_t m = ts->host.site_mut[(size_t) s]; m < ts->host.site_mut[(size_t) s + 1]; m++) {
            mx = std::max(mx, ts->host.mut_allele[(size_t) m]);
        }
        site_off[(size_t) s + 1] = site_off[(size_t) s] + mx + 1;
    }
    g->num_site_keys = site_off[(size_t) v.num_sites];
    const int64_t n = (p.branch ? 2 * v.num_items + ((int64_t) 1 << p.K) : 0)
        + (p.site ? g->num_site_keys : 0);
    const int64_t nk = std::max<int64_t>(n, 1);
    const size_t cub = gen_cub_bytes(nk);
    const int64_t stride = align_up(nk, 32) * 8;
    const int64_t bytes = 8 * stride + align_up((int64_t) cub, 256)
        + align_up((v.num_sites + 1) * 8, 256);
    if (cudaMalloc(&g->buf, (size_t) bytes) != cudaSuccess) {
        cudaGetLastError();
        general_release(g);
        return TSG_ERR_NO_MEMORY;
    }
    char *b = (char *) g->buf;
    uint64_t *klo = (uint64_t *) (b + 0 * stride), *khi = (uint64_t *) (b + 1 * stride);
    uint64_t *tlo = (uint64_t *) (b + 2 * stride), *thi = (uint64_t *) (b + 3 * stride);
    int64_t *flag = (int64_t *) (b + 4 * stride), *pos = (int64_t *) (b + 5 * stride);
    g->ulo = (uint64_t *) (b + 6 * stride);
    g->uhi = (uint64_t *) (b + 7 * stride);
    void *cub_tmp = b + 8 * stride;
    g->site_off = (int64_t *) (b + 8 * stride + align_up((int64_t) cub, 256));
    cudaStream_t st = g->st;
    const WsDev &w = g->w;
    if (cudaMemcpyAsync(g->site_off, site_off.data(), site_off.size() * 8, cudaMemcpyHostToDevice,
            st) != cudaSuccess
        || cudaMemsetAsync(w.err, 0, 8, st) != cudaSuccess) {
        general_release(g);
        return TSG_ERR_CUDA;
    }
    k_node_mask<<<grid_for(v.num_nodes), 256, 0, st>>>(v, g->d, w.node_mask);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ret = cudaGetLastError() == cudaSuccess ? 0 : TSG_ERR_CUDA;
    if (ret == 0) {
        const unsigned gr = (unsigned) q->smem_grid;
        const size_t sb = (size_t) q->smem_bytes;
        switch (g->form) {
            case 0: k_replay_items<16, 1, uint16_t, float, false, false><<<gr, 512, sb, st>>>(v, p, g->d, w, 0); break;
            case 1: k_replay_items<16, 2, uint16_t, float, false, false><<<gr, 512, sb, st>>>(v, p, g->d, w, 0); break;
            case 2: k_replay_items<32, 1, int32_t, float, false, false><<<gr, 512, 0, st>>>(v, p, g->d, w, q->slot_bytes); break;
            default: k_replay_items<32, 2, int32_t, float, false, false><<<gr, 512, 0, st>>>(v, p, g->d, w, q->slot_bytes); break;
        }
        g_launches.fetch_add(1, std::memory_order_relaxed);
        ret = cudaGetLastError() == cudaSuccess ? 0 : TSG_ERR_CUDA;
    }
    if (ret == 0 && p.branch) {
        // the leaves' branch areas per window and membership pattern
        if (cudaMemsetAsync(w.leaf_area, 0,
                (size_t) ((int64_t) p.Wn << p.K) * TSG_FX_LIMBS * 8 * 3, st) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
        } else {
            if (v.num_edges > 0) {
                k_leaf_areas<<<grid_for(v.num_edges), 256, 0, st>>>(v, p, g->d, w);
                g_launches.fetch_add(1, std::memory_order_relaxed);
            }
            k_leaf_prefix<<<(unsigned) (1 << p.K), 256, 0, st>>>(p, g->d, w);
            g_launches.fetch_add(1, std::memory_order_relaxed);
            ret = cudaGetLastError() == cudaSuccess ? 0 : TSG_ERR_CUDA;
        }
    }
    if (ret == 0) {
        ret = gen_collect(g->form, v, p, w, g->site_off, g->num_site_keys, klo, khi, tlo, thi,
            flag, pos, cub_tmp, cub, g->ulo, g->uhi, &g->U, st);
    }
    if (ret == 0) {
        int32_t herr = 0;
        if (cudaMemcpyAsync(&herr, w.err, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess
            || cudaStreamSynchronize(st) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
        } else if (herr != 0) {
            ret = TSG_ERR_DEVICE_CHECK;
        }
    }
    if (ret != 0) {
        general_release(g);
        return ret;
    }
    *num_states = g->U;
    *out = g;
    return 0;
}

int tsg_general_stat_states(tsg_general_t *g, int32_t *states)
{
    if (g->U == 0) {
        return 0;
    }
    int32_t *d = nullptr;
    if (cudaMalloc(&d, (size_t) (g->U * g->K * 4)) != cudaSuccess) {
        cudaGetLastError();
        return TSG_ERR_NO_MEMORY;
    }
    int ret = gen_unpack(g->q->W, g->ulo, g->uhi, g->U, g->K, d, g->st);
    if (ret == 0
        && (cudaMemcpyAsync(states, d, (size_t) (g->U * g->K * 4), cudaMemcpyDeviceToHost, g->st)
                != cudaSuccess
            || cudaStreamSynchronize(g->st) != cudaSuccess)) {
        ret = TSG_ERR_CUDA;
    }
    cudaFree(d);
    return ret;
}

}  // extern "C"

namespace tsg {

// The finish step with the values table (U x R) already on the device.
// Node mode: every node's window integrals of f (values dF, one row per
// listed state), result [Wn x N x R].
static int node_finish(tsg_general *g, const double *dF, double *result)
{
    const tsg_query_t *q = g->q;
    const TSView &v = q->ts->v;
    const int64_t n = (int64_t) q->p.Wn * v.num_nodes * g->R;
    const int64_t nb = align_up(std::max<int64_t>(n * 8, 8), 256);
    double *dres = nullptr;
    if (cudaMalloc(&dres, (size_t) (nb + 8)) != cudaSuccess) {
        cudaGetLastError();
        return TSG_ERR_NO_MEMORY;
    }
    int32_t *derr = (int32_t *) ((char *) dres + nb), herr = 0;
    int ret = cudaMemsetAsync(derr, 0, 4, g->st) == cudaSuccess ? 0 : TSG_ERR_CUDA;
    if (ret == 0) {
        ret = node_walk(v, q->p.Wn, g->d.windows, g->node_keys, g->node_idx, dF, g->R,
            q->span_normalise, dres, derr, g->st);
    }
    if (ret == 0
        && (cudaGetLastError() != cudaSuccess
            || cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, g->st) != cudaSuccess
            || cudaStreamSynchronize(g->st) != cudaSuccess)) {
        ret = TSG_ERR_CUDA;
    }
    if (ret == 0 && herr != 0) {
        ret = TSG_ERR_DEVICE_CHECK;
    }
    if (ret == 0 && n > 0
        && (cudaMemcpyAsync(result, dres, (size_t) (n * 8), cudaMemcpyDeviceToHost, g->st)
                != cudaSuccess
            || cudaStreamSynchronize(g->st) != cudaSuccess)) {
        ret = TSG_ERR_CUDA;
    }
    cudaFree(dres);
    return ret;
}

static int general_finish(tsg_general *g, const double *dF, double *result)
{
    if (g->node) {
        return node_finish(g, dF, result);
    }
    const tsg_query_t *q = g->q;
    const TSView &v = q->ts->v;
    const int64_t Wn = q->p.Wn, R = g->R;
    const int64_t rb_max = q->p.R;
    double *dres = nullptr;
    if (cudaMalloc(&dres, (size_t) (Wn * rb_max * 8)) != cudaSuccess) {
        cudaGetLastError();
        return TSG_ERR_NO_MEMORY;
    }
    cudaStream_t st = g->st;
    int ret = 0;
    std::vector<double> block((size_t) (Wn * rb_max));
    for (int64_t r0 = 0; ret == 0 && r0 < R; r0 += rb_max) {
        QueryParams pb = q->p;
        pb.R = (int32_t) std::min<int64_t>(rb_max, R - r0);
        ret = g->weighted
            ? genw_eval(v, pb, g->d, g->w, g->ids, dF, g->site_off, g->sbase, g->lbase,
                  g->leaf_acc, (int32_t) R, (int32_t) r0, st)
            : gen_eval(g->form, v, pb, g->w, g->site_off, g->ulo, g->uhi, g->U, dF, (int32_t) R,
                  (int32_t) r0, st);
        if (ret != 0) {
            break;
        }
        if (pb.branch) {
            k_span_windows<<<(unsigned) ((v.num_segs + 3) / 4), 128, 0, st>>>(v, pb, g->d, g->w);
            g_launches.fetch_add(1, std::memory_order_relaxed);
            if (cudaMemsetAsync(g->w.rs0, 0, (size_t) pb.R * 8, st) != cudaSuccess) {
                ret = TSG_ERR_CUDA;
                break;
            }
            k_span_scan<<<(unsigned) pb.R, 512, 0, st>>>(g->w.D, g->w.rs0, g->w.RS,
                v.num_segs, (int) pb.R);
            g_launches.fetch_add(1, std::memory_order_relaxed);
        }
        if (pb.site) {
            if (v.num_sites > 0) {
                k_site_windows<<<(unsigned) pb.Wn, 1024, 0, st>>>(pb, g->d, g->w,
                    v.num_sites, 0);
                g_launches.fetch_add(1, std::memory_order_relaxed);
            } else if (cudaMemsetAsync(g->w.site_win, 0, (size_t) (pb.Wn * pb.R * 8), st)
                != cudaSuccess) {
                ret = TSG_ERR_CUDA;
                break;
            }
        }
        k_window_reduce<<<grid_for((int64_t) pb.Wn * pb.R), 256, 0, st>>>(pb, g->d, g->w,
            q->span_normalise, 1, dres);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        if (cudaGetLastError() != cudaSuccess
            || cudaMemcpyAsync(block.data(), dres, (size_t) (Wn * pb.R * 8),
                   cudaMemcpyDeviceToHost, st) != cudaSuccess
            || cudaStreamSynchronize(st) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
            break;
        }
        for (int64_t wdx = 0; wdx < Wn; wdx++) {
            for (int64_t r = 0; r < pb.R; r++) {
                result[wdx * R + r0 + r] = block[(size_t) (wdx * pb.R + r)];
            }
        }
    }
    cudaFree(dres);
    return ret;
}

}  // namespace tsg

extern "C" {

int tsg_general_stat_finish(tsg_general_t *g, const double *values, double *result)
{
    double *dF = nullptr;
    if (cudaMalloc(&dF, (size_t) std::max<int64_t>(g->U * g->R * 8, 8)) != cudaSuccess) {
        cudaGetLastError();
        return TSG_ERR_NO_MEMORY;
    }
    int ret = 0;
    if (g->U > 0
        && cudaMemcpyAsync(dF, values, (size_t) (g->U * g->R * 8), cudaMemcpyHostToDevice, g->st)
            != cudaSuccess) {
        ret = TSG_ERR_CUDA;
    }
    if (ret == 0) {
        ret = general_finish(g, dF, result);
    }
    cudaFree(dF);
    return ret;
}


int64_t tsg_general_stat_result_size(const tsg_general_t *g)
{
    const int64_t rows = g->node ? g->q->ts->v.num_nodes : 1;
    return (int64_t) g->q->p.Wn * rows * g->R;
}

int tsg_general_stat_free(tsg_general_t *g)
{
    general_release(g);
    return 0;
}

}  // extern "C"

namespace tsg {

// Real-valued weights: the replay of a query with one all-sample set (its
// windows and workspace) and placeholder terms; the states are the weights
// below each node.  weights: n x K by sample index, or N x K by node id
// (node_weights: any node may carry weight, as mean_descendants' reference
// sets do).
static int weighted_prepare(tsg_general_t **out, const tsg_treeseq_t *ts, uint64_t K,
    const double *weights, bool node_weights, uint64_t R, uint64_t Wn, const double *windows,
    uint32_t options, int64_t *num_states)
{
    *out = nullptr;
    if (R < 1) {
        return TSG_ERR_BAD_RESULT_DIMS;
    }
    if (K < 1) {
        return TSG_ERR_BAD_STATE_DIMS;
    }
    if (K > TSG_MAX_SAMPLE_SETS) {
        return TSG_ERR_TOO_MANY_SAMPLE_SETS;
    }
    if (options & TSG_STAT_BOTH_MODES) {
        return TSG_ERR_MULTIPLE_STAT_MODES;
    }
    // node mode replays as branch mode does (its items are the nodes' state
    // changes) but reads no times
    const bool node = options & TSG_STAT_NODE;
    uint32_t qopt = options & ~(uint32_t) (TSG_PRECISION_F32_KAHAN | TSG_FORCE_GLOBAL_SWEEP);
    if (node) {
        if (options & (TSG_STAT_SITE | TSG_STAT_BRANCH)) {
            return TSG_ERR_MULTIPLE_STAT_MODES;
        }
        qopt = (qopt & ~(uint32_t) TSG_STAT_NODE) | TSG_STAT_BRANCH
            | TSG_STAT_ALLOW_TIME_UNCALIBRATED;
    }
    const TSView &v = ts->v;
    const int64_t n = v.num_samples;
    // the query carries the windows, the mode and the workspace plan: one
    // set of all samples (the weights are the replay's own)
    std::vector<uint64_t> sizes(1, (uint64_t) n);
    std::vector<int32_t> sets((size_t) n);
    for (int64_t u = 0; u < v.num_nodes; u++) {
        const int32_t si = ts->h_sample_index[(size_t) u];
        if (si >= 0) {
            sets[(size_t) si] = (int32_t) u;
        }
    }
    const uint64_t Rb = std::min<uint64_t>(R, TSG_ITEM_RMAX);
    std::vector<tsg_output_t> outs((size_t) Rb);
    for (auto &o : outs) {
        o.type = TSG_DIVERSITY;
        o.idx[0] = o.idx[1] = o.idx[2] = o.idx[3] = 0;
    }
    tsg_general *g = new tsg_general();
    g->R = (int32_t) R;
    g->K = (int32_t) K;
    g->weighted = true;
    g->node = node;
    int ret = tsg_query_create(&g->q, ts, 1, sizes.data(), sets.data(), Rb, outs.data(), Wn,
        windows, qopt);
    if (ret != 0) {
        delete g;
        return ret;
    }
    tsg_query_t *q = g->q;
    if (!q->smem) {
        general_release(g);
        return TSG_ERR_TOO_MANY_SAMPLE_SETS;
    }
    if (cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking) != cudaSuccess
        || tsg_workspace_create(&g->ws) != 0
        || (ret = tsg_workspace_reserve(g->ws, q->ws_bytes)) != 0) {
        cudaGetLastError();
        general_release(g);
        return ret != 0 ? ret : TSG_ERR_CUDA;
    }
    const QueryParams &p = q->p;
    g->w = ws_bind(q, g->ws);
    g->d = q->d;
    std::vector<int64_t> site_off((size_t) v.num_sites + 1, 0);
    for (int64_t s = 0; s < v.num_sites; s++) {
        int32_t mx = 0;
        for (int32_t m = ts->host.site_mut[(size_t) s]; m < ts->host.site_mut[(size_t) s + 1]; m++) {
            mx = std::max(mx, ts->host.mut_allele[(size_t) m]);
        }
        site_off[(size_t) s + 1] = site_off[(size_t) s] + mx + 1;
    }
    const int64_t nsk = site_off[(size_t) v.num_sites];
    const int64_t items = p.branch ? v.num_items : 0;
    g->sbase = 2 * items;
    g->lbase = g->sbase + (p.site ? nsk : 0);
    const int64_t U = node ? v.num_items + v.num_nodes : g->lbase + (p.branch ? v.num_leaves : 0);
    g->U = U;
    std::vector<double> total((size_t) K, 0.0);
    for (int64_t j = 0; j < n; j++) {
        const int64_t row = node_weights ? (int64_t) sets[(size_t) j] : j;
        for (uint64_t k = 0; k < K; k++) {
            total[(size_t) k] += weights[row * (int64_t) K + (int64_t) k];
        }
    }
    const int64_t wrows = node_weights ? v.num_nodes : n;
    const int64_t L = std::max<int64_t>(v.max_local, 1);
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(v.num_spans,
        2 * (int64_t) std::max(device_count_sms(), 1)));
    // one allocation: W, totals, site offsets, per-CTA state, ids, states,
    // mutation states, leaf accumulators, error word and span counter
    int64_t off = 0;
    auto take = [&](int64_t bytes) {
        const int64_t o = off;
        off += align_up(std::max<int64_t>(bytes, 8), 256);
        return o;
    };
    const int64_t oW = take(wrows * (int64_t) K * 8), oT = take((int64_t) K * 8);
    const int64_t oSO = take((v.num_sites + 1) * 8);
    const int64_t oX = take(grid * L * (int64_t) K * 8), oP = take(grid * L * 4), oF = take(grid * L);
    const int64_t oI = take(items * 16), oS = take(U * (int64_t) K * 8);
    const int64_t oM = take(v.num_mutations * (int64_t) K * 8);
    const int64_t oA = take((int64_t) Wn * (int64_t) Rb * TSG_FX_LIMBS * 8 * 6), oE = take(8);
    // node mode: the replay's item states, the initial states, sort buffers
    const int64_t NI = node ? items : 0, NN = node ? v.num_nodes : 0;
    const size_t sort_bytes = node ? node_sort_bytes(NI) : 0;
    const int64_t oXS = take(2 * NI * (int64_t) K * 8), oIN = take(NN * (int64_t) K * 8);
    const int64_t oK0 = take(NI * 8), oK1 = take(NI * 8), oJ0 = take(NI * 4), oJ1 = take(NI * 4);
    const int64_t oST = take((int64_t) sort_bytes);
    if (cudaMalloc(&g->wbuf, (size_t) off) != cudaSuccess) {
        cudaGetLastError();
        general_release(g);
        return TSG_ERR_NO_MEMORY;
    }
    char *b = (char *) g->wbuf;
    double *dW = (double *) (b + oW), *dT = (double *) (b + oT);
    g->site_off = (int64_t *) (b + oSO);
    g->ids = (int4 *) (b + oI);
    g->states = (double *) (b + oS);
    g->leaf_acc = (unsigned long long *) (b + oA);
    int32_t *derr = (int32_t *) (b + oE);
    cudaStream_t st = g->st;
    ret = 0;
    if (cudaMemcpyAsync(dW, weights, (size_t) (wrows * (int64_t) K * 8), cudaMemcpyHostToDevice,
            st) != cudaSuccess
        || cudaMemcpyAsync(dT, total.data(), (size_t) (K * 8), cudaMemcpyHostToDevice, st) != cudaSuccess
        || cudaMemcpyAsync(g->site_off, site_off.data(), site_off.size() * 8,
               cudaMemcpyHostToDevice, st) != cudaSuccess
        || cudaMemsetAsync(derr, 0, 8, st) != cudaSuccess) {
        ret = TSG_ERR_CUDA;
    }
    double *dXS = (double *) (b + oXS), *dIN = (double *) (b + oIN);
    if (ret == 0 && node) {
        ret = node_init(v, (int) K, dW, node_weights, dIN, st);
    }
    if (ret == 0) {
        ret = genw_replay(v, p, dW, node_weights, (int) K, (double *) (b + oX), (int32_t *) (b + oP),
            (uint8_t *) (b + oF), (int) grid, g->ids, node ? dXS : g->states,
            (double *) (b + oM), node ? dIN : nullptr, derr, derr + 1, st);
    }
    if (ret == 0 && node) {
        g->node_keys = (uint64_t *) (b + oK1);
        g->node_idx = (int32_t *) (b + oJ1);
        ret = node_order(v, (int) K, g->ids, dXS, dIN, (uint64_t *) (b + oK0), g->node_keys,
            (int32_t *) (b + oJ0), g->node_idx, b + oST, sort_bytes, g->states, derr, st);
    } else if (ret == 0) {
        ret = genw_states(v, (int) K, dW, dT, (double *) (b + oM), g->site_off,
            p.site ? g->states + g->sbase * (int64_t) K : nullptr,
            p.branch ? g->states + g->lbase * (int64_t) K : nullptr, st);
    }
    if (ret == 0) {
        int32_t herr = 0;
        if (cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess
            || cudaStreamSynchronize(st) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
        } else if (herr != 0) {
            ret = TSG_ERR_DEVICE_CHECK;
        }
    }
    if (ret != 0) {
        general_release(g);
        return ret;
    }
    *num_states = U;
    *out = g;
    return 0;
}

}  // namespace tsg

extern "C" {

int tsg_general_weighted_prepare(tsg_general_t **out, const tsg_treeseq_t *ts, uint64_t K,
    const double *weights, uint64_t R, uint64_t Wn, const double *windows, uint32_t options,
    int64_t *num_states)
{
    return weighted_prepare(out, ts, K, weights, false, R, Wn, windows, options, num_states);
}

// tsk_treeseq_mean_descendants (c/tskit/trees.c:1076-1220): for every node
// and reference set, the mean number of the set's nodes below it over the
// parts of the sequence where it is above any reference node.  The sets
// (any nodes, flattened with their sizes) become node weights with a last
// column for their union; node mode integrates each set's count and the
// union's indicator along the genome for every node.
int tsg_treeseq_mean_descendants(const tsg_treeseq_t *self, uint64_t num_sets,
    const uint64_t *set_sizes, const int32_t *sets, uint32_t options, double *result)
{
    (void) options;
    const int64_t N = self->v.num_nodes;
    if (num_sets == 0 || num_sets + 1 > TSG_MAX_SAMPLE_SETS) {
        return num_sets == 0 ? TSG_ERR_BAD_PARAM_VALUE : TSG_ERR_TOO_MANY_SAMPLE_SETS;
    }
    const uint64_t K = num_sets + 1;
    std::vector<double> w((size_t) (N * (int64_t) K), 0.0);
    for (uint64_t k = 0, j = 0; k < num_sets; k++) {
        for (uint64_t l = 0; l < set_sizes[k]; l++, j++) {
            const int32_t u = sets[j];
            if (u < 0 || u >= N) {
                return TSG_ERR_NODE_OUT_OF_BOUNDS;
            }
            w[(size_t) ((int64_t) u * (int64_t) K + (int64_t) k)] = 1.0;
            w[(size_t) ((int64_t) u * (int64_t) K + (int64_t) num_sets)] = 1.0;
        }
    }
    tsg_general_t *g = nullptr;
    int64_t U = 0;
    int ret = weighted_prepare(&g, self, K, w.data(), true, K, 0, nullptr,
        TSG_STAT_NODE | TSG_STAT_POLARISED, &U);
    if (ret != 0) {
        return ret;
    }
    std::vector<double> sums((size_t) (N * (int64_t) K));
    double *dF = nullptr;
    if (cudaMalloc(&dF, (size_t) std::max<int64_t>(U * (int64_t) K * 8, 8)) != cudaSuccess) {
        cudaGetLastError();
        ret = TSG_ERR_NO_MEMORY;
    } else {
        ret = genw_summary_descendants(g->states, U, (int) K, dF, g->st);
        if (ret == 0) {
            ret = general_finish(g, dF, sums.data());
        }
    }
    cudaFree(dF);
    tsg_general_stat_free(g);
    if (ret != 0) {
        return ret;
    }
    for (int64_t u = 0; u < N; u++) {
        const double *row = sums.data() + u * (int64_t) K;
        const double span = row[num_sets];
        for (uint64_t k = 0; k < num_sets; k++) {
            result[u * (int64_t) num_sets + (int64_t) k] = span > 0 ? row[k] / span : 0.0;
        }
    }
    return 0;
}

// tsk_treeseq_genetic_relatedness_weighted (c/tskit/trees.c:4838-4897): the
// weights with a column of 1/n appended, the pair summary evaluated on the
// device at every state of the weighted replay.
int tsg_treeseq_genetic_relatedness_weighted(const tsg_treeseq_t *self, uint64_t num_weights,
    const double *weights, uint64_t num_index_tuples, const int32_t *index_tuples,
    uint64_t num_windows, const double *windows, double *result, uint32_t options)
{
    const int64_t n = self->v.num_samples;
    if (num_weights == 0) {
        return TSG_ERR_INSUFFICIENT_WEIGHTS;
    }
    for (uint64_t k = 0; k < 2 * num_index_tuples; k++) {
        if (index_tuples[k] < 0 || (uint64_t) index_tuples[k] >= num_weights) {
            return TSG_ERR_BAD_SAMPLE_SET_INDEX;
        }
    }
    const uint64_t K1 = num_weights + 1;
    std::vector<double> w((size_t) (n * K1)), total((size_t) K1, 0.0);
    for (int64_t j = 0; j < n; j++) {
        for (uint64_t k = 0; k < num_weights; k++) {
            w[(size_t) (j * K1 + k)] = weights[j * num_weights + k];
            total[(size_t) k] += weights[j * num_weights + k];
        }
        w[(size_t) (j * K1 + num_weights)] = 1.0 / (double) n;
    }
    // the complement of a state (unpolarised branch statistics) is taken
    // from the weights' own column sums, as general_stat forms them; the
    // summary's scale for the appended column is exactly 1
    double ones = 0.0;
    for (int64_t j = 0; j < n; j++) {
        ones += w[(size_t) (j * K1 + num_weights)];
    }
    total[(size_t) num_weights] = 1.0;
    tsg_general_t *g = nullptr;
    int64_t U = 0;
    int ret = tsg_general_weighted_prepare(&g, self, K1, w.data(), num_index_tuples, num_windows,
        windows, options, &U);
    if (ret != 0) {
        return ret;
    }
    const int64_t R = (int64_t) num_index_tuples;
    double *dF = nullptr, *dT = nullptr;
    int32_t *dI = nullptr;
    if (cudaMalloc(&dF, (size_t) std::max<int64_t>(U * R * 8, 8)) != cudaSuccess
        || cudaMalloc(&dT, (size_t) (K1 * 8)) != cudaSuccess
        || cudaMalloc(&dI, (size_t) std::max<int64_t>(R * 8, 8)) != cudaSuccess) {
        cudaGetLastError();
        ret = TSG_ERR_NO_MEMORY;
    } else if (cudaMemcpyAsync(dT, total.data(), (size_t) (K1 * 8), cudaMemcpyHostToDevice, g->st)
            != cudaSuccess
        || cudaMemcpyAsync(dI, index_tuples, (size_t) (R * 8), cudaMemcpyHostToDevice, g->st)
            != cudaSuccess) {
        ret = TSG_ERR_CUDA;
    } else {
        const bool branch = g->q->p.branch, polarised = g->q->p.polarised;
        ret = genw_summary_relatedness(g->states, U, (int) K1, dT, dI, (int) R,
            ones, !(options & TSG_STAT_NONCENTRED), branch && !polarised, dF, g->st);
        if (ret == 0) {
            ret = general_finish(g, dF, result);
        }
    }
    cudaFree(dF);
    cudaFree(dT);
    cudaFree(dI);
    tsg_general_stat_free(g);
    return ret;
}

}  // extern "C"

namespace tsg {

// general_stat with real weights w (n x K, sample order) and a summary
// evaluated on the device: summary(g, U, total, complement, values) fills
// the values of the U listed states (U x R), complement saying whether the
// unpolarised branch / node wrapper applies (f(x) + f(total - x), with the
// weights' own column sums, c/tskit/trees.c:1944-1972).
template <typename Summary>
static int weighted_device_stat(const tsg_treeseq_t *ts, uint64_t K, const std::vector<double> &w,
    uint64_t R, uint64_t Wn, const double *windows, uint32_t options, Summary summary,
    double *result)
{
    const int64_t n = ts->v.num_samples;
    std::vector<double> total((size_t) K, 0.0);
    for (int64_t j = 0; j < n; j++) {
        for (uint64_t k = 0; k < K; k++) {
            total[(size_t) k] += w[(size_t) (j * (int64_t) K + (int64_t) k)];
        }
    }
    tsg_general_t *g = nullptr;
    int64_t U = 0;
    int ret = tsg_general_weighted_prepare(&g, ts, K, w.data(), R, Wn, windows, options, &U);
    if (ret != 0) {
        return ret;
    }
    double *dF = nullptr, *dT = nullptr;
    if (cudaMalloc(&dF, (size_t) std::max<int64_t>(U * (int64_t) R * 8, 8)) != cudaSuccess
        || cudaMalloc(&dT, (size_t) (K * 8)) != cudaSuccess) {
        cudaGetLastError();
        ret = TSG_ERR_NO_MEMORY;
    } else if (cudaMemcpyAsync(dT, total.data(), (size_t) (K * 8), cudaMemcpyHostToDevice, g->st)
        != cudaSuccess) {
        ret = TSG_ERR_CUDA;
    } else {
        ret = summary(g, U, dT, g->q->p.branch && !g->q->p.polarised, dF);
        if (ret == 0) {
            ret = general_finish(g, dF, result);
        }
    }
    cudaFree(dF);
    cudaFree(dT);
    tsg_general_stat_free(g);
    return ret;
}

// trait statistics: kind 0 covariance, 1 correlation, 2 linear model
static int trait_stat(const tsg_treeseq_t *ts, int kind, uint64_t K, const std::vector<double> &w,
    uint64_t R, const std::vector<double> &V, uint64_t Wn, const double *windows,
    uint32_t options, double *result)
{
    if (K > TSG_MAX_SAMPLE_SETS) {
        return TSG_ERR_TOO_MANY_SAMPLE_SETS;
    }
    const double n = (double) ts->v.num_samples;
    double *dV = nullptr;
    if (!V.empty()) {
        if (cudaMalloc(&dV, V.size() * 8) != cudaSuccess) {
            cudaGetLastError();
            return TSG_ERR_NO_MEMORY;
        }
        if (cudaMemcpy(dV, V.data(), V.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaFree(dV);
            return TSG_ERR_CUDA;
        }
    }
    const int ret = weighted_device_stat(ts, K, w, R, Wn, windows, options,
        [&](tsg_general *g, int64_t U, const double *dT, bool complement, double *dF) {
            return genw_summary_trait(g->states, U, (int) K, (int) R, kind, n, dV, dT, complement,
                dF, g->st);
        },
        result);
    cudaFree(dV);
    return ret;
}

}  // namespace tsg

extern "C" {

// tsk_treeseq_trait_covariance (c/tskit/trees.c:3976-4022): the weights
// centred, f = x^2 / (2 (n - 1)^2) per column.
int tsg_treeseq_trait_covariance(const tsg_treeseq_t *self, uint64_t num_weights,
    const double *weights, uint64_t num_windows, const double *windows, uint32_t options,
    double *result)
{
    const int64_t n = self->v.num_samples;
    if (num_weights == 0) {
        return TSG_ERR_INSUFFICIENT_WEIGHTS;
    }
    const uint64_t K = num_weights;
    std::vector<double> means((size_t) K, 0.0), w((size_t) (n * (int64_t) K));
    for (int64_t j = 0; j < n; j++) {
        for (uint64_t k = 0; k < K; k++) {
            means[(size_t) k] += weights[j * (int64_t) K + (int64_t) k];
        }
    }
    for (uint64_t k = 0; k < K; k++) {
        means[(size_t) k] /= (double) n;
    }
    for (int64_t j = 0; j < n; j++) {
        for (uint64_t k = 0; k < K; k++) {
            w[(size_t) (j * (int64_t) K + (int64_t) k)] =
                weights[j * (int64_t) K + (int64_t) k] - means[(size_t) k];
        }
    }
    return trait_stat(self, 0, K, w, K, {}, num_windows, windows, options, result);
}

// tsk_treeseq_trait_correlation (c/tskit/trees.c:4047-4104): the weights
// standardised (sample standard deviation) with a column of 1/n appended,
// f = x^2 / (2 p (1 - p) n (n - 1)) for a frequency p strictly in (0, 1).
int tsg_treeseq_trait_correlation(const tsg_treeseq_t *self, uint64_t num_weights,
    const double *weights, uint64_t num_windows, const double *windows, uint32_t options,
    double *result)
{
    const int64_t n = self->v.num_samples;
    if (num_weights < 1) {
        return TSG_ERR_INSUFFICIENT_WEIGHTS;
    }
    const uint64_t nw = num_weights, K = nw + 1;
    std::vector<double> means((size_t) nw, 0.0), meansqs((size_t) nw, 0.0), sds((size_t) nw);
    for (int64_t j = 0; j < n; j++) {
        for (uint64_t k = 0; k < nw; k++) {
            const double x = weights[j * (int64_t) nw + (int64_t) k];
            means[(size_t) k] += x;
            meansqs[(size_t) k] += x * x;
        }
    }
    for (uint64_t k = 0; k < nw; k++) {
        means[(size_t) k] /= (double) n;
        meansqs[(size_t) k] -= means[(size_t) k] * means[(size_t) k] * (double) n;
        meansqs[(size_t) k] /= (double) (n - 1);
        sds[(size_t) k] = std::sqrt(meansqs[(size_t) k]);
    }
    std::vector<double> w((size_t) (n * (int64_t) K));
    for (int64_t j = 0; j < n; j++) {
        for (uint64_t k = 0; k < nw; k++) {
            w[(size_t) (j * (int64_t) K + (int64_t) k)] =
                (weights[j * (int64_t) nw + (int64_t) k] - means[(size_t) k]) / sds[(size_t) k];
        }
        w[(size_t) (j * (int64_t) K + (int64_t) nw)] = 1.0 / (double) n;
    }
    return trait_stat(self, 1, K, w, nw, {}, num_windows, windows, options, result);
}

// tsk_treeseq_trait_linear_model (c/tskit/trees.c:4154-4218): traits,
// covariates (already standardised by the caller) and a column of ones;
// V = W^T Z; f as trait_linear_model_summary_func.
int tsg_treeseq_trait_linear_model(const tsg_treeseq_t *self, uint64_t num_weights,
    const double *weights, uint64_t num_covariates, const double *covariates,
    uint64_t num_windows, const double *windows, uint32_t options, double *result)
{
    const int64_t n = self->v.num_samples;
    if (num_weights < 1) {
        return TSG_ERR_INSUFFICIENT_WEIGHTS;
    }
    const uint64_t nw = num_weights, nc = num_covariates, K = nw + nc + 1;
    std::vector<double> V((size_t) (nw * nc), 0.0), w((size_t) (n * (int64_t) K));
    for (int64_t k = 0; k < n; k++) {
        for (uint64_t i = 0; i < nw; i++) {
            for (uint64_t j = 0; j < nc; j++) {
                V[(size_t) (i * nc + j)] += weights[k * (int64_t) nw + (int64_t) i]
                    * covariates[k * (int64_t) nc + (int64_t) j];
            }
        }
    }
    for (int64_t k = 0; k < n; k++) {
        double *row = w.data() + k * (int64_t) K;
        for (uint64_t i = 0; i < nw; i++) {
            row[i] = weights[k * (int64_t) nw + (int64_t) i];
        }
        for (uint64_t i = 0; i < nc; i++) {
            row[nw + i] = covariates[k * (int64_t) nc + (int64_t) i];
        }
        row[nw + nc] = 1.0;
    }
    if (V.empty()) {
        V.push_back(0.0);
    }
    return trait_stat(self, 2, K, w, nw, V, num_windows, windows, options, result);
}

int tsg_general_weighted_states(tsg_general_t *g, double *states)
{
    if (!g->weighted) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    if (g->U == 0) {
        return 0;
    }
    if (cudaMemcpyAsync(states, g->states, (size_t) (g->U * g->K * 8), cudaMemcpyDeviceToHost,
            g->st) != cudaSuccess
        || cudaStreamSynchronize(g->st) != cudaSuccess) {
        return TSG_ERR_CUDA;
    }
    return 0;
}

}  // extern "C"

// ----------------------------------------------------------- host entry points
namespace tsg {

// extra: host data staged after the query's arrays (the relatedness
// vector's weights), bound as the query's weights.
static int run_sync_query(const tsg_treeseq_t *cts, tsg_query_t *q, double *result,
    const void *extra = nullptr, int64_t extra_bytes = 0)
{
    NvtxRange nvtx("tsg.sync_query");
    tsg_treeseq_t *ts = const_cast<tsg_treeseq_t *>(cts);
    int ret;
    std::lock_guard<std::mutex> lock(ts->sync_mutex);
    const int64_t nres = tsg_query_result_size(q);
    const int64_t blob = align_up((int64_t) q->blob.size(), 256);
    const int64_t xb = align_up(extra_bytes, 256);
    const int64_t need = blob + xb + nres * 8;
    cudaStream_t st = ts->sync_stream;
    if (ts->sync_ws == nullptr) {
        tsg_workspace_create(&ts->sync_ws);
    }
    if ((ret = tsg_workspace_reserve(ts->sync_ws, q->ws_bytes)) != 0) {
        tsg_query_free(q);
        return ret;
    }
    if (need > ts->stage_bytes) {
        cudaFree(ts->stage);
        ts->stage = nullptr;
        ts->stage_bytes = 0;
        if (cudaMalloc(&ts->stage, (size_t) need) != cudaSuccess) {
            cudaGetLastError();
            tsg_query_free(q);
            return TSG_ERR_NO_MEMORY;
        }
        ts->stage_bytes = need;
    }
    double *d_res = (double *) ((char *) ts->stage + blob + xb);
    if (cudaMemcpyAsync(ts->stage, q->blob.data(), q->blob.size(), cudaMemcpyHostToDevice, st)
            != cudaSuccess
        || (extra_bytes > 0
            && cudaMemcpyAsync((char *) ts->stage + blob, extra, (size_t) extra_bytes,
                   cudaMemcpyHostToDevice, st) != cudaSuccess)) {
        tsg_query_free(q);
        return TSG_ERR_CUDA;
    }
    query_bind(q, ts->stage);
    if (extra_bytes > 0) {
        q->weights = (const double *) ((char *) ts->stage + blob);
    }
    if ((ret = tsg_query_launch(q, ts->sync_ws, d_res, st)) == 0) {
        // the result and the launch's check word come back in the same
        // stream, one synchronisation for both
        int32_t herr = 0;
        const char *werr = (const char *) ts->sync_ws->ptr + q->ws_bytes - 256;
        if (cudaMemcpyAsync(result, d_res, (size_t) nres * 8, cudaMemcpyDeviceToHost, st)
                != cudaSuccess
            || cudaMemcpyAsync(&herr, werr, sizeof(int32_t), cudaMemcpyDeviceToHost, st)
                != cudaSuccess
            || cudaStreamSynchronize(st) != cudaSuccess) {
            ret = TSG_ERR_CUDA;
        } else {
            ret = herr == 0 ? 0 : TSG_ERR_DEVICE_CHECK;
        }
    }
    tsg_query_free(q);
    return ret;
}

// Sample-set statistics in node mode (tsk_treeseq_sample_count_stat with
// TSK_STAT_NODE, c/tskit/trees.c:2174-2220 and 1788-1918): the sets as 0/1
// weights through the weighted replay, the built-in summaries evaluated on
// the device at every listed state.  Result [Wn x N x R].
static int node_sets(const tsg_treeseq_t *ts, uint64_t K, const uint64_t *sizes,
    const int32_t *sets, uint64_t R, const tsg_output_t *outs, uint64_t Wn,
    const double *windows, uint32_t options, double *result)
{
    if (options & (TSG_STAT_SITE | TSG_STAT_BRANCH | TSG_STAT_BOTH_MODES)) {
        return TSG_ERR_MULTIPLE_STAT_MODES;
    }
    // the sets, terms and windows are checked as for branch mode
    tsg_query_t *q = nullptr;
    int ret = query_build(&q, ts, K, sizes, sets, R, outs, Wn, windows,
        (options & ~(uint32_t) TSG_STAT_NODE) | TSG_STAT_BRANCH
            | TSG_STAT_ALLOW_TIME_UNCALIBRATED);
    if (ret != 0) {
        return ret;
    }
    const QueryParams p = q->p;
    tsg_query_free(q);
    const int64_t n = ts->v.num_samples;
    std::vector<double> W((size_t) (n * (int64_t) K), 0.0);
    uint64_t at = 0;
    for (uint64_t k = 0; k < K; k++) {
        for (uint64_t j = 0; j < sizes[k]; j++, at++) {
            W[(size_t) ((int64_t) ts->h_sample_index[(size_t) sets[at]] * (int64_t) K
                + (int64_t) k)] = 1.0;
        }
    }
    tsg_general_t *g = nullptr;
    int64_t U = 0;
    ret = tsg_general_weighted_prepare(&g, ts, K, W.data(), R, Wn, windows, options, &U);
    if (ret != 0) {
        return ret;
    }
    double *vals = nullptr;
    if (cudaMalloc(&vals, (size_t) std::max<int64_t>(U * (int64_t) R * 8, 8)) != cudaSuccess) {
        cudaGetLastError();
        ret = TSG_ERR_NO_MEMORY;
    } else {
        ret = node_term_values(p, g->states, U, (int) K, !p.polarised, vals, g->st);
        if (ret == 0) {
            ret = general_finish(g, vals, result);
        }
    }
    cudaFree(vals);
    tsg_general_stat_free(g);
    return ret;
}

// The synchronous entry points reuse the tree sequence's own workspace and
// staging buffer (grown on demand, serialised by a mutex), so a call makes no
// device allocation once they are large enough.
static int run_sync(const tsg_treeseq_t *ts, uint64_t K, const uint64_t *sizes,
    const int32_t *sets, uint64_t R, const tsg_output_t *outs, uint64_t Wn,
    const double *windows, uint32_t options, double *result)
{
    if (R > TSG_MAX_OUTPUTS || K > TSG_MAX_SAMPLE_SETS) {
        // more outputs or sets than one sweep carries: groups of outputs
        // whose sets fit one sweep, each swept with just its sets, their
        // columns put back in place (the centred relatedness averages over
        // all sets, so it cannot be split by sets)
        // every set checked as the reference does, used by an output or not
        std::vector<int64_t> seen((size_t) ts->v.num_samples, -1);
        for (uint64_t k = 0, j = 0; k < K; k++) {
            if (sizes[k] == 0) {
                return TSG_ERR_EMPTY_SAMPLE_SET;
            }
            for (uint64_t l = 0; l < sizes[k]; l++) {
                const int32_t u = sets[j++];
                if (u < 0 || u >= ts->v.num_nodes) {
                    return TSG_ERR_NODE_OUT_OF_BOUNDS;
                }
                const int32_t si = ts->h_sample_index[(size_t) u];
                if (si < 0) {
                    return TSG_ERR_BAD_SAMPLES;
                }
                if (seen[(size_t) si] == (int64_t) k) {
                    return TSG_ERR_DUPLICATE_SAMPLE;
                }
                seen[(size_t) si] = (int64_t) k;
            }
        }
        if (K > TSG_MAX_SAMPLE_SETS) {
            for (uint64_t r = 0; r < R; r++) {
                if (outs[r].type == TSG_RELATEDNESS) {
                    return TSG_ERR_TOO_MANY_SAMPLE_SETS;
                }
            }
        }
        std::vector<uint64_t> off((size_t) K + 1, 0);
        for (uint64_t k = 0; k < K; k++) {
            off[(size_t) k + 1] = off[(size_t) k] + sizes[k];
        }
        const int64_t nmodes = (options & TSG_STAT_BOTH_MODES) ? 2 : 1;
        const int64_t rows = (options & TSG_STAT_NODE) ? ts->v.num_nodes : 1;
        const int64_t nw = windows == nullptr ? 1 : (int64_t) Wn;
        uint64_t r0 = 0;
        while (r0 < R) {
            // the group: outputs r0.. while their sets number at most
            // TSG_MAX_SAMPLE_SETS and they at most TSG_MAX_OUTPUTS
            std::vector<int32_t> map((size_t) K, -1), used;
            uint64_t r1 = r0;
            while (r1 < R && r1 - r0 < TSG_MAX_OUTPUTS) {
                const int wdt = tuple_width(outs[r1].type);
                std::vector<int32_t> add;
                for (int j = 0; j < wdt; j++) {
                    const int32_t ix = outs[r1].idx[j];
                    if (ix < 0 || (uint64_t) ix >= K) {
                        return TSG_ERR_BAD_SAMPLE_SET_INDEX;
                    }
                    if (map[(size_t) ix] < 0
                        && std::find(add.begin(), add.end(), ix) == add.end()) {
                        add.push_back(ix);
                    }
                }
                if (used.size() + add.size() > TSG_MAX_SAMPLE_SETS) {
                    break;
                }
                for (int32_t ix : add) {
                    map[(size_t) ix] = (int32_t) used.size();
                    used.push_back(ix);
                }
                r1++;
            }
            if (r1 == r0) {
                return TSG_ERR_TOO_MANY_SAMPLE_SETS;
            }
            std::vector<uint64_t> gsizes;
            std::vector<int32_t> gsets;
            for (int32_t k : used) {
                gsizes.push_back(sizes[k]);
                gsets.insert(gsets.end(), sets + off[(size_t) k], sets + off[(size_t) k + 1]);
            }
            std::vector<tsg_output_t> gouts(outs + r0, outs + r1);
            for (auto &o : gouts) {
                const int wdt = tuple_width(o.type);
                for (int j = 0; j < wdt; j++) {
                    o.idx[j] = map[(size_t) o.idx[j]];
                }
            }
            const uint64_t rc = r1 - r0;
            std::vector<double> part((size_t) (nmodes * nw * rows * (int64_t) rc), 0.0);
            const int ret = run_sync(ts, used.size(), gsizes.data(), gsets.data(), rc,
                gouts.data(), Wn, windows, options, part.data());
            if (ret != 0) {
                return ret;
            }
            for (int64_t b = 0; b < nmodes * nw * rows; b++) {
                std::copy(part.begin() + b * (int64_t) rc, part.begin() + (b + 1) * (int64_t) rc,
                    result + b * (int64_t) R + (int64_t) r0);
            }
            r0 = r1;
        }
        return 0;
    }
    if (options & TSG_STAT_NODE) {
        return node_sets(ts, K, sizes, sets, R, outs, Wn, windows, options, result);
    }
    tsg_query_t *q = nullptr;
    int ret = query_build(&q, ts, K, sizes, sets, R, outs, Wn, windows, options);
    if (ret != 0) {
        return ret;
    }
    return run_sync_query(ts, q, result);
}

static int one_way(const tsg_treeseq_t *ts, int32_t type, uint64_t K, const uint64_t *sizes,
    const int32_t *sets, uint64_t Wn, const double *windows, uint32_t options, double *result)
{
    if (K == 0) {
        return TSG_ERR_INSUFFICIENT_SAMPLE_SETS;
    }
    std::vector<tsg_output_t> outs((size_t) K);
    for (uint64_t k = 0; k < K; k++) {
        outs[(size_t) k].type = type;
        outs[(size_t) k].idx[0] = (int32_t) k;
        outs[(size_t) k].idx[1] = outs[(size_t) k].idx[2] = outs[(size_t) k].idx[3] = 0;
    }
    return run_sync(ts, K, sizes, sets, K, outs.data(), Wn, windows, options, result);
}

static int k_way(const tsg_treeseq_t *ts, int32_t type, int width, uint64_t K,
    const uint64_t *sizes, const int32_t *sets, uint64_t num_tuples, const int32_t *tuples,
    uint64_t Wn, const double *windows, uint32_t options, double *result)
{
    // check_sample_stat_inputs (c/tskit/trees.c:4667-4688)
    if (K < 1) {
        return TSG_ERR_INSUFFICIENT_SAMPLE_SETS;
    }
    if (num_tuples < 1) {
        return TSG_ERR_INSUFFICIENT_INDEX_TUPLES;
    }
    std::vector<tsg_output_t> outs((size_t) num_tuples);
    for (uint64_t r = 0; r < num_tuples; r++) {
        outs[(size_t) r].type = type;
        for (int j = 0; j < 4; j++) {
            int32_t ix = j < width ? tuples[r * width + j] : 0;
            if (ix < 0 || ix >= (int32_t) K) {
                return TSG_ERR_BAD_SAMPLE_SET_INDEX;
            }
            outs[(size_t) r].idx[j] = ix;
        }
    }
    return run_sync(ts, K, sizes, sets, num_tuples, outs.data(), Wn, windows, options, result);
}

}  // namespace tsg

extern "C" {

int tsg_treeseq_sample_count_stat(const tsg_treeseq_t *self, uint64_t K, const uint64_t *sizes,
    const int32_t *sets, uint64_t R, const tsg_output_t *outputs, uint64_t Wn,
    const double *windows, uint32_t options, double *result)
{
    return run_sync(self, K, sizes, sets, R, outputs, Wn, windows, options, result);
}

int tsg_treeseq_allele_frequency_spectrum(const tsg_treeseq_t *self, uint64_t K,
    const uint64_t *sizes, const int32_t *sets, uint64_t Wn, const double *windows, uint64_t TW,
    const double *time_windows, uint32_t options, double *result)
{
    tsg_query_t *q = nullptr;
    int ret = afs_build(&q, self, K, sizes, sets, Wn, windows, TW, time_windows, options);
    if (ret != 0) {
        return ret;
    }
    return run_sync_query(self, q, result);
}

int tsg_treeseq_genetic_relatedness_vector(const tsg_treeseq_t *self, uint64_t num_weights,
    const double *weights, uint64_t num_windows, const double *windows, uint64_t num_focal,
    const int32_t *focal, double *result, uint32_t options)
{
    tsg_query_t *q = nullptr;
    int ret = matvec_build(&q, self, num_weights, num_windows, windows, num_focal, focal, options);
    if (ret != 0) {
        return ret;
    }
    return run_sync_query(self, q, result, weights,
        self->v.num_samples * (int64_t) num_weights * 8);
}

int tsg_treeseq_diversity(const tsg_treeseq_t *self, uint64_t K, const uint64_t *sizes,
    const int32_t *sets, uint64_t Wn, const double *windows, uint32_t options, double *result)
{
    return one_way(self, TSG_DIVERSITY, K, sizes, sets, Wn, windows, options, result);
}

int tsg_treeseq_segregating_sites(const tsg_treeseq_t *self, uint64_t K, const uint64_t *sizes,
    const int32_t *sets, uint64_t Wn, const double *windows, uint32_t options, double *result)
{
    return one_way(self, TSG_SEGREGATING_SITES, K, sizes, sets, Wn, windows, options, result);
}

int tsg_treeseq_Y1(const tsg_treeseq_t *self, uint64_t K, const uint64_t *sizes,
    const int32_t *sets, uint64_t Wn, const double *windows, uint32_t options, double *result)
{
    return one_way(self, TSG_Y1, K, sizes, sets, Wn, windows, options, result);
}

#define TSG_K_WAY(name, type, width)                                                     \
    int name(const tsg_treeseq_t *self, uint64_t K, const uint64_t *sizes,               \
        const int32_t *sets, uint64_t nt, const int32_t *tuples, uint64_t Wn,            \
        const double *windows, uint32_t options, double *result)                         \
    {                                                                                    \
        return k_way(self, type, width, K, sizes, sets, nt, tuples, Wn, windows, options, \
            result);                                                                     \
    }

TSG_K_WAY(tsg_treeseq_divergence, TSG_DIVERGENCE, 2)
TSG_K_WAY(tsg_treeseq_Y2, TSG_Y2, 2)
TSG_K_WAY(tsg_treeseq_f2, TSG_F2, 2)
TSG_K_WAY(tsg_treeseq_Y3, TSG_Y3, 3)
TSG_K_WAY(tsg_treeseq_f3, TSG_F3, 3)
TSG_K_WAY(tsg_treeseq_f4, TSG_F4, 4)

int tsg_treeseq_genetic_relatedness(const tsg_treeseq_t *self, uint64_t K, const uint64_t *sizes,
    const int32_t *sets, uint64_t nt, const int32_t *tuples, uint64_t Wn, const double *windows,
    uint32_t options, double *result)
{
    int32_t type = (options & TSG_STAT_NONCENTRED) ? TSG_RELATEDNESS_NONCENTRED : TSG_RELATEDNESS;
    return k_way(self, type, 2, K, sizes, sets, nt, tuples, Wn, windows, options, result);
}

}  // extern "C"

// ------------------------------------------------ launch without allocation
//
// Some callers cannot allocate device memory while they run a query: a host
// application that hands this library a fixed device-memory budget and owns
// every allocation itself, or a latency-critical serving path where a
// cudaMalloc (with its implicit synchronisation) is not acceptable.  For them
// tsg_query_launch_noalloc runs a prepared query with its scratch taken from
// a fixed array that is part of this library's device image instead of a
// tsg_workspace_t.  The array is TSG_NOALLOC_SCRATCH_BYTES on every GPU that
// loads the library, for as long as the process lives.

static __device__ __align__(256) unsigned char g_noalloc_scratch[TSG_NOALLOC_SCRATCH_BYTES];
// The device-side check word of the last no-allocation launch on this GPU,
// copied out of the scratch array when the launch ends: a later launch of
// another query lays the array out differently and would overwrite the
// word's old position with its own data.
static __device__ __align__(16) int32_t g_noalloc_err[4];

namespace tsg {

// Device address of g_noalloc_scratch, looked up once per device with that
// device current (the host-side symbol is not a device address).
static std::mutex g_noalloc_mutex;
static void *g_noalloc_ptr[64];
static int32_t *g_noalloc_err_ptr[64];

static int noalloc_scratch(void **out, int32_t **err_word)
{
    int dev = 0;
    TSG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        return TSG_ERR_BAD_PARAM_VALUE;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (g_noalloc_ptr[dev] == nullptr) {
        void *p = nullptr, *pe = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            set_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
            return TSG_ERR_CUDA;
        }
        e = cudaGetSymbolAddress(&pe, g_noalloc_err);
        if (e != cudaSuccess) {
            set_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_err)");
            return TSG_ERR_CUDA;
        }
        g_noalloc_err_ptr[dev] = (int32_t *) pe;
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    *err_word = g_noalloc_err_ptr[dev];
    return 0;
}

}  // namespace tsg

extern "C" {

int tsg_query_launch_noalloc(const tsg_query_t *q, double *result_device, void *cuda_stream)
{
    if (q->ws_bytes > (int64_t) TSG_NOALLOC_SCRATCH_BYTES) {
        return TSG_ERR_NOALLOC_TOO_LARGE;
    }
    void *scratch = nullptr;
    int32_t *err_word = nullptr;
    int ret = noalloc_scratch(&scratch, &err_word);
    if (ret != 0) {
        return ret;
    }
    // a workspace descriptor over the static array: no device allocation;
    // every word the launch needs zeroed is cleared by the launch itself
    tsg_workspace_t ws{};
    ws.ptr = scratch;
    ws.bytes = (int64_t) TSG_NOALLOC_SCRATCH_BYTES;
    ret = tsg_query_launch(q, &ws, result_device, cuda_stream);
    if (ret != 0) {
        return ret;
    }
    // keep this launch's check word where tsg_noalloc_check reads it,
    // whatever query runs next (the word sits at the tail of the layout)
    TSG_CUDA(cudaMemcpyAsync(err_word, (const char *) scratch + q->ws_bytes - 256,
        sizeof(int32_t), cudaMemcpyDeviceToDevice, (cudaStream_t) cuda_stream));
    return 0;
}

int tsg_noalloc_check(const tsg_query_t *q)
{
    (void) q;
    void *scratch = nullptr;
    int32_t *err_word = nullptr;
    int ret = noalloc_scratch(&scratch, &err_word);
    if (ret != 0) {
        return ret;
    }
    int32_t h = 0;
    TSG_CUDA(cudaMemcpy(&h, err_word, sizeof(int32_t), cudaMemcpyDeviceToHost));
    return h == 0 ? 0 : TSG_ERR_DEVICE_CHECK;
}

}  // extern "C"
