// Branch-mode genetic relatedness matrix-vector product on the GPU.
//
// Replaces tsk_treeseq_genetic_relatedness_vector (c/tskit/trees.c:10402-
// 10816), which keeps per node: x[u] (position of its last update), w[u]
// (sum of the centred weights of the samples below u) and v[u] (area-weighted
// sums not yet pushed down to the samples), and maintains the invariant that
// a focal node's output is the sum of v over its root path: an edge event
// settles the accumulation of every node on the path (add_z), and moves v
// across the changed edge (the child's v absorbs the old ancestors' v on
// removal and cancels the new ancestors' v on insertion).  At a window end
// the path sums are read and v is cleared.
//
// The invariant makes the work separable along the genome: the output of a
// window is the sum over spans of the path sums each span's own accumulation
// gives on the span's last tree.  Here a work item is (a group of consecutive
// spans, 32 weight columns): one CTA rebuilds each span's first tree (parent
// pointers, and w bottom-up with every parent summing its children in edge
// order, so the sums are deterministic), warp 0 replays the span's edge
// events exactly as the reference does (lane = weight column, so each root
// path step is one coalesced row operation), and at window ends and at the
// span end all warps form the path sums: each stateful node's prefix
// Q[u] = v[u] + Q[parent] is computed once (memoised, claimed with a flag) and
// each focal node adds its own v.  A group writes its partial sums per window
// in span order; k_mv_reduce adds the groups in order, then the outputs are
// centred over the focal nodes and span-normalised (trees.c:10667-10700,
// 10772-10774).  All arithmetic is FP64.  A CTA's node state is its own, so
// every fence between its warps is block-scoped.
#include "tsg_query.cuh"

namespace tsg {

#define MV_NONE 0xFFFFFFFFu
#define MV_BUSY(e) (((e) << 2) | 1u)
#define MV_DONE(e) (((e) << 2) | 2u)
#define MV_SPIN_LIMIT (1 << 22)

// Per-CTA node state: stateful nodes (up to L) and the tree sequence's
// leaves (nL), 32 weight columns each.
struct MvSlot {
    double *time, *x, *v, *w;  // L, L, 32 L, 32 L
    uint32_t *par, *cnt, *flag;  // L each
    int32_t *segb, *sege;      // L each: the node's children in the span's alive list
    double *lx, *lv;           // nL, 32 nL
    uint32_t *lpar;            // nL
    uint32_t *stack;           // TSG_MV_WARPS x (L + 1)
    int32_t *gmap;             // N: stateful local id of a node (internal focal nodes)
};

__host__ __device__ static inline int64_t mv_align(int64_t v) { return (v + 255) / 256 * 256; }

__host__ __device__ static inline int64_t mv_layout(unsigned char *base, int64_t L, int64_t nL,
    int64_t N, MvSlot *s)
{
    int64_t off = 0;
    auto take = [&](int64_t bytes) {
        unsigned char *p = base + off;
        off += mv_align(bytes);
        return p;
    };
    MvSlot t;
    t.time = (double *) take(L * 8);
    t.x = (double *) take(L * 8);
    t.v = (double *) take(L * 32 * 8);
    t.w = (double *) take(L * 32 * 8);
    t.par = (uint32_t *) take(L * 4);
    t.cnt = (uint32_t *) take(L * 4);
    t.flag = (uint32_t *) take(L * 4);
    t.segb = (int32_t *) take(L * 4);
    t.sege = (int32_t *) take(L * 4);
    t.lx = (double *) take(nL * 8);
    t.lv = (double *) take(nL * 32 * 8);
    t.lpar = (uint32_t *) take(nL * 4);
    t.stack = (uint32_t *) take((int64_t) TSG_MV_WARPS * (L + 1) * 4);
    t.gmap = (int32_t *) take(N * 4);
    if (s != nullptr) {
        *s = t;
    }
    return off;
}

int64_t matvec_slot_bytes(const TSView &v, int64_t L)
{
    return mv_layout(nullptr, L, v.num_leaves, v.num_nodes, nullptr);
}

__device__ __forceinline__ uint32_t ld_flag(const uint32_t *p)
{
    return *(volatile const uint32_t *) p;
}

// centred weight of a leaf node for this lane's column
__device__ __forceinline__ double mv_leaf_w(const TSView &ts, const MvParams &m, int32_t g, int col)
{
    const int32_t si = ts.sample_index[g];
    return (si >= 0 && col < m.W) ? m.wc[(int64_t) si * m.W + col] : 0.0;
}

// Q[p] = sum of v over p's root path after settling each node at `pos`,
// memoised in v (flag DONE(epoch)); one warp, lane = column.
__device__ double mv_prefix(const MvSlot &S, const MvParams &m, uint32_t p, double pos,
    uint32_t epoch, int64_t Ls, uint32_t *stack)
{
    const int lane = threadIdx.x & 31;
    int64_t top = 0;
    uint32_t a = p;
    double base = 0.0;
    while (a != MV_NONE) {
        if (ld_flag(&S.flag[a]) == MV_DONE(epoch)) {
            __threadfence_block();
            base = __ldcg(&S.v[(int64_t) a * 32 + lane]);
            break;
        }
        if (top > Ls) {
            dev_error(m.err, DEV_PATH_TOO_LONG);
            return 0.0;
        }
        if (lane == 0) {
            stack[top] = a;
        }
        top++;
        a = S.par[a];
    }
    __syncwarp();
    for (int64_t k = top - 1; k >= 0; k--) {
        const uint32_t b = *(volatile uint32_t *) &stack[k];
        bool mine = false;
        for (int spin = 0;; spin++) {
            uint32_t f = 0;
            if (lane == 0) {
                f = ld_flag(&S.flag[b]);
            }
            f = __shfl_sync(0xffffffffu, f, 0);
            if (f == MV_DONE(epoch)) {
                break;
            }
            if (f == MV_BUSY(epoch)) {
                if (spin > MV_SPIN_LIMIT) {
                    dev_error(m.err, DEV_PATH_TOO_LONG);
                    return 0.0;
                }
                __nanosleep(32);
                continue;
            }
            uint32_t old = 0;
            if (lane == 0) {
                old = atomicCAS(&S.flag[b], f, MV_BUSY(epoch));
            }
            old = __shfl_sync(0xffffffffu, old, 0);
            if (old == f) {
                mine = true;
                break;
            }
        }
        if (mine) {
            const uint32_t pb = S.par[b];
            const double xb = S.x[b];
            double vb = S.v[(int64_t) b * 32 + lane];
            if (pb != MV_NONE && xb != pos) {
                vb += (S.time[pb] - S.time[b]) * (pos - xb) * S.w[(int64_t) b * 32 + lane];
            }
            const double q = vb + base;
            S.v[(int64_t) b * 32 + lane] = q;
            __threadfence_block();
            __syncwarp();
            if (lane == 0) {
                S.x[b] = pos;
                atomicExch(&S.flag[b], MV_DONE(epoch));
            }
            base = q;
        } else {
            __threadfence_block();
            base = __ldcg(&S.v[(int64_t) b * 32 + lane]);
        }
    }
    return base;
}

__global__ void __launch_bounds__(TSG_MV_WARPS * 32) k_mv_centre_weights(MvParams m, int64_t n)
{
    // one block per column: mean over the samples in a fixed tree order
    __shared__ double red[TSG_MV_WARPS * 32];
    const int col = blockIdx.x;
    double s = 0;
    if (m.centre) {
        const int64_t chunk = (n + blockDim.x - 1) / blockDim.x;
        const int64_t b = (int64_t) threadIdx.x * chunk;
        const int64_t e = b + chunk < n ? b + chunk : n;
        for (int64_t j = b; j < e; j++) {
            s += m.weights[j * m.W + col];
        }
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int) threadIdx.x < o) {
            red[threadIdx.x] += red[threadIdx.x + o];
        }
        __syncthreads();
    }
    const double mean = m.centre ? red[0] / (double) n : 0.0;
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        m.wc[j * m.W + col] = m.weights[j * m.W + col] - mean;
    }
}

__global__ void __launch_bounds__(TSG_MV_WARPS * 32) k_matvec(TSView ts, MvParams m)
{
    __shared__ int s_item;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nthreads = blockDim.x;
    MvSlot S;
    mv_layout(m.slots + (int64_t) blockIdx.x * m.slot_bytes, m.L, ts.num_leaves, ts.num_nodes, &S);
    uint32_t *stack = S.stack + (int64_t) warp * (m.L + 1);
    const int64_t nL = ts.num_leaves;
    const double W0 = m.windows[0], WE = m.windows[m.Wn];
    uint32_t epoch = 0;

    for (;;) {
        if (threadIdx.x == 0) {
            s_item = atomicAdd(m.counter, 1);
        }
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= m.G * m.ncb) {
            break;
        }
        const int g = item / m.ncb, cb = item % m.ncb;
        if (m.group_wlo[g] < 0) {
            continue;
        }
        const int col = cb * 32 + lane;
        int last_written = -1;
        for (int32_t s = m.group_span[g]; s < m.group_span[g + 1]; s++) {
            const int32_t t0 = ts.span_tree[s], t1 = ts.span_tree[s + 1];
            const double Xs = ts.breakpoints[t0], Xe = ts.breakpoints[t1];
            if (Xe <= W0 || Xs >= WE) {
                continue;
            }
            const int64_t lo = ts.span_local_off[s];
            const int32_t Ls = (int32_t) (ts.span_local_off[s + 1] - lo);
            const int32_t *l2g = ts.span_l2g + lo;
            const int64_t a0 = ts.span_alive_off[s], a1 = ts.span_alive_off[s + 1];

            // ---- seek: the first tree, x = span start, v = 0, w bottom-up
            for (int32_t l = threadIdx.x; l < Ls; l += nthreads) {
                const int32_t gl = l2g[l];
                S.time[l] = ts.node_time[gl];
                S.x[l] = Xs;
                S.par[l] = MV_NONE;
                S.cnt[l] = 0;
                S.flag[l] = 0;
                S.segb[l] = 0;
                S.sege[l] = 0;
                S.gmap[gl] = l;
            }
            for (int32_t l = warp; l < Ls; l += TSG_MV_WARPS) {
                const int32_t gl = l2g[l];
                S.v[(int64_t) l * 32 + lane] = 0.0;
                S.w[(int64_t) l * 32 + lane] = mv_leaf_w(ts, m, gl, col);
            }
            for (int64_t li = warp; li < nL; li += TSG_MV_WARPS) {
                S.lv[li * 32 + lane] = 0.0;
                if (lane == 0) {
                    S.lx[li] = Xs;
                    S.lpar[li] = MV_NONE;
                }
            }
            __syncthreads();
            for (int64_t i = a0 + threadIdx.x; i < a1; i += nthreads) {
                const int2 pc = ts.span_alive_enc[i];
                if (pc.y >= 0) {
                    S.par[pc.y] = (uint32_t) pc.x;
                } else {
                    S.lpar[ts.leaf_index[-pc.y - 1]] = (uint32_t) pc.x;
                }
                atomicAdd(&S.cnt[pc.x], 1u);
                if (i == a0 || ts.span_alive_enc[i - 1].x != pc.x) {
                    S.segb[pc.x] = (int32_t) (i - a0);
                }
                if (i == a1 - 1 || ts.span_alive_enc[i + 1].x != pc.x) {
                    S.sege[pc.x] = (int32_t) (i - a0 + 1);
                }
            }
            __syncthreads();
            for (int64_t i = a0 + warp; i < a1; i += TSG_MV_WARPS) {
                const int2 pc = ts.span_alive_enc[i];
                if (pc.y >= 0 && (__ldcg(&S.cnt[pc.y]) & 0xFFFFu) != 0) {
                    continue;  // completed by its own children
                }
                uint32_t p = (uint32_t) pc.x;
                for (int32_t guard = 0; p != MV_NONE; guard++) {
                    if (guard > Ls) {
                        dev_error(m.err, DEV_PATH_TOO_LONG);
                        break;
                    }
                    __threadfence_block();
                    __syncwarp();
                    uint32_t old = 0;
                    if (lane == 0) {
                        old = atomicAdd(&S.cnt[p], 0x10000u);
                    }
                    old = __shfl_sync(0xffffffffu, old, 0);
                    if ((old >> 16) + 1 != (old & 0xFFFFu)) {
                        break;
                    }
                    __threadfence_block();
                    // the last child to arrive: own weight plus the children in
                    // edge order
                    double acc = __ldcg(&S.w[(int64_t) p * 32 + lane]);
                    for (int32_t k = S.segb[p]; k < S.sege[p]; k++) {
                        const int32_t c = ts.span_alive_enc[a0 + k].y;
                        acc += c >= 0 ? __ldcg(&S.w[(int64_t) c * 32 + lane])
                                      : mv_leaf_w(ts, m, -c - 1, col);
                    }
                    S.w[(int64_t) p * 32 + lane] = acc;
                    p = S.par[p];
                }
            }
            __threadfence_block();
            __syncthreads();

            // ---- replay (warp 0) with window ends (all warps)
            auto transition = [&](int32_t t) {
                const double pos = ts.breakpoints[t];
                // settle node c's own area, then move v across the edge
                auto event = [&](int32_t p, int32_t c, double sign) {
                    double *vrow, *xp;
                    const double *wrow;
                    uint32_t *parp;
                    double tc, wc;
                    if (c >= 0) {
                        vrow = &S.v[(int64_t) c * 32 + lane];
                        wrow = &S.w[(int64_t) c * 32 + lane];
                        xp = &S.x[c];
                        parp = &S.par[c];
                        tc = S.time[c];
                        wc = *wrow;
                    } else {
                        const int32_t gl = -c - 1;
                        const int32_t li = ts.leaf_index[gl];
                        vrow = &S.lv[(int64_t) li * 32 + lane];
                        wrow = nullptr;
                        xp = &S.lx[li];
                        parp = &S.lpar[li];
                        tc = ts.node_time[gl];
                        wc = mv_leaf_w(ts, m, gl, col);
                    }
                    double vc = *vrow;
                    if (sign < 0) {
                        const uint32_t pc = *parp;
                        if (pc != MV_NONE) {
                            vc += (S.time[pc] - tc) * (pos - *xp) * wc;
                        }
                    }
                    // one root-path step per iteration; the next node's state is
                    // loaded before this node's is stored
                    uint32_t a = (uint32_t) p;
                    uint32_t pa = S.par[a];
                    double va = S.v[(int64_t) a * 32 + lane];
                    double wa = S.w[(int64_t) a * 32 + lane];
                    double xa = S.x[a], ta = S.time[a];
                    for (int32_t guard = 0; a != MV_NONE; guard++) {
                        if (guard > Ls) {
                            dev_error(m.err, DEV_PATH_TOO_LONG);
                            break;
                        }
                        uint32_t ppa = MV_NONE;
                        double vn = 0, wn = 0, xn = 0, tn = 0;
                        if (pa != MV_NONE) {
                            ppa = S.par[pa];
                            vn = S.v[(int64_t) pa * 32 + lane];
                            wn = S.w[(int64_t) pa * 32 + lane];
                            xn = S.x[pa];
                            tn = S.time[pa];
                            va += (tn - ta) * (pos - xa) * wa;
                        }
                        vc -= sign * va;
                        wa += sign * wc;
                        S.v[(int64_t) a * 32 + lane] = va;
                        S.w[(int64_t) a * 32 + lane] = wa;
                        __syncwarp();
                        if (lane == 0) {
                            S.x[a] = pos;
                        }
                        __syncwarp();
                        a = pa;
                        pa = ppa;
                        va = vn;
                        wa = wn;
                        xa = xn;
                        ta = tn;
                    }
                    *vrow = vc;
                    __syncwarp();
                    if (lane == 0) {
                        *xp = pos;
                        *parp = sign < 0 ? MV_NONE : (uint32_t) p;
                    }
                    __syncwarp();
                    (void) wrow;
                };
                for (int32_t r = ts.tree_out[t]; r < ts.tree_out[t + 1]; r++) {
                    const int2 pc = ts.rem_enc[r];
                    event(pc.x, pc.y, -1.0);
                }
                for (int32_t i = ts.tree_in[t]; i < ts.tree_in[t + 1]; i++) {
                    const int2 pc = ts.ins_enc[i];
                    event(pc.x, pc.y, +1.0);
                }
            };

            // path sums of every focal node at `pos` into the group's partial
            // block of window mw; clear v after a window end
            auto output = [&](double pos, int mw, bool window_end) {
                epoch++;
                const int64_t pair = m.pair_off[g] + (mw - m.group_wlo[g]);
                const bool first = mw > last_written;
                // settle every leaf at pos (only focal leaves reach the output)
                for (int64_t li = warp; li < nL; li += TSG_MV_WARPS) {
                    const double lx = S.lx[li];
                    if (lx != pos) {
                        const uint32_t p = S.lpar[li];
                        if (p != MV_NONE) {
                            const int32_t j = ts.leaves[li];
                            S.lv[li * 32 + lane] += (S.time[p] - ts.node_time[j]) * (pos - lx)
                                * mv_leaf_w(ts, m, j, col);
                        }
                        __syncwarp();
                        if (lane == 0) {
                            S.lx[li] = pos;
                        }
                    }
                }
                __threadfence_block();
                __syncthreads();
                for (int64_t i = warp; i < m.nf; i += TSG_MV_WARPS) {
                    const int32_t j = m.focal[i];
                    const int32_t li = ts.leaf_index[j];
                    double row = 0.0;
                    if (li >= 0) {
                        const uint32_t p = S.lpar[li];
                        row = S.lv[(int64_t) li * 32 + lane];
                        if (p != MV_NONE) {
                            row += mv_prefix(S, m, p, pos, epoch, Ls, stack);
                        }
                    } else {
                        const int32_t l = S.gmap[j];
                        if (l >= 0 && l < Ls && l2g[l] == j) {
                            row = mv_prefix(S, m, (uint32_t) l, pos, epoch, Ls, stack);
                        }
                    }
                    if (col < m.W) {
                        double *o = m.partial + (pair * m.nf + i) * m.W + col;
                        *o = first ? row : *o + row;
                    }
                }
                last_written = mw;
                __threadfence_block();
                __syncthreads();
                if (window_end) {
                    for (int32_t l = warp; l < Ls; l += TSG_MV_WARPS) {
                        S.v[(int64_t) l * 32 + lane] = 0.0;
                    }
                    for (int64_t li = warp; li < nL; li += TSG_MV_WARPS) {
                        S.lv[li * 32 + lane] = 0.0;
                    }
                    __syncthreads();
                }
            };

            int mw = Xs < W0 ? -1 : (int) upper_bound(m.windows, (int64_t) m.Wn + 1, Xs) - 1;
            // warp 0 replays up to the tree holding the next window boundary
            // (the other warps wait: they are needed only at window ends),
            // then all warps handle the boundaries that tree reaches
            int32_t t = t0;
            while (t < t1 && mw < m.Wn) {
                const double B = mw < 0 ? W0 : m.windows[mw + 1];
                int32_t te = t1 - 1;
                if (B <= Xe) {
                    te = t + (int32_t) lower_bound(ts.breakpoints + t + 1, (int64_t) (t1 - t), B);
                }
                if (warp == 0) {
                    for (int32_t tt = t > t0 ? t : t0 + 1; tt <= te; tt++) {
                        transition(tt);
                    }
                }
                __threadfence_block();
                __syncthreads();
                if (B > Xe) {
                    break;
                }
                const double right = ts.breakpoints[te + 1];
                while (mw < m.Wn) {
                    const double Bw = mw < 0 ? W0 : m.windows[mw + 1];
                    if (Bw > right) {
                        break;
                    }
                    if (mw < 0) {
                        // accumulation starts at the first window
                        for (int32_t l = threadIdx.x; l < Ls; l += nthreads) {
                            S.x[l] = Bw;
                        }
                        for (int64_t li = threadIdx.x; li < nL; li += nthreads) {
                            S.lx[li] = Bw;
                        }
                        for (int32_t l = warp; l < Ls; l += TSG_MV_WARPS) {
                            S.v[(int64_t) l * 32 + lane] = 0.0;
                        }
                        for (int64_t li = warp; li < nL; li += TSG_MV_WARPS) {
                            S.lv[li * 32 + lane] = 0.0;
                        }
                        __syncthreads();
                        mw = 0;
                    } else {
                        output(Bw, mw, true);
                        mw++;
                    }
                }
                t = te + 1;
            }
            if (mw >= 0 && mw < m.Wn && m.windows[mw] < Xe) {
                output(Xe, mw, false);
            }
            __syncthreads();
        }
    }
}

// Sum of the groups' partial blocks for each window, in group order.
__global__ void __launch_bounds__(256) k_mv_reduce(MvParams m, double *result)
{
    const int64_t per = m.nf * m.W;
    const int64_t total = (int64_t) m.Wn * per;
    for (int64_t idx = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t) gridDim.x * blockDim.x) {
        const int mw = (int) (idx / per);
        const int64_t r = idx % per;
        double y = 0;
        for (int32_t g = m.win_glo[mw]; g <= m.win_ghi[mw]; g++) {
            y += m.partial[(m.pair_off[g] + (mw - m.group_wlo[g])) * per + r];
        }
        result[idx] = y;
    }
}

// Centre each window's outputs over the focal nodes (per column), then span
// normalise.  One block per (window, column).
__global__ void __launch_bounds__(256) k_mv_finish(MvParams m, int span_normalise, double *result)
{
    __shared__ double red[256];
    const int mw = blockIdx.x / m.W, col = blockIdx.x % m.W;
    double *y = result + (int64_t) mw * m.nf * m.W + col;
    double mean = 0;
    if (m.centre) {
        const int64_t chunk = (m.nf + blockDim.x - 1) / blockDim.x;
        const int64_t b = (int64_t) threadIdx.x * chunk;
        const int64_t e = b + chunk < m.nf ? b + chunk : m.nf;
        double s = 0;
        for (int64_t i = b; i < e; i++) {
            s += y[i * m.W];
        }
        red[threadIdx.x] = s;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if ((int) threadIdx.x < o) {
                red[threadIdx.x] += red[threadIdx.x + o];
            }
            __syncthreads();
        }
        mean = red[0] / (double) m.nf;
    }
    const double span = m.windows[mw + 1] - m.windows[mw];
    for (int64_t i = threadIdx.x; i < m.nf; i += blockDim.x) {
        double v = y[i * m.W] - mean;
        if (span_normalise) {
            v /= span;
        }
        y[i * m.W] = v;
    }
}

const void *k_matvec_ptr() { return (const void *) k_matvec; }

int launch_matvec(unsigned grid, cudaStream_t st, const TSView &v, const MvParams &m,
    int span_normalise, double *result)
{
    if (m.W == 0 || m.nf == 0) {
        return 0;
    }
    k_mv_centre_weights<<<(unsigned) m.W, TSG_MV_WARPS * 32, 0, st>>>(m, v.num_samples);
    TSG_LAUNCHED();
    k_matvec<<<grid, TSG_MV_WARPS * 32, 0, st>>>(v, m);
    TSG_LAUNCHED();
    const int64_t total = (int64_t) m.Wn * m.nf * m.W;
    const int64_t blocks = std::min<int64_t>((total + 255) / 256, 65535LL * 4);
    k_mv_reduce<<<(unsigned) std::max<int64_t>(blocks, 1), 256, 0, st>>>(m, result);
    TSG_LAUNCHED();
    k_mv_finish<<<(unsigned) ((int64_t) m.Wn * m.W), 256, 0, st>>>(m, span_normalise, result);
    TSG_LAUNCHED();
    return 0;
}

}  // namespace tsg
