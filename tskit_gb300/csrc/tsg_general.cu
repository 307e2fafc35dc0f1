// Statistics with an arbitrary summary function (general_stat /
// sample_count_stat with a user callback, c/tskit/trees.c:1352-1776 with
// general_stat_func_t, python/tskit/trees.py:7917-8105).
//
// The callback cannot run on the GPU, but it is only ever evaluated at the
// count vectors the sweep meets, and those are few next to the number of
// evaluations: the item replay runs as for the built-in statistics, every
// count vector it produces (both sides of every branch item, every allele
// state of every site) is gathered, sorted and deduplicated on the device,
// the host evaluates the callback once per distinct vector, and the items
// are then valued by binary search in that table (FP64) and reduced exactly
// as the built-in statistics are.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "tsg_fixed.cuh"
#include "tsg_replay.cuh"

namespace tsg {

__device__ __forceinline__ void key_put(uint64_t *klo, uint64_t *khi, int64_t i, const Pack &x)
{
    klo[i] = x.lo;
    khi[i] = x.hi;
}

// Two keys per item: the counts its value reads (before and after; the
// "after" counts twice when there was no branch before or the counts did
// not change).
template <int W, int KQ>
__global__ void __launch_bounds__(256) k_gen_keys_items(TSView ts, QueryParams q, WsDev w,
    uint64_t *klo, uint64_t *khi)
{
    const Item<KQ> *items = (const Item<KQ> *) w.items;
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < ts.num_items;
         i += (int64_t) gridDim.x * blockDim.x) {
        const Item<KQ> it = items[i];
        const Pack b = item_pack<KQ>(it.x1);
        const Pack a = it.p0 >= 0 ? item_pack<KQ>(it.x0) : b;
        key_put(klo, khi, 2 * i, a);
        key_put(klo, khi, 2 * i + 1, b);
    }
}

// Allele states of one site (get_allele_weights, trees.c:1525-1612) in
// integers; calls emit(allele, state) for every allele.
template <int W, int KQ, typename Emit>
__device__ __forceinline__ void site_states(const TSView &ts, const QueryParams &q,
    const uint64_t *mcnt, int64_t site, int32_t A, Emit emit)
{
    const int32_t m0 = ts.site_mut[site], m1 = ts.site_mut[site + 1];
    constexpr int KM = 2 * (64 / W);
    for (int32_t a = 0; a < A; a++) {
        int64_t st[KM];
#pragma unroll
        for (int k = 0; k < KM; k++) {
            st[k] = (a == 0 && k < q.K) ? (int64_t) q.set_size[k] : 0;
        }
        for (int32_t m = m0; m < m1; m++) {
            Pack xm;
            xm.lo = mcnt[(int64_t) m * KQ];
            xm.hi = KQ > 1 ? mcnt[(int64_t) m * KQ + (KQ > 1 ? 1 : 0)] : 0ull;
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
        emit(a, ps);
    }
}

template <int W, int KQ>
__global__ void __launch_bounds__(256) k_gen_keys_sites(TSView ts, QueryParams q,
    const uint64_t *mcnt, const int64_t *site_off, uint64_t *klo, uint64_t *khi, int64_t base)
{
    const int64_t s = blockIdx.x * (int64_t) blockDim.x + threadIdx.x;
    if (s >= ts.num_sites) {
        return;
    }
    const int64_t o = base + site_off[s];
    site_states<W, KQ>(ts, q, mcnt, s, (int32_t) (site_off[s + 1] - site_off[s]),
        [&](int32_t a, const Pack &x) { key_put(klo, khi, o + a, x); });
}

// the membership pattern of every possible leaf (branch mode: leaves are
// accounted per pattern)
template <int W>
__global__ void k_gen_keys_patterns(int K, uint64_t *klo, uint64_t *khi, int64_t base)
{
    const int np = 1 << K;
    for (int pat = blockIdx.x * blockDim.x + threadIdx.x; pat < np; pat += gridDim.x * blockDim.x) {
        key_put(klo, khi, base + pat, pk_from_mask<W>((uint32_t) pat, K));
    }
}

__global__ void k_gen_flags(const uint64_t *lo, const uint64_t *hi, int64_t n, int64_t *flag)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n;
         i += (int64_t) gridDim.x * blockDim.x) {
        flag[i] = (i == 0 || lo[i] != lo[i - 1] || hi[i] != hi[i - 1]) ? 1 : 0;
    }
}

__global__ void k_gen_compact(const uint64_t *lo, const uint64_t *hi, const int64_t *pos,
    const int64_t *flag, int64_t n, uint64_t *ulo, uint64_t *uhi)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n;
         i += (int64_t) gridDim.x * blockDim.x) {
        if (flag[i]) {
            ulo[pos[i]] = lo[i];
            uhi[pos[i]] = hi[i];
        }
    }
}

// index of key (hi, lo) in the sorted distinct keys
__device__ __forceinline__ int64_t gen_lookup(const uint64_t *ulo, const uint64_t *uhi,
    int64_t U, const Pack &x)
{
    int64_t a = 0, b = U;
    while (a < b) {
        const int64_t m = (a + b) >> 1;
        const bool less = uhi[m] < x.hi || (uhi[m] == x.hi && ulo[m] < x.lo);
        if (less) {
            a = m + 1;
        } else {
            b = m;
        }
    }
    // every looked-up vector was collected; stay inside the table regardless
    return a < U ? a : U - 1;
}

// Item values for outputs [r0, r0 + q.R) of the table F (U x R_total), one
// warp per chunk, FP64.
template <int W, int KQ, int RMAX>
__global__ void __launch_bounds__(256) k_gen_eval_items(TSView ts, QueryParams q, WsDev w,
    const uint64_t *ulo, const uint64_t *uhi, int64_t U, const double *F, int32_t R_total,
    int32_t r0)
{
    const int lane = threadIdx.x & 31;
    const int R = q.R;
    const int64_t c = (int64_t) blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= ts.num_chunks) {
        return;
    }
    const Item<KQ> *items = (const Item<KQ> *) w.items;
    const double *time = ts.span_time + ts.span_local_off[ts.chunk_span[c]];
    double acc[RMAX];
#pragma unroll
    for (int r = 0; r < RMAX; r++) {
        acc[r] = 0;
    }
    for (int64_t i = ts.chunk_begin[c] + lane; i < ts.chunk_end[c]; i += 32) {
        const Item<KQ> it = items[i];
        double bl0, bl1;
        item_branches<KQ>(it, time, bl0, bl1);
        const Pack x0 = item_pack<KQ>(it.x0), x1 = item_pack<KQ>(it.x1);
        const bool same = x0.lo == x1.lo && x0.hi == x1.hi;
        const double *f1 = F + gen_lookup(ulo, uhi, U, x1) * R_total + r0;
        if (!same && bl0 != 0) {
            const double *f0 = F + gen_lookup(ulo, uhi, U, x0) * R_total + r0;
            const bool path = bl0 == bl1;
#pragma unroll
            for (int r = 0; r < RMAX; r++) {
                if (r < R) {
                    acc[r] += path ? bl1 * (f1[r] - f0[r]) : bl1 * f1[r] - bl0 * f0[r];
                }
            }
        } else {
            const double c1 = same ? bl1 - bl0 : bl1;
#pragma unroll
            for (int r = 0; r < RMAX; r++) {
                if (r < R) {
                    acc[r] += c1 * f1[r];
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < RMAX; r++) {
        if (r < R) {
            const double v = warp_sum(acc[r]);
            if (lane == r) {
                w.dD[c * R + r] = v;
            }
        }
    }
}

// Each site: the sum over its alleles (the ancestral one skipped when
// polarised) of f at the allele's state (trees.c:1614-1652).
template <int W, int KQ, int RMAX>
__global__ void __launch_bounds__(256) k_gen_eval_sites(TSView ts, QueryParams q, WsDev w,
    const int64_t *site_off, const uint64_t *ulo, const uint64_t *uhi, int64_t U, const double *F,
    int32_t R_total, int32_t r0)
{
    const int64_t s = blockIdx.x * (int64_t) blockDim.x + threadIdx.x;
    if (s >= ts.num_sites) {
        return;
    }
    const int R = q.R;
    double val[RMAX];
#pragma unroll
    for (int r = 0; r < RMAX; r++) {
        val[r] = 0;
    }
    site_states<W, KQ>(ts, q, w.mcnt, s, (int32_t) (site_off[s + 1] - site_off[s]),
        [&](int32_t a, const Pack &x) {
            if (a == 0 && q.polarised) {
                return;
            }
            const double *f = F + gen_lookup(ulo, uhi, U, x) * R_total + r0;
#pragma unroll
            for (int r = 0; r < RMAX; r++) {
                if (r < R) {
                    val[r] += f[r];
                }
            }
        });
#pragma unroll
    for (int r = 0; r < RMAX; r++) {
        if (r < R) {
            w.site_val[(int64_t) r * ts.num_sites + s] = val[r];
        }
    }
}

// The leaves' window sums from the table: sum over patterns of F(pattern) x
// the pattern's branch area in the window.
template <int W>
__global__ void __launch_bounds__(256) k_gen_leaf_terms(QueryParams q, WsDev w,
    const uint64_t *ulo, const uint64_t *uhi, int64_t U, const double *F, int32_t R_total,
    int32_t r0)
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
                v += F[gen_lookup(ulo, uhi, U, x) * R_total + r0 + r] * area;
            }
        }
        w.leaf_win[idx] = v;
    }
}

static unsigned gen_grid(int64_t n)
{
    const int64_t g = (n + 255) / 256;
    return (unsigned) (g < 1 ? 1 : (g > 65535LL * 8 ? 65535LL * 8 : g));
}

// Keys of every count vector the query's replay produced: items (branch)
// and allele states (site), sorted and deduplicated.  Returns the number of
// distinct keys in *U (device arrays ulo / uhi hold them).
int gen_collect(int form, const TSView &v, const QueryParams &q, const WsDev &w,
    const int64_t *site_off, int64_t num_site_keys, uint64_t *klo, uint64_t *khi, uint64_t *tlo,
    uint64_t *thi, int64_t *flag, int64_t *pos, void *cub_tmp, size_t cub_bytes, uint64_t *ulo,
    uint64_t *uhi, int64_t *U, cudaStream_t st)
{
    const int64_t ni = q.branch ? 2 * v.num_items + ((int64_t) 1 << q.K) : 0;
    const int64_t n = ni + (q.site ? num_site_keys : 0);
    if (n == 0) {
        *U = 0;
        return 0;
    }
    if (q.branch && v.num_items > 0) {
        switch (form) {
            case 0: k_gen_keys_items<16, 1><<<gen_grid(v.num_items), 256, 0, st>>>(v, q, w, klo, khi); break;
            case 1: k_gen_keys_items<16, 2><<<gen_grid(v.num_items), 256, 0, st>>>(v, q, w, klo, khi); break;
            case 2: k_gen_keys_items<32, 1><<<gen_grid(v.num_items), 256, 0, st>>>(v, q, w, klo, khi); break;
            default: k_gen_keys_items<32, 2><<<gen_grid(v.num_items), 256, 0, st>>>(v, q, w, klo, khi); break;
        }
        TSG_LAUNCHED();
    }
    if (q.branch) {
        const int64_t base = 2 * v.num_items;
        if (form < 2) {
            k_gen_keys_patterns<16><<<gen_grid((int64_t) 1 << q.K), 256, 0, st>>>(q.K, klo, khi, base);
        } else {
            k_gen_keys_patterns<32><<<gen_grid((int64_t) 1 << q.K), 256, 0, st>>>(q.K, klo, khi, base);
        }
        TSG_LAUNCHED();
    }
    if (q.site && v.num_sites > 0) {
        const unsigned g = (unsigned) ((v.num_sites + 255) / 256);
        switch (form) {
            case 0: k_gen_keys_sites<16, 1><<<g, 256, 0, st>>>(v, q, w.mcnt, site_off, klo, khi, ni); break;
            case 1: k_gen_keys_sites<16, 2><<<g, 256, 0, st>>>(v, q, w.mcnt, site_off, klo, khi, ni); break;
            case 2: k_gen_keys_sites<32, 1><<<g, 256, 0, st>>>(v, q, w.mcnt, site_off, klo, khi, ni); break;
            default: k_gen_keys_sites<32, 2><<<g, 256, 0, st>>>(v, q, w.mcnt, site_off, klo, khi, ni); break;
        }
        TSG_LAUNCHED();
    }
    // stable LSD order: by the low word, then by the high word
    size_t bytes = cub_bytes;
    if (cub::DeviceRadixSort::SortPairs(cub_tmp, bytes, klo, tlo, khi, thi, (int) n, 0, 64, st)
        != cudaSuccess) {
        return TSG_ERR_CUDA;
    }
    bytes = cub_bytes;
    if (cub::DeviceRadixSort::SortPairs(cub_tmp, bytes, thi, khi, tlo, klo, (int) n, 0, 64, st)
        != cudaSuccess) {
        return TSG_ERR_CUDA;
    }
    k_gen_flags<<<gen_grid(n), 256, 0, st>>>(klo, khi, n, flag);
    TSG_LAUNCHED();
    bytes = cub_bytes;
    if (cub::DeviceScan::ExclusiveSum(cub_tmp, bytes, flag, pos, (int) n, st) != cudaSuccess) {
        return TSG_ERR_CUDA;
    }
    k_gen_compact<<<gen_grid(n), 256, 0, st>>>(klo, khi, pos, flag, n, ulo, uhi);
    TSG_LAUNCHED();
    int64_t last_pos = 0, last_flag = 0;
    TSG_CUDA(cudaMemcpyAsync(&last_pos, pos + n - 1, 8, cudaMemcpyDeviceToHost, st));
    TSG_CUDA(cudaMemcpyAsync(&last_flag, flag + n - 1, 8, cudaMemcpyDeviceToHost, st));
    TSG_CUDA(cudaStreamSynchronize(st));
    *U = last_pos + last_flag;
    return 0;
}

size_t gen_cub_bytes(int64_t n)
{
    size_t a = 0, b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, a, (uint64_t *) nullptr, (uint64_t *) nullptr,
        (uint64_t *) nullptr, (uint64_t *) nullptr, (int) n, 0, 64);
    cub::DeviceScan::ExclusiveSum(nullptr, b, (int64_t *) nullptr, (int64_t *) nullptr, (int) n);
    return std::max(a, b);
}

int gen_eval(int form, const TSView &v, const QueryParams &q, const WsDev &w,
    const int64_t *site_off, const uint64_t *ulo, const uint64_t *uhi, int64_t U, const double *F,
    int32_t R_total, int32_t r0, cudaStream_t st)
{
    if (q.branch && v.num_chunks > 0) {
        const unsigned ge = (unsigned) ((v.num_chunks + 7) / 8);
        switch (form) {
            case 0: k_gen_eval_items<16, 1, 32><<<ge, 256, 0, st>>>(v, q, w, ulo, uhi, U, F, R_total, r0); break;
            case 1: k_gen_eval_items<16, 2, 32><<<ge, 256, 0, st>>>(v, q, w, ulo, uhi, U, F, R_total, r0); break;
            case 2: k_gen_eval_items<32, 1, 32><<<ge, 256, 0, st>>>(v, q, w, ulo, uhi, U, F, R_total, r0); break;
            default: k_gen_eval_items<32, 2, 32><<<ge, 256, 0, st>>>(v, q, w, ulo, uhi, U, F, R_total, r0); break;
        }
        TSG_LAUNCHED();
    }
    if (q.branch) {
        const unsigned gl = gen_grid((int64_t) q.Wn * q.R);
        if (form < 2) {
            k_gen_leaf_terms<16><<<gl, 256, 0, st>>>(q, w, ulo, uhi, U, F, R_total, r0);
        } else {
            k_gen_leaf_terms<32><<<gl, 256, 0, st>>>(q, w, ulo, uhi, U, F, R_total, r0);
        }
        TSG_LAUNCHED();
    }
    if (q.site && v.num_sites > 0) {
        const unsigned g = (unsigned) ((v.num_sites + 255) / 256);
        switch (form) {
            case 0: k_gen_eval_sites<16, 1, 32><<<g, 256, 0, st>>>(v, q, w, site_off, ulo, uhi, U, F, R_total, r0); break;
            case 1: k_gen_eval_sites<16, 2, 32><<<g, 256, 0, st>>>(v, q, w, site_off, ulo, uhi, U, F, R_total, r0); break;
            case 2: k_gen_eval_sites<32, 1, 32><<<g, 256, 0, st>>>(v, q, w, site_off, ulo, uhi, U, F, R_total, r0); break;
            default: k_gen_eval_sites<32, 2, 32><<<g, 256, 0, st>>>(v, q, w, site_off, ulo, uhi, U, F, R_total, r0); break;
        }
        TSG_LAUNCHED();
    }
    return 0;
}

// Distinct keys unpacked to count vectors (U x K int32).
template <int W>
__global__ void k_gen_unpack(const uint64_t *ulo, const uint64_t *uhi, int64_t U, int K,
    int32_t *out)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < U;
         i += (int64_t) gridDim.x * blockDim.x) {
        const Pack p{ulo[i], uhi[i]};
        for (int k = 0; k < K; k++) {
            out[i * K + k] = (int32_t) pk_get<W>(p, k);
        }
    }
}

int gen_unpack(int W, const uint64_t *ulo, const uint64_t *uhi, int64_t U, int K, int32_t *out,
    cudaStream_t st)
{
    if (U == 0) {
        return 0;
    }
    if (W == 16) {
        k_gen_unpack<16><<<gen_grid(U), 256, 0, st>>>(ulo, uhi, U, K, out);
    } else {
        k_gen_unpack<32><<<gen_grid(U), 256, 0, st>>>(ulo, uhi, U, K, out);
    }
    TSG_LAUNCHED();
    return 0;
}

// ---------------------------------------------------------------------------
// Real-valued weights (general_stat with W f64 [n x K], c/tskit/trees.c:
// 1352-1776 with arbitrary weights): the states are the weights below each
// node, K doubles.  Same span plan and touch-list semantics as the counting
// replay (the items land where the plan puts them), one warp replaying each
// span with the node state in a per-CTA global slot; every state an item,
// a site or a leaf needs is listed for the host's summary function (real
// states rarely repeat, so they are not deduplicated).  Deterministic: the
// seek adds children in edge order, one warp replays in reference order.

// Replay: items (ids, and states x0 | x1 per item), states under every
// mutation.  Lane k carries weight component k (K <= 32) in the seek; a
// root-path batch takes one node per lane, each adding all components.
__global__ void __launch_bounds__(64) k_wreplay(TSView ts, QueryParams q, const double *W,
    int node_w, int K, double *slots_x, int32_t *slots_par, uint8_t *slots_touched, int4 *ids,
    double *xs, double *mstate, double *init, int32_t *err, int32_t *counter)
{
    __shared__ int s_span;
    __shared__ int32_t s_list[TSG_TOUCH_CAP];
    const int64_t L = ts.max_local;
    double *x = slots_x + (int64_t) blockIdx.x * L * K;
    int32_t *par = slots_par + (int64_t) blockIdx.x * L;
    uint8_t *touched = slots_touched + (int64_t) blockIdx.x * L;
    const int lane = threadIdx.x & 31;
    // a node's own weight: W by sample index, or by node id (node_w)
    auto leaf_w = [&](int32_t g, int k) {
        if (node_w) {
            return k < K ? W[(int64_t) g * K + k] : 0.0;
        }
        const int32_t si = ts.sample_index[g];
        return si >= 0 && k < K ? W[(int64_t) si * K + k] : 0.0;
    };
    for (;;) {
        if (threadIdx.x == 0) {
            s_span = atomicAdd(counter, 1);
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
        const double *time = ts.span_time + lo;
        const int64_t a0 = ts.span_alive_off[s], a1 = ts.span_alive_off[s + 1];
        for (int32_t l = threadIdx.x; l < Ls; l += blockDim.x) {
            par[l] = -1;
            touched[l] = 0;
            for (int k = 0; k < K; k++) {
                x[(int64_t) l * K + k] = leaf_w(l2g[l], k);
            }
        }
        __syncthreads();
        if (threadIdx.x >= 32) {
            continue;
        }
        // seek: the alive edges in edge order (children before parents);
        // lane k adds component k
        for (int64_t i = a0; i < a1; i++) {
            const int2 pc = ts.span_alive_enc[i];
            if (lane < K) {
                const double xc = pc.y >= 0 ? x[(int64_t) pc.y * K + lane] : leaf_w(-pc.y - 1, lane);
                x[(int64_t) pc.x * K + lane] += xc;
            }
            if (lane == 0 && pc.y >= 0) {
                par[pc.y] = pc.x;
            }
        }
        __syncwarp();
        // node mode: the first tree's state of every stateful node of span 0
        if (init != nullptr && s == 0) {
            for (int32_t l = lane; l < Ls; l += 32) {
                const int32_t gl = l2g[l];
                if (gl < 0 || gl >= ts.num_nodes) {
                    dev_error(err, DEV_NODE_OUT_OF_BOUNDS);
                    continue;
                }
                for (int k = 0; k < K; k++) {
                    init[(int64_t) gl * K + k] = x[(int64_t) l * K + k];
                }
            }
            __syncwarp();
        }
        // first tree of the sequence: its stateful nodes in alive-list order
        if (q.branch && s == 0) {
            int64_t at = ts.tree_item_off[t0];
            for (int64_t i = a0; i < a1; i++) {
                const int2 pc = ts.span_alive_enc[i];
                if (pc.y < 0) {
                    continue;
                }
                if (at < ts.tree_item_off[t0 + 1]) {
                    if (lane == 0) {
                        ids[at] = make_int4(pc.y, -1, pc.x, 0);
                    }
                    if (lane < K) {
                        xs[(2 * at) * K + lane] = 0.0;
                        xs[(2 * at + 1) * K + lane] = x[(int64_t) pc.y * K + lane];
                    }
                }
                at++;
            }
            if (lane == 0 && at != ts.tree_item_off[t0 + 1]) {
                dev_error(err, DEV_ITEM_PLAN);
            }
        }
        int64_t cursor = 0, climit = 0;
        int32_t nopen = 0;
        auto close_list = [&]() {
            __syncwarp();
            for (int32_t i = lane; i < nopen; i += 32) {
                const int32_t u = s_list[i];
                if (cursor + i < climit) {
                    ids[cursor + i].z = par[u];
                    for (int k = 0; k < K; k++) {
                        xs[(2 * (cursor + i) + 1) * K + k] = x[(int64_t) u * K + k];
                    }
                }
                touched[u] = 0;
            }
            __syncwarp();
            cursor += nopen;
            nopen = 0;
        };
        // lanes with `active` set touch node u (distinct per lane), parent p0
        auto touch = [&](bool active, int32_t u, int32_t p0) {
            bool fresh = active && !touched[u];
            unsigned m = __ballot_sync(0xffffffffu, fresh);
            if (nopen + __popc(m) > TSG_TOUCH_CAP) {
                close_list();
                fresh = active;
                m = __ballot_sync(0xffffffffu, fresh);
            }
            if (fresh) {
                const int32_t at = nopen + __popc(m & ((1u << lane) - 1u));
                s_list[at] = u;
                touched[u] = 1;
                if (cursor + at < climit) {
                    ids[cursor + at] = make_int4(u, p0, -1, 0);
                    for (int k = 0; k < K; k++) {
                        xs[(2 * (cursor + at)) * K + k] = x[(int64_t) u * K + k];
                    }
                } else {
                    dev_error(err, DEV_ITEM_PLAN);
                }
            }
            nopen += __popc(m);
            __syncwarp();
        };
        // touches in the counting replay's batches: a stateful child on
        // lane 0 with the first 31 nodes of the parent's root path, then 32
        // path nodes at a time (the span plan counts items so)
        auto event = [&](int32_t p, int32_t c, int sign) {
            double xc[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                xc[k] = k < K ? (c >= 0 ? x[(int64_t) c * K + k] : leaf_w(-c - 1, k)) : 0.0;
            }
            int32_t v = p;
            int32_t batches = 0;
            bool first = true;
            while (v >= 0) {
                const bool is_child = first && c >= 0 && lane == 0;
                int32_t mine = -1;
                for (int j = (first && c >= 0) ? 1 : 0; j < 32 && v >= 0; j++) {
                    if (lane == j) {
                        mine = v;
                    }
                    v = par[v];
                }
                if (++batches > (Ls >> 5) + 1) {
                    dev_error(err, DEV_PATH_TOO_LONG);
                    v = -1;
                }
                int32_t up = __shfl_down_sync(0xffffffffu, mine, 1);
                if (lane == 31) {
                    up = v;
                }
                if (is_child) {
                    mine = c;
                    up = par[c];
                }
                const bool act = mine >= 0;
                if (q.branch) {
                    touch(act, mine, act ? up : -1);
                }
                if (is_child) {
                    par[c] = sign > 0 ? p : -1;
                } else if (act && K <= 8) {
#pragma unroll
                    for (int k = 0; k < 8; k++) {
                        if (k < K) {
                            x[(int64_t) mine * K + k] += sign > 0 ? xc[k] : -xc[k];
                        }
                    }
                } else if (act) {
                    // more components than registers: the child's state
                    // (not on the path, so unchanged here) read again
                    for (int k = 0; k < K; k++) {
                        const double xk = c >= 0 ? x[(int64_t) c * K + k] : leaf_w(-c - 1, k);
                        x[(int64_t) mine * K + k] += sign > 0 ? xk : -xk;
                    }
                }
                __syncwarp();
                first = false;
            }
        };
        const int32_t tend = q.branch && t1 < ts.num_trees ? t1 + 1 : t1;
        for (int32_t t = t0; t < tend; t++) {
            if (t > t0) {
                cursor = ts.tree_item_off[t];
                climit = ts.tree_item_off[t + 1];
                for (int32_t i = ts.tree_out[t]; i < ts.tree_out[t + 1]; i++) {
                    const int2 pc = ts.rem_enc[i];
                    event(pc.x, pc.y, -1);
                }
                for (int32_t i = ts.tree_in[t]; i < ts.tree_in[t + 1]; i++) {
                    const int2 pc = ts.ins_enc[i];
                    event(pc.x, pc.y, +1);
                }
                if (q.branch) {
                    close_list();
                    if (lane == 0 && cursor != climit) {
                        dev_error(err, DEV_ITEM_PLAN);
                    }
                }
            }
            if (q.site && t < t1) {
                const int32_t m0 = ts.site_mut[ts.tree_sites[t]];
                const int32_t m1 = ts.site_mut[ts.tree_sites[t + 1]];
                for (int32_t m = m0; m < m1; m++) {
                    const int32_t enc = ts.mut_enc[m];
                    if (lane < K) {
                        mstate[(int64_t) m * K + lane] =
                            enc >= 0 ? x[(int64_t) enc * K + lane] : leaf_w(-enc - 1, lane);
                    }
                }
            }
            __syncwarp();
        }
    }
}

// Allele states of every site (get_allele_weights, trees.c:1525-1612) and
// the weights of every leaf, appended to the state list.
__global__ void k_wsite_states(TSView ts, int K, const double *total, const double *mstate,
    const int64_t *site_off, double *states)
{
    for (int64_t site = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; site < ts.num_sites;
         site += (int64_t) gridDim.x * blockDim.x) {
        const int32_t m0 = ts.site_mut[site], m1 = ts.site_mut[site + 1];
        const int64_t A = site_off[site + 1] - site_off[site];
        for (int64_t a = 0; a < A; a++) {
            double *st = states + (site_off[site] + a) * K;
            for (int k = 0; k < K; k++) {
                double v = a == 0 ? total[k] : 0.0;
                for (int32_t m = m0; m < m1; m++) {
                    if (ts.mutation_allele[m] == a) {
                        v += mstate[(int64_t) m * K + k];
                    }
                    if (ts.mutation_alt[m] == a) {
                        v -= mstate[(int64_t) m * K + k];
                    }
                }
                st[k] = v;
            }
        }
    }
}

__global__ void k_wleaf_states(TSView ts, int K, const double *W, double *states)
{
    for (int64_t li = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; li < ts.num_leaves;
         li += (int64_t) gridDim.x * blockDim.x) {
        const int32_t si = ts.sample_index[ts.leaves[li]];
        for (int k = 0; k < K; k++) {
            states[li * K + k] = si >= 0 ? W[(int64_t) si * K + k] : 0.0;
        }
    }
}

// Item values for outputs [r0, r0 + q.R) of the values table (U x R_total:
// item i's states at rows 2i and 2i + 1), one warp per chunk, FP64.
__global__ void __launch_bounds__(256) k_weval_items(TSView ts, QueryParams q, WsDev w,
    const int4 *ids, const double *vals, int32_t R_total, int32_t r0)
{
    const int lane = threadIdx.x & 31;
    const int64_t c = (int64_t) blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= ts.num_chunks) {
        return;
    }
    const double *time = ts.span_time + ts.span_local_off[ts.chunk_span[c]];
    for (int r = 0; r < q.R; r++) {
        double acc = 0;
        for (int64_t i = ts.chunk_begin[c] + lane; i < ts.chunk_end[c]; i += 32) {
            const int4 id = ids[i];
            const double tu = time[id.x];
            const double bl1 = id.z >= 0 ? time[id.z] - tu : 0.0;
            double v = bl1 * vals[(2 * i + 1) * R_total + r0 + r];
            if (id.y >= 0) {
                v -= (time[id.y] - tu) * vals[(2 * i) * R_total + r0 + r];
            }
            acc += v;
        }
        acc = warp_sum(acc);
        if (lane == 0) {
            w.dD[c * q.R + r] = acc;
        }
    }
}

// Per site: the sum of its alleles' values (the ancestral one skipped when
// polarised), term-major.
__global__ void k_wsite_values(TSView ts, QueryParams q, WsDev w, const int64_t *site_off,
    const double *vals, int64_t sbase, int32_t R_total, int32_t r0)
{
    for (int64_t site = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; site < ts.num_sites;
         site += (int64_t) gridDim.x * blockDim.x) {
        const int64_t a0 = q.polarised ? 1 : 0, A = site_off[site + 1] - site_off[site];
        for (int r = 0; r < q.R; r++) {
            double v = 0;
            for (int64_t a = a0; a < A; a++) {
                v += vals[(sbase + site_off[site] + a) * R_total + r0 + r];
            }
            w.site_val[(int64_t) r * ts.num_sites + site] = v;
        }
    }
}

// Leaf branches: per window and term, the exact sum over leaf edges of
// F_r(leaf weights) x branch length x overlap, in signed fixed point
// (positive and negative parts): partial windows get their overlap, the
// windows in between a difference array (as k_leaf_areas).  Layout of acc:
// [sign][partial, plus, minus][window][term][limbs].
__global__ void __launch_bounds__(256) k_wleaf_areas(TSView ts, QueryParams q, QueryDev qd,
    const double *vals, int64_t lbase, int32_t R_total, int32_t r0, unsigned long long *acc,
    int32_t *err)
{
    const int R = q.R;
    const int64_t block = (int64_t) q.Wn * R * TSG_FX_LIMBS;
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < ts.num_edges;
         i += (int64_t) gridDim.x * blockDim.x) {
        const int32_t c = ts.ins_child[i];
        if (ts.node_is_parent[c]) {
            continue;
        }
        const double bl = ts.node_time[ts.ins_parent[i]] - ts.node_time[c];
        const double left = ts.ins_left[i], right = ts.ins_right[i];
        int w0 = (int) upper_bound(qd.windows, (int64_t) q.Wn + 1, left) - 1;
        int w1 = (int) lower_bound(qd.windows, (int64_t) q.Wn + 1, right) - 1;
        w0 = w0 < 0 ? 0 : (w0 >= q.Wn ? q.Wn - 1 : w0);
        w1 = w1 < w0 ? w0 : (w1 >= q.Wn ? q.Wn - 1 : w1);
        const int64_t li = ts.leaf_index[c];
        for (int r = 0; r < R; r++) {
            const double f = vals[(lbase + li) * R_total + r0 + r] * bl;
            unsigned long long *base = acc + (f < 0 ? 3 * block : 0);
            const double af = f < 0 ? -f : f;
            auto at = [&](int kind, int wi) {
                return base + kind * block + ((int64_t) wi * R + r) * TSG_FX_LIMBS;
            };
            if (w0 == w1) {
                fx_add(at(0, w0), af * (right - left), err);
                continue;
            }
            fx_add(at(0, w0), af * (qd.windows[w0 + 1] - left), err);
            fx_add(at(0, w1), af * (right - qd.windows[w1]), err);
            if (w1 > w0 + 1) {
                fx_add(at(1, w0 + 1), af, err);
                fx_add(at(2, w1), af, err);
            }
        }
    }
}

// One block per term: the running sum over windows of the difference arrays
// (exact per window, then a fixed-order FP64 prefix) times the window
// length, plus the partial windows, into w.leaf_win.
__global__ void __launch_bounds__(256) k_wleaf_prefix(QueryParams q, QueryDev qd, WsDev w,
    const unsigned long long *acc)
{
    __shared__ double s_run[256];
    const int R = q.R, r = blockIdx.x;
    const int64_t block = (int64_t) q.Wn * R * TSG_FX_LIMBS;
    auto at = [&](int sign, int kind, int wi) {
        return acc + sign * 3 * block + kind * block + ((int64_t) wi * R + r) * TSG_FX_LIMBS;
    };
    auto delta = [&](int wi) {
        return fx_diff_value(at(0, 1, wi), at(0, 2, wi)) - fx_diff_value(at(1, 1, wi), at(1, 2, wi));
    };
    const int per = (q.Wn + blockDim.x - 1) / blockDim.x;
    const int w0 = threadIdx.x * per, w1 = min(q.Wn, w0 + per);
    double run = 0;
    for (int wi = w0; wi < w1; wi++) {
        run += delta(wi);
    }
    s_run[threadIdx.x] = run;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0;
        for (int j = 0; j < (int) blockDim.x; j++) {
            const double v = s_run[j];
            s_run[j] = a;
            a += v;
        }
    }
    __syncthreads();
    double active = s_run[threadIdx.x];
    for (int wi = w0; wi < w1; wi++) {
        active += delta(wi);
        w.leaf_win[(int64_t) wi * R + r] = active * (qd.windows[wi + 1] - qd.windows[wi])
            + fx_value(at(0, 0, wi)) - fx_value(at(1, 0, wi));
    }
}

int genw_replay(const TSView &v, const QueryParams &q, const double *W, bool node_w, int K,
    double *slots_x, int32_t *slots_par, uint8_t *slots_touched, int grid, int4 *ids, double *xs,
    double *mstate, double *init, int32_t *err, int32_t *counter, cudaStream_t st)
{
    k_wreplay<<<(unsigned) grid, 64, 0, st>>>(v, q, W, node_w ? 1 : 0, K, slots_x, slots_par,
        slots_touched, ids, xs, mstate, init, err, counter);
    TSG_LAUNCHED();
    return 0;
}

int genw_states(const TSView &v, int K, const double *W, const double *total,
    const double *mstate, const int64_t *site_off, double *site_states, double *leaf_states,
    cudaStream_t st)
{
    if (v.num_sites > 0 && site_states != nullptr) {
        k_wsite_states<<<gen_grid(v.num_sites), 256, 0, st>>>(v, K, total, mstate, site_off,
            site_states);
        TSG_LAUNCHED();
    }
    if (v.num_leaves > 0 && leaf_states != nullptr) {
        k_wleaf_states<<<gen_grid(v.num_leaves), 256, 0, st>>>(v, K, W, leaf_states);
        TSG_LAUNCHED();
    }
    return 0;
}

int genw_eval(const TSView &v, const QueryParams &q, const QueryDev &d, const WsDev &w,
    const int4 *ids, const double *vals, const int64_t *site_off, int64_t sbase, int64_t lbase,
    unsigned long long *leaf_acc, int32_t R_total, int32_t r0, cudaStream_t st)
{
    if (q.branch) {
        k_weval_items<<<(unsigned) ((v.num_chunks + 7) / 8), 256, 0, st>>>(v, q, w, ids, vals,
            R_total, r0);
        TSG_LAUNCHED();
        TSG_CUDA(cudaMemsetAsync(leaf_acc, 0,
            (size_t) q.Wn * q.R * TSG_FX_LIMBS * 8 * 6, st));
        if (v.num_edges > 0 && v.num_leaves > 0) {
            k_wleaf_areas<<<gen_grid(v.num_edges), 256, 0, st>>>(v, q, d, vals, lbase, R_total,
                r0, leaf_acc, w.err);
            TSG_LAUNCHED();
        }
        k_wleaf_prefix<<<(unsigned) q.R, 256, 0, st>>>(q, d, w, leaf_acc);
        TSG_LAUNCHED();
    }
    if (q.site && v.num_sites > 0) {
        k_wsite_values<<<gen_grid(v.num_sites), 256, 0, st>>>(v, q, w, site_off, vals, sbase,
            R_total, r0);
        TSG_LAUNCHED();
    }
    return 0;
}

// genetic_relatedness_weighted's summary (c/tskit/trees.c:4801-4837) at
// every listed state: the weights carry a last column of 1/n; for pair k =
// (i, j), (x_i - n_i p)(x_j - n_j p) with p the last component (centred) or
// x_i x_j, plus the same at total - x when unpolarised branch.
__global__ void k_wsummary_relatedness(const double *states, int64_t U, int K1,
    const double *total, const int32_t *tuples, int R, double ones, int centred,
    int complement, double *vals)
{
    for (int64_t u = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; u < U;
         u += (int64_t) gridDim.x * blockDim.x) {
        const double *x = states + u * K1;
        for (int k = 0; k < R; k++) {
            const int i = tuples[2 * k], j = tuples[2 * k + 1];
            double v;
            if (centred) {
                const double p = x[K1 - 1];
                v = (x[i] - total[i] * p) * (x[j] - total[j] * p);
                if (complement) {
                    const double pc = ones - p;
                    v += ((total[i] - x[i]) - total[i] * pc) * ((total[j] - x[j]) - total[j] * pc);
                }
            } else {
                v = x[i] * x[j];
                if (complement) {
                    v += (total[i] - x[i]) * (total[j] - x[j]);
                }
            }
            vals[u * R + k] = v;
        }
    }
}

// The trait statistics' summaries (c/tskit/trees.c:3961-3974 covariance,
// 4026-4044 correlation, 4108-4152 linear model) at every listed state,
// plus the complement (total - x) when unpolarised.  kind 0: covariance, K
// columns; 1: correlation, K - 1 traits and the frequency last; 2: linear
// model, R traits, K - R - 1 covariates, the sample count last, V the
// traits' projections on the covariates (R x (K - R - 1)).
__device__ double trait_summary(int kind, const double *x, int K, int R, int r, double n,
    const double *V)
{
    switch (kind) {
        case 0:
            return (x[r] * x[r]) / (2 * (n - 1) * (n - 1));
        case 1: {
            const double p = x[K - 1];
            if ((p > 0.0) && (p < 1.0)) {
                return (x[r] * x[r]) / (2 * (p * (1 - p)) * n * (n - 1));
            }
            return 0.0;
        }
        default: {
            const double m = x[K - 1];
            const int nc = K - R - 1;
            if (!((m > 0.0) && (m < n))) {
                return 0.0;
            }
            double a = x[r], denom = m;
            for (int j = 0; j < nc; j++) {
                const double z = x[R + j];
                a -= z * V[(int64_t) r * nc + j];
                denom -= z * z;
            }
            // the reference's tolerance for a trait in the covariates' span
            if (denom < 1e-8) {
                return 0.0;
            }
            return (a * a) / (2 * denom * denom);
        }
    }
}

__global__ void k_wsummary_trait(const double *states, int64_t U, int K, int R, int kind,
    double n, const double *V, const double *total, int complement, double *vals)
{
    double c[TSG_MAX_SAMPLE_SETS];
    for (int64_t u = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; u < U;
         u += (int64_t) gridDim.x * blockDim.x) {
        const double *x = states + u * K;
        if (complement) {
            for (int k = 0; k < K && k < TSG_MAX_SAMPLE_SETS; k++) {
                c[k] = total[k] - x[k];
            }
        }
        for (int r = 0; r < R; r++) {
            double v = trait_summary(kind, x, K, R, r, n, V);
            if (complement) {
                v += trait_summary(kind, c, K, R, r, n, V);
            }
            vals[u * R + r] = v;
        }
    }
}

int genw_summary_trait(const double *states, int64_t U, int K, int R, int kind, double n,
    const double *V, const double *total, bool complement, double *vals, cudaStream_t st)
{
    if (U == 0) {
        return 0;
    }
    k_wsummary_trait<<<gen_grid(U), 256, 0, st>>>(states, U, K, R, kind, n, V, total,
        complement ? 1 : 0, vals);
    TSG_LAUNCHED();
    return 0;
}

// mean_descendants (c/tskit/trees.c:1076-1220): per state, the counts of
// the K - 1 reference sets and whether the union count is positive; the
// node walk integrates them into each node's spans, divided on the host.
__global__ void k_wsummary_descendants(const double *states, int64_t U, int K, double *vals)
{
    for (int64_t u = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; u < U;
         u += (int64_t) gridDim.x * blockDim.x) {
        const double *x = states + u * K;
        const double any = x[K - 1] > 0 ? 1.0 : 0.0;
        for (int k = 0; k < K - 1; k++) {
            vals[u * K + k] = any * x[k];
        }
        vals[u * K + K - 1] = any;
    }
}

int genw_summary_descendants(const double *states, int64_t U, int K, double *vals,
    cudaStream_t st)
{
    if (U == 0) {
        return 0;
    }
    k_wsummary_descendants<<<gen_grid(U), 256, 0, st>>>(states, U, K, vals);
    TSG_LAUNCHED();
    return 0;
}

int genw_summary_relatedness(const double *states, int64_t U, int K1, const double *total,
    const int32_t *tuples, int R, double ones, bool centred, bool complement, double *vals,
    cudaStream_t st)
{
    if (U == 0) {
        return 0;
    }
    k_wsummary_relatedness<<<gen_grid(U), 256, 0, st>>>(states, U, K1, total, tuples, R, ones,
        centred ? 1 : 0, complement ? 1 : 0, vals);
    TSG_LAUNCHED();
    return 0;
}

// ---------------------------------------------------------------------------
// Node mode (tsk_treeseq_node_general_stat, c/tskit/trees.c:1788-1918): per
// node and window, the integral along the genome of f at the node's state.
// A node's state is piecewise constant and changes only where the replay
// touches it, so the replay's items (node, tree, state after) sorted by
// (node, tree), with each node's state at the start of the sequence, give
// every node's intervals: one thread per node and output walks them in
// genome order, adding (end - start) x f(state) per interval and window in
// the order the reference's sweep adds them.

// every node's own weight (by sample index, or by node id with node_w),
// before the first tree's state is written over it by the replay
__global__ void k_node_init(TSView ts, int K, const double *W, int node_w, double *init)
{
    for (int64_t g = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; g < ts.num_nodes;
         g += (int64_t) gridDim.x * blockDim.x) {
        const int32_t si = ts.sample_index[g];
        for (int k = 0; k < K; k++) {
            init[g * K + k] = node_w ? W[g * K + k] : si >= 0 ? W[(int64_t) si * K + k] : 0.0;
        }
    }
}

// sort keys (global node << 32 | tree) of the items, one warp per chunk
// (an item whose node is out of range is flagged and sorts last, outside
// every node's range)
__global__ void __launch_bounds__(256) k_node_keys(TSView ts, const int4 *ids, uint64_t *keys,
    int32_t *idx, int32_t *err)
{
    const int lane = threadIdx.x & 31;
    const int64_t c = (int64_t) blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= ts.num_chunks) {
        return;
    }
    const int32_t s = ts.chunk_span[c], t = ts.chunk_tree[c];
    const int64_t lo = ts.span_local_off[s];
    const int64_t Ls = ts.span_local_off[s + 1] - lo;
    const int32_t *l2g = ts.span_l2g + lo;
    for (int64_t i = ts.chunk_begin[c] + lane; i < ts.chunk_end[c] && i < ts.num_items; i += 32) {
        const int32_t u = ids[i].x;
        const int32_t g = u >= 0 && u < Ls ? l2g[u] : -1;
        idx[i] = (int32_t) i;
        if (g < 0 || g >= ts.num_nodes) {
            dev_error(err, DEV_ITEM_PLAN);
            keys[i] = ~0ull;
            continue;
        }
        keys[i] = ((uint64_t) (uint32_t) g << 32) | (uint32_t) t;
    }
}

// the state list: each item's state after its transition, then each node's
// state at the start of the sequence
__global__ void k_node_states(int64_t I, int64_t N, int K, const double *xs, const double *init,
    double *states)
{
    for (int64_t u = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; u < I + N;
         u += (int64_t) gridDim.x * blockDim.x) {
        const double *src = u < I ? xs + (2 * u + 1) * K : init + (u - I) * K;
        for (int k = 0; k < K; k++) {
            states[u * K + k] = src[k];
        }
    }
}

// result [Wn x N x R]; vals: f at state row u (U x R)
__global__ void k_node_walk(TSView ts, int Wn, const double *windows, const uint64_t *keys,
    const int32_t *idx, int64_t I, const double *vals, int R, int span_normalise,
    double *result, int32_t *err)
{
    const int64_t N = ts.num_nodes;
    for (int64_t tid = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; tid < N * R;
         tid += (int64_t) gridDim.x * blockDim.x) {
        const int64_t g = tid / R;
        const int r = (int) (tid - g * R);
        int64_t j = lower_bound(keys, I, (uint64_t) g << 32);
        const int64_t hi = lower_bound(keys, I, (uint64_t) (g + 1) << 32);
        double f = vals[(I + g) * R + r];
        int w = 0;
        double last = windows[0], acc = 0.0;
        auto flush = [&]() {
            const double v = span_normalise ? acc / (windows[w + 1] - windows[w]) : acc;
            result[((int64_t) w * N + g) * R + r] = v;
            acc = 0.0;
            w++;
            last = windows[w];
        };
        for (; j < hi; j++) {
            const uint32_t t = (uint32_t) keys[j];
            const int32_t i = idx[j];
            if (t >= (uint64_t) ts.num_trees || i < 0 || i >= I) {
                dev_error(err, DEV_ITEM_PLAN);
                break;
            }
            // items lie strictly inside the sequence, so before the last
            // window's end
            const double p = ts.breakpoints[t];
            while (w + 1 < Wn && windows[w + 1] <= p) {
                acc += (windows[w + 1] - last) * f;
                flush();
            }
            acc += (p - last) * f;
            last = p;
            f = vals[(int64_t) i * R + r];
        }
        while (w < Wn) {
            acc += (windows[w + 1] - last) * f;
            flush();
        }
    }
}

// f of the built-in summaries at real-valued states (counts as doubles),
// with the summary functions' own divisions (c/tskit/trees.c:3934 diversity,
// 4221 segregating sites, 4248 Y1, 4690 divergence, 4729/4755 relatedness,
// 4899 Y2, 4938 f2, 5177 Y3, 5219 f3, 5266 f4): a node's summary is exactly
// zero wherever the reference's is, e.g. at the root.
__device__ double node_summary(const QueryParams &q, int r, const double *x)
{
    const Term &t = q.term[r];
    const int i = t.idx[0], j = t.idx[1], k = t.idx[2], l = t.idx[3];
    const double xi = x[i], xj = x[j], xk = x[k], xl = x[l];
    const double ni = q.set_size[i], nj = q.set_size[j], nk = q.set_size[k], nl = q.set_size[l];
    switch (t.type) {
        case TSG_DIVERSITY:
            return xi * (ni - xi) / (ni * (ni - 1));
        case TSG_SEGREGATING_SITES:
            return (double) (xi > 0) * (1 - xi / ni);
        case TSG_Y1:
            return xi * (ni - xi) * (ni - xi - 1) / (ni * (ni - 1) * (ni - 2));
        case TSG_DIVERGENCE:
            return xi * (nj - xj) / (ni * (nj - (double) (i == j)));
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
        case TSG_RELATEDNESS: {
            double sumx = 0.0;
            for (int m = 0; m < q.K; m++) {
                sumx += x[m] / q.set_size[m];
            }
            const double meanx = sumx / (double) q.K;
            return (xi / ni - meanx) * (xj / nj - meanx);
        }
        case TSG_RELATEDNESS_NONCENTRED:
            return xi * xj / (ni * nj);
        default:
            return NAN;
    }
}

// plus f at the complement (set sizes - x) when unpolarised
// (c/tskit/trees.c:1944-1972)
__global__ void k_node_term_values(QueryParams q, const double *states, int64_t U, int K,
    int unpol, double *vals)
{
    double c[TSG_MAX_SAMPLE_SETS];
    for (int64_t u = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; u < U;
         u += (int64_t) gridDim.x * blockDim.x) {
        const double *x = states + u * K;
        for (int k = 0; k < K && k < TSG_MAX_SAMPLE_SETS; k++) {
            c[k] = q.set_size[k] - x[k];
        }
        for (int r = 0; r < q.R; r++) {
            double v = node_summary(q, r, x);
            if (unpol) {
                v += node_summary(q, r, c);
            }
            vals[u * q.R + r] = v;
        }
    }
}

int node_init(const TSView &v, int K, const double *W, bool node_w, double *init,
    cudaStream_t st)
{
    if (v.num_nodes > 0) {
        k_node_init<<<gen_grid(v.num_nodes), 256, 0, st>>>(v, K, W, node_w ? 1 : 0, init);
        TSG_LAUNCHED();
    }
    return 0;
}

size_t node_sort_bytes(int64_t I)
{
    size_t temp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, temp, (const uint64_t *) nullptr,
        (uint64_t *) nullptr, (const int32_t *) nullptr, (int32_t *) nullptr,
        (int) std::max<int64_t>(I, 1), 0, 64);
    return temp;
}

// items sorted by (node, tree), and the state list
int node_order(const TSView &v, int K, const int4 *ids, const double *xs, const double *init,
    uint64_t *keys, uint64_t *keys_sorted, int32_t *idx, int32_t *idx_sorted, void *temp,
    size_t temp_bytes, double *states, int32_t *err, cudaStream_t st)
{
    const int64_t I = v.num_items, N = v.num_nodes;
    if (I > 0 && v.num_chunks > 0) {
        k_node_keys<<<(unsigned) ((v.num_chunks + 7) / 8), 256, 0, st>>>(v, ids, keys, idx, err);
        TSG_LAUNCHED();
        int bits = 32;
        while (bits < 64 && ((uint64_t) N >> (bits - 32)) != 0) {
            bits++;
        }
        size_t tb = temp_bytes;
        if (cub::DeviceRadixSort::SortPairs(temp, tb, keys, keys_sorted, idx, idx_sorted, (int) I,
                0, bits, st) != cudaSuccess) {
            return TSG_ERR_CUDA;
        }
        TSG_LAUNCHED();
    }
    if (I + N > 0) {
        k_node_states<<<gen_grid(I + N), 256, 0, st>>>(I, N, K, xs, init, states);
        TSG_LAUNCHED();
    }
    return 0;
}

int node_term_values(const QueryParams &q, const double *states, int64_t U, int K, bool unpol,
    double *vals, cudaStream_t st)
{
    if (U > 0) {
        k_node_term_values<<<gen_grid(U), 256, 0, st>>>(q, states, U, K, unpol ? 1 : 0, vals);
        TSG_LAUNCHED();
    }
    return 0;
}

int node_walk(const TSView &v, int Wn, const double *windows, const uint64_t *keys_sorted,
    const int32_t *idx_sorted, const double *vals, int R, bool span_normalise, double *result,
    int32_t *err, cudaStream_t st)
{
    const int64_t n = v.num_nodes * (int64_t) R;
    if (n > 0) {
        k_node_walk<<<gen_grid(n), 256, 0, st>>>(v, Wn, windows, keys_sorted, idx_sorted,
            v.num_items, vals, R, span_normalise ? 1 : 0, result, err);
        TSG_LAUNCHED();
    }
    return 0;
}

}  // namespace tsg
