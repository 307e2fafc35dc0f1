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

}  // namespace tsg
