// Summary terms on packed counts, and the per-span node state
// (included by tsg_stats.cu after its definitions).
//
// A span's stateful nodes carry: time (f64), per-set sample counts packed as
// W-bit fields in two 64-bit words (W = 16: up to 8 sets, W = 32: up to 4),
// a seek counter word and a parent local id.  The state lives in shared
// memory (W = 16, 16-bit ids) when it fits, else in a per-CTA slice of global
// memory (W = 32, 32-bit ids).  Leaves are never stored: their counts are
// their own sample-set memberships.  Summary terms use precomputed
// reciprocal denominators (no divisions) and read counts with register
// shifts (no indexed arrays).

#pragma once

#include "tsg_query.cuh"

namespace tsg {

#define TSG_KMAX 8

// Counts stay in [0, set size] through every update, so packed adds and
// subtracts never carry between fields.
struct Pack {
    uint64_t lo, hi;
};

template <int W>
__device__ __forceinline__ uint32_t pk_get(const Pack &p, int k)
{
    constexpr int FPW = 64 / W;
    const uint64_t w = k < FPW ? p.lo : p.hi;
    return (uint32_t) ((w >> (W * (k % FPW))) & ((1ull << W) - 1ull));
}

template <int W>
__device__ __forceinline__ void pk_set(Pack &p, int k, uint64_t v)
{
    constexpr int FPW = 64 / W;
    if (k < FPW) {
        p.lo |= v << (W * k);
    } else {
        p.hi |= v << (W * (k - FPW));
    }
}

template <int W>
__device__ __forceinline__ Pack pk_from_mask(uint32_t m, int K)
{
    constexpr int KM = 2 * (64 / W);
    Pack p{0, 0};
#pragma unroll
    for (int k = 0; k < KM; k++) {
        if (k < K && ((m >> k) & 1u)) {
            pk_set<W>(p, k, 1ull);
        }
    }
    return p;
}

// query constants in the evaluation's arithmetic
template <typename F>
__device__ __forceinline__ F q_size(const QueryParams &q, int k);
template <>
__device__ __forceinline__ float q_size<float>(const QueryParams &q, int k) { return q.set_size_f[k]; }
template <>
__device__ __forceinline__ double q_size<double>(const QueryParams &q, int k) { return q.set_size[k]; }
template <typename F>
__device__ __forceinline__ F q_rsize(const QueryParams &q, int k);
template <>
__device__ __forceinline__ float q_rsize<float>(const QueryParams &q, int k) { return q.inv_size_f[k]; }
template <>
__device__ __forceinline__ double q_rsize<double>(const QueryParams &q, int k) { return q.inv_size[k]; }
template <typename F>
__device__ __forceinline__ F q_inv(const QueryParams &q, int r);
template <>
__device__ __forceinline__ float q_inv<float>(const QueryParams &q, int r) { return q.inv_f[r]; }
template <>
__device__ __forceinline__ double q_inv<double>(const QueryParams &q, int r) { return q.inv[r]; }
template <typename F>
__device__ __forceinline__ F q_invK(const QueryParams &q);
template <>
__device__ __forceinline__ float q_invK<float>(const QueryParams &q) { return q.inv_K_f; }
template <>
__device__ __forceinline__ double q_invK<double>(const QueryParams &q) { return q.inv_K; }

// A count (below 2^23, which the FP32 form requires of every set size) as
// F: for FP32 by placing it in the significand of 2^23 and subtracting 2^23
// (exact, and on the FP32 pipe).
template <typename F>
__device__ __forceinline__ F cnt_to(uint32_t v);
template <>
__device__ __forceinline__ float cnt_to<float>(uint32_t v)
{
    return __int_as_float((int) (0x4B000000u | v)) - 8388608.0f;
}
template <>
__device__ __forceinline__ double cnt_to<double>(uint32_t v)
{
    return (double) v;
}

template <typename F>
__device__ __forceinline__ F term_inv(int type, F xi, F xj, F xk, F xl, F ni, F nj, F nk, F nl,
    F inv, F ri, F rj, F meanx)
{
    switch (type) {
        case TSG_DIVERSITY:
            return xi * (ni - xi) * inv;
        case TSG_SEGREGATING_SITES:
            return (F) (xi > 0) * (1 - xi * inv);
        case TSG_Y1:
            return xi * (ni - xi) * (ni - xi - 1) * inv;
        case TSG_DIVERGENCE:
            return xi * (nj - xj) * inv;
        case TSG_Y2:
            return xi * (nj - xj) * (nj - xj - 1) * inv;
        case TSG_F2:
            return (xi * (xi - 1) * (nj - xj) * (nj - xj - 1) - xi * (ni - xi) * (nj - xj) * xj)
                * inv;
        case TSG_Y3:
            return xi * (nj - xj) * (nk - xk) * inv;
        case TSG_F3:
            return (xi * (xi - 1) * (nj - xj) * (nk - xk) - xi * (ni - xi) * (nj - xj) * xk) * inv;
        case TSG_F4:
            return (xi * xk * (nj - xj) * (nl - xl) - xi * xl * (nj - xj) * (nk - xk)) * inv;
        case TSG_RELATEDNESS:
            return (xi * ri - meanx) * (xj * rj - meanx);
        case TSG_RELATEDNESS_NONCENTRED:
            return xi * xj * inv;
        default:
            return (F) NAN;
    }
}

// The term's value as an exact integer numerator over its denominator (the
// value is num * inv): every summary function but the centred relatedness is
// an integer polynomial in the counts and set sizes over a fixed product of
// set sizes.  With every set size below 2^15 the products stay below 2^61.
// Returns false for the centred relatedness.
__device__ __forceinline__ bool term_num(int type, int64_t xi, int64_t xj, int64_t xk,
    int64_t xl, int64_t ni, int64_t nj, int64_t nk, int64_t nl, int64_t &num)
{
    switch (type) {
        case TSG_DIVERSITY:
            num = xi * (ni - xi);
            return true;
        case TSG_SEGREGATING_SITES:
            num = xi > 0 ? ni - xi : 0;
            return true;
        case TSG_Y1:
            num = xi * (ni - xi) * (ni - xi - 1);
            return true;
        case TSG_DIVERGENCE:
            num = xi * (nj - xj);
            return true;
        case TSG_Y2:
            num = xi * (nj - xj) * (nj - xj - 1);
            return true;
        case TSG_F2:
            num = xi * (xi - 1) * (nj - xj) * (nj - xj - 1) - xi * (ni - xi) * (nj - xj) * xj;
            return true;
        case TSG_Y3:
            num = xi * (nj - xj) * (nk - xk);
            return true;
        case TSG_F3:
            num = xi * (xi - 1) * (nj - xj) * (nk - xk) - xi * (ni - xi) * (nj - xj) * xk;
            return true;
        case TSG_F4:
            num = xi * xk * (nj - xj) * (nl - xl) - xi * xl * (nj - xj) * (nk - xk);
            return true;
        case TSG_RELATEDNESS_NONCENTRED:
            num = xi * xj;
            return true;
        default:
            num = 0;
            return false;
    }
}

// Means over the sets of x_k / n_k and of (n_k - x_k) / n_k (centred
// relatedness only).
template <typename F, int W>
__device__ __forceinline__ void pk_means(const QueryParams &q, const Pack &P, F &mx, F &mc)
{
    constexpr int KM = 2 * (64 / W);
    mx = 0;
    mc = 0;
    if (q.need_mean) {
#pragma unroll
        for (int k = 0; k < KM; k++) {
            if (k < q.K) {
                const F x = cnt_to<F>(pk_get<W>(P, k)), n = q_size<F>(q, k), r = q_rsize<F>(q, k);
                mx += x * r;
                mc += (n - x) * r;
            }
        }
        mx *= q_invK<F>(q);
        mc *= q_invK<F>(q);
    }
}

// F_r(x): f_r(x), plus f_r(n - x) when unpolarised (c/tskit/trees.c:1944-1972).
template <typename F, bool UNPOL, int W>
__device__ __forceinline__ F term_F(const QueryParams &q, int r, const Pack &P, F mx, F mc)
{
    const Term &t = q.term[r];
    const F ni = q_size<F>(q, t.idx[0]), nj = q_size<F>(q, t.idx[1]);
    const F nk = q_size<F>(q, t.idx[2]), nl = q_size<F>(q, t.idx[3]);
    const F ri = q_rsize<F>(q, t.idx[0]), rj = q_rsize<F>(q, t.idx[1]);
    const F xi = cnt_to<F>(pk_get<W>(P, t.idx[0])), xj = cnt_to<F>(pk_get<W>(P, t.idx[1]));
    const F xk = cnt_to<F>(pk_get<W>(P, t.idx[2])), xl = cnt_to<F>(pk_get<W>(P, t.idx[3]));
    const F inv = q_inv<F>(q, r);
    F v = term_inv<F>(t.type, xi, xj, xk, xl, ni, nj, nk, nl, inv, ri, rj, mx);
    if (UNPOL) {
        v += term_inv<F>(t.type, ni - xi, nj - xj, nk - xk, nl - xl, ni, nj, nk, nl, inv, ri, rj, mc);
    }
    return v;
}

// Node state of one span.  IdxT: 16-bit ids in shared memory, 32-bit ids in
// global memory; the all-ones id means "no parent".  Counts and parents live
// in the span's state area; node times come from the span plan (read-only,
// global) and the seek counters from per-CTA global scratch.
template <typename IdxT>
struct SpanState {
    const double *time;  // span-local node times
    uint64_t *xq;        // KQ words per node
    uint32_t *cnt;       // seek counters: children (low 16 bits), arrivals (high 16 bits)
    IdxT *par;
    int KQ;
    static constexpr uint32_t NONE = (uint32_t) (IdxT) ~(IdxT) 0;
};

template <typename IdxT>
__device__ __forceinline__ Pack pk_load(const SpanState<IdxT> &sp, int64_t l)
{
    Pack p;
    p.lo = sp.xq[l * sp.KQ];
    p.hi = sp.KQ > 1 ? sp.xq[l * sp.KQ + 1] : 0ull;
    return p;
}

template <typename IdxT>
__device__ __forceinline__ void pk_store(const SpanState<IdxT> &sp, int64_t l, const Pack &p)
{
    sp.xq[l * sp.KQ] = p.lo;
    if (sp.KQ > 1) {
        sp.xq[l * sp.KQ + 1] = p.hi;
    }
}

// counts of an encoded node (local stateful id >= 0, or -(global + 1))
template <int W, typename IdxT>
__device__ __forceinline__ Pack load_counts(const SpanState<IdxT> &sp, const QueryDev &qd,
    int32_t enc, int K)
{
    if (enc >= 0) {
        return pk_load(sp, enc);
    }
    return pk_from_mask<W>(qd.node_mask[-enc - 1], K);
}

}  // namespace tsg
