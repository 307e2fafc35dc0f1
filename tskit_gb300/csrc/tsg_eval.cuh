// Item evaluation of the item pipeline (run by the replay kernel's
// evaluating warps, instantiated per arithmetic in its own translation unit).
#pragma once

#include "tsg_replay.cuh"

namespace tsg {


// FP32 compensated accumulation.  The item value bl1 * f1 - bl0 * f0 is
// formed without rounding as a sum of FP32 terms -- each product split into
// its rounded value and its exact error by an FMA, their difference by
// Knuth's TwoSum -- and added to a (hi, lo) pair by TwoSum again.  Item
// values along one node's history then telescope to the value at the node's
// current state, so rounding does not build up along the running sum.  The
// __f*_rn intrinsics keep the compiler from contracting the steps into FMAs.
__device__ __forceinline__ void acc2_add(float &hi, float &lo, float bl1, float f1, float bl0,
    float f0)
{
    const float p1 = __fmul_rn(bl1, f1);
    const float e1 = __fmaf_rn(bl1, f1, -p1);
    const float p0 = __fmul_rn(bl0, f0);
    const float e0 = __fmaf_rn(bl0, f0, -p0);
    // s + d == p1 - p0
    const float s = __fsub_rn(p1, p0);
    const float z = __fsub_rn(s, p1);
    const float d = __fadd_rn(__fsub_rn(p1, __fsub_rn(s, z)), __fsub_rn(-p0, z));
    // t + g == hi + s
    const float t = __fadd_rn(hi, s);
    const float y = __fsub_rn(t, hi);
    const float g = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, y)), __fsub_rn(s, y));
    hi = t;
    lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(g, d), __fsub_rn(e1, e0)));
}

// The summary term at counts x as an exact integer numerator (its value is
// the numerator times q.inv[r]): every summary function but the centred
// relatedness is an integer polynomial in the counts and set sizes.  With
// every set size below 2^15 each factor pair fits 32 bits and each product
// needs at most one 32 x 32 -> 64-bit multiply.
__device__ __forceinline__ int64_t term_num32(int type, int32_t xi, int32_t xj, int32_t xk,
    int32_t xl, int32_t ni, int32_t nj, int32_t nk, int32_t nl)
{
    const int32_t ci = ni - xi, cj = nj - xj, ck = nk - xk, cl = nl - xl;
    switch (type) {
        case TSG_DIVERSITY:
            return (int64_t) (xi * ci);
        case TSG_SEGREGATING_SITES:
            return xi > 0 ? (int64_t) ci : 0;
        case TSG_Y1:
            return (int64_t) (xi * ci) * (int64_t) (ci - 1);
        case TSG_DIVERGENCE:
            return (int64_t) (xi * cj);
        case TSG_Y2:
            return (int64_t) xi * (int64_t) (cj * (cj - 1));
        case TSG_F2:
            return (int64_t) (xi * (xi - 1)) * (int64_t) (cj * (cj - 1))
                - (int64_t) (xi * ci) * (int64_t) (cj * xj);
        case TSG_Y3:
            return (int64_t) (xi * cj) * (int64_t) ck;
        case TSG_F3:
            return (int64_t) (xi * (xi - 1)) * (int64_t) (cj * ck)
                - (int64_t) (xi * ci) * (int64_t) (cj * xk);
        case TSG_F4:
            return (int64_t) (xi * xk) * (int64_t) (cj * cl)
                - (int64_t) (xi * xl) * (int64_t) (cj * ck);
        case TSG_RELATEDNESS_NONCENTRED:
            return (int64_t) (xi * xj);
        default:
            return 0;
    }
}

// N(x), plus N(n - x) when unpolarised (c/tskit/trees.c:1944-1972)
template <bool UNPOL, int W>
__device__ __forceinline__ int64_t item_num(const Term &t, const int32_t *n, const Pack &x)
{
    const int32_t i = t.idx[0], j = t.idx[1], k = t.idx[2], l = t.idx[3];
    const int32_t xi = (int32_t) pk_get<W>(x, i), xj = (int32_t) pk_get<W>(x, j);
    const int32_t xk = (int32_t) pk_get<W>(x, k), xl = (int32_t) pk_get<W>(x, l);
    int64_t v = term_num32(t.type, xi, xj, xk, xl, n[i], n[j], n[k], n[l]);
    if (UNPOL) {
        v += term_num32(t.type, n[i] - xi, n[j] - xj, n[k] - xk, n[l] - xl, n[i], n[j], n[k],
            n[l]);
    }
    return v;
}

// |v| < 2^53 as a double, exactly, from its bits (integer instructions
// only: GB300 issues FP64 work, conversions included, at a small fraction of
// its integer rate); larger magnitudes go through the rounding converter.
__device__ __forceinline__ double i64_to_f64(int64_t v)
{
    const uint64_t a = v < 0 ? (uint64_t) (-v) : (uint64_t) v;
    if (a == 0) {
        return 0.0;
    }
    if (a >> 53) {
        return (double) v;
    }
    const int e = 63 - __clzll((long long) a);  // the leading one's position, 0..52
    const uint64_t m = (a << (52 - e)) & ((1ull << 52) - 1ull);
    const uint64_t bits = (v < 0 ? (1ull << 63) : 0ull) | ((uint64_t) (e + 1023) << 52) | m;
    return __longlong_as_double((long long) bits);
}

// Value of every item of chunk c for every term, summed over the chunk into
// w.dD (one warp; chunks never cross trees; `time`: the node times of the
// numbering the chunk's items use).  An item is worth
// F(x1) * bl1 - F(x0) * bl0.  Lane r takes term r (at most 32 terms) and
// walks the chunk's items in order, so no sum crosses lanes; a first pass
// (a lane per item) forms the items' branch lengths.  GB300 issues a warp's
// FP64 instruction over 16 cycles, so FP64 work per chunk (sums across
// lanes) and per item is kept to a minimum.
//
// FP64 (every term an integer polynomial over a product of set sizes,
// q.site_int): the value is (bl1 N(x1) - bl0 N(x0)) / D with exact integer
// numerators N, summed as bl * (N(x1) - N(x0)) for a root-path item (same
// branch), (bl1 - bl0) * N(x) for a moved subtree (same counts) or bl1 * N(x)
// where there was no branch before, else both products; the numerators
// become doubles exactly (i64_to_f64) and the chunk's sum is scaled by 1 / D
// once: about one FP64 fused multiply-add per item and warp.
//
// Otherwise (FP64 with the centred relatedness, or FP32): the summary
// functions in F; FP32 forms each item's value exactly from the FP32 values
// and adds it to a compensated pair (acc2_add).
template <typename F, bool UNPOL, int W, int KQ>
__device__ __forceinline__ void eval_chunk(const TSView &ts, const QueryParams &q, const WsDev &w,
    int64_t c, int lane, const double *time)
{
    constexpr bool F32 = sizeof(F) == sizeof(float);
    const int R = q.R;
    const Item<KQ> *items = (const Item<KQ> *) w.items;
    const int64_t b = ts.chunk_begin[c], e = ts.chunk_end[c];
    const bool num_form = !F32 && q.site_int;
    // pass 1, a lane per item: the branch lengths in the evaluation's
    // arithmetic: (bl1, bl0), or in the integer form (bl1 - bl0, bl0) for
    // an item with the same counts before and after
    F *bls = (F *) w.bl;
    for (int64_t i = b + lane; i < e; i += 32) {
        const Item<KQ> it = items[i];
        const double tu = time[it.u];
        const double bl0 = it.p0 >= 0 ? time[it.p0] - tu : 0.0;
        const double bl1 = it.p1 >= 0 ? time[it.p1] - tu : 0.0;
        bool same = it.x0[0] == it.x1[0];
        if (KQ > 1) {
            same = same && it.x0[KQ > 1 ? 1 : 0] == it.x1[KQ > 1 ? 1 : 0];
        }
        bls[2 * i] = (F) (num_form && same ? bl1 - bl0 : bl1);
        bls[2 * i + 1] = (F) bl0;
    }
    __syncwarp();
    // pass 2, a lane per term
    const bool act = lane < R;
    const int r = act ? lane : 0;
    if (num_form) {
        const Term t = q.term[r];
        double acc = 0;
#pragma unroll 4
        for (int64_t i = b; i < e; i++) {
            const Item<KQ> it = items[i];
            const double fa = (double) bls[2 * i], fb = (double) bls[2 * i + 1];
            const Pack x0 = item_pack<KQ>(it.x0);
            const Pack x1 = item_pack<KQ>(it.x1);
            const bool same = x0.lo == x1.lo && x0.hi == x1.hi;
            const int64_t n1 = item_num<UNPOL, W>(t, q.set_size_i, x1);
            const uint64_t ba = (uint64_t) __double_as_longlong(fa);
            const uint64_t bb = (uint64_t) __double_as_longlong(fb);
            if (same || bb == 0) {
                acc = fma(fa, i64_to_f64(n1), acc);
            } else {
                const int64_t n0 = item_num<UNPOL, W>(t, q.set_size_i, x0);
                if (ba == bb) {
                    acc = fma(fa, i64_to_f64(n1 - n0), acc);
                } else {
                    acc = fma(fa, i64_to_f64(n1), fma(-fb, i64_to_f64(n0), acc));
                }
            }
        }
        // a term whose denominator is zero (a set too small for it) is NaN
        // wherever the running sum takes a node's value, as in the reference
        if (act) {
            const double inv = q.inv[r];
            w.dD[c * R + r] = e <= b ? 0.0 : isfinite(inv) ? acc * inv : (double) NAN;
        }
        return;
    }
    F acc = 0, lo = 0;
    for (int64_t i = b; i < e; i++) {
        const Item<KQ> it = items[i];
        const F bl1 = bls[2 * i], bl0 = bls[2 * i + 1];
        const Pack x0 = item_pack<KQ>(it.x0);
        const Pack x1 = item_pack<KQ>(it.x1);
        const bool same = x0.lo == x1.lo && x0.hi == x1.hi;
        F m1x, m1c;
        pk_means<F, W>(q, x1, m1x, m1c);
        const F f1 = term_F<F, UNPOL, W>(q, r, x1, m1x, m1c);
        if (!same && bl0 != 0) {
            F m0x, m0c;
            pk_means<F, W>(q, x0, m0x, m0c);
            const F f0 = term_F<F, UNPOL, W>(q, r, x0, m0x, m0c);
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
    if (act) {
        w.dD[c * R + r] = (double) acc + (double) lo;
    }
}

}  // namespace tsg
