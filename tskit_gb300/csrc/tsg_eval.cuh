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

// Value of every item of chunk c for every term, summed over the chunk into
// w.dD (one warp; chunks never cross trees).  An item is worth
// F(x1) * bl1 - F(x0) * bl0 (F(x0) is not evaluated when there was no branch
// before, nor when the counts did not change).  FP64: evaluated as
// bl * (F(x1) - F(x0)) when the branch length is unchanged (root paths),
// (bl1 - bl0) * F(x) when the counts are unchanged (moved subtrees), else
// directly.  FP32: every item exactly, compensated sums (acc2_add).  Terms go
// in groups of GROUP (accumulators in registers); the chunk's items (at most
// TSG_ITEM_CHUNK / 32 per lane) are re-read from cache for every group.
template <typename F, bool UNPOL, int W, int KQ, int GROUP>
__device__ __forceinline__ void eval_chunk(const TSView &ts, const QueryParams &q, const WsDev &w,
    int64_t c, int lane)
{
    constexpr bool F32 = sizeof(F) == sizeof(float);
    const int R = q.R;
    const Item<KQ> *items = (const Item<KQ> *) w.items;
    const int64_t b = ts.chunk_begin[c], e = ts.chunk_end[c];
    const double *time = ts.span_time + ts.span_local_off[ts.chunk_span[c]];
    // the items' branch lengths, once per chunk into scratch (each lane
    // reads back only its own items)
    F *bls = (F *) w.bl;
    for (int64_t i = b + lane; i < e; i += 32) {
        const int4 up = *(const int4 *) &items[i].u;
        const double tu = time[up.x];
        bls[2 * i] = (F) (up.y >= 0 ? time[up.y] - tu : 0.0);
        bls[2 * i + 1] = (F) (up.z >= 0 ? time[up.z] - tu : 0.0);
    }
    for (int g0 = 0; g0 < R; g0 += GROUP) {
        F acc[GROUP], lo[GROUP];
#pragma unroll
        for (int j = 0; j < GROUP; j++) {
            acc[j] = 0;
            lo[j] = 0;
        }
        for (int64_t i = b + lane; i < e; i += 32) {
            const Item<KQ> it = items[i];
            const F bl0 = bls[2 * i], bl1 = bls[2 * i + 1];
            const Pack x0 = item_pack<KQ>(it.x0);
            const Pack x1 = item_pack<KQ>(it.x1);
            const bool same = x0.lo == x1.lo && x0.hi == x1.hi;
            F m1x, m1c;
            pk_means<F, W>(q, x1, m1x, m1c);
            if (!same && bl0 != 0) {
                F m0x, m0c;
                pk_means<F, W>(q, x0, m0x, m0c);
                const bool path = bl0 == bl1;
#pragma unroll
                for (int j = 0; j < GROUP; j++) {
                    if (g0 + j < R) {
                        const F f1 = term_F<F, UNPOL, W>(q, g0 + j, x1, m1x, m1c);
                        const F f0 = term_F<F, UNPOL, W>(q, g0 + j, x0, m0x, m0c);
                        if constexpr (F32) {
                            acc2_add(acc[j], lo[j], bl1, f1, bl0, f0);
                        } else {
                            acc[j] += path ? bl1 * (f1 - f0) : bl1 * f1 - bl0 * f0;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < GROUP; j++) {
                    if (g0 + j < R) {
                        const F f1 = term_F<F, UNPOL, W>(q, g0 + j, x1, m1x, m1c);
                        if constexpr (F32) {
                            acc2_add(acc[j], lo[j], bl1, f1, bl0, same ? f1 : (F) 0);
                        } else {
                            acc[j] += (same ? bl1 - bl0 : bl1) * f1;
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < GROUP; j++) {
            if (g0 + j < R) {
                const double v = warp_sum((double) acc[j] + (double) lo[j]);
                if (lane == j) {
                    w.dD[c * R + g0 + j] = v;
                }
            }
        }
    }
}

}  // namespace tsg
