// Item evaluation kernel of the item pipeline (instantiated per arithmetic
// in its own translation unit).
#pragma once

#include "tsg_replay.cuh"

namespace tsg {

#define TSG_EVAL_GROUP 8

// Value of every item of a chunk for every term, summed per chunk (one
// warp per chunk; chunks never cross trees).
template <typename F, bool UNPOL, int RMAX, int W, int KQ>
__global__ void __launch_bounds__(256, 3) k_eval_items(TSView ts, QueryParams q, WsDev w)
{
    __shared__ F s_leaf[1 << TSG_LEAF_TABLE_KMAX][RMAX];
    const int lane = threadIdx.x & 31;
    const int R = q.R;
    if (q.K <= TSG_LEAF_TABLE_KMAX) {
        // F of every membership pattern a leaf can have
        const int npat = 1 << q.K;
        for (int i = threadIdx.x; i < npat * R; i += blockDim.x) {
            const int pat = i / R, r = i % R;
            const Pack x = pk_from_mask<W>((uint32_t) pat, q.K);
            F mx, mc;
            pk_means<F, W>(q, x, mx, mc);
            s_leaf[pat][r] = term_F<F, UNPOL, W>(q, r, x, mx, mc);
        }
        __syncthreads();
    }
    const int64_t c = (int64_t) blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= ts.num_chunks) {
        return;
    }
    const Item<KQ> *items = (const Item<KQ> *) w.items;
    const int64_t b = ts.chunk_begin[c], e = ts.chunk_end[c];
    // terms in groups of TSG_EVAL_GROUP (accumulators stay in registers); the
    // chunk's items (at most TSG_ITEM_CHUNK / 32 per lane) are re-read from
    // cache for every group.  Plain sums in F per lane, then FP64.
    for (int g0 = 0; g0 < R; g0 += TSG_EVAL_GROUP) {
        F acc[TSG_EVAL_GROUP];
#pragma unroll
        for (int j = 0; j < TSG_EVAL_GROUP; j++) {
            acc[j] = 0;
        }
        for (int64_t i = b + lane; i < e; i += 32) {
            const Item<KQ> it = items[i];
            const F bl = sizeof(F) == sizeof(float) ? (F) it.blf : (F) it.bl;
            if (it.kind >= TSG_ITEM_LEAF_PLUS) {
                const int pat = (int) it.xn[0];
                const F sb = it.kind == TSG_ITEM_LEAF_PLUS ? bl : -bl;
#pragma unroll
                for (int j = 0; j < TSG_EVAL_GROUP; j++) {
                    if (g0 + j < R) {
                        acc[j] += sb * s_leaf[pat][g0 + j];
                    }
                }
                continue;
            }
            const Pack xn = item_pack<KQ>(it.xn);
            F mxn, mcn;
            pk_means<F, W>(q, xn, mxn, mcn);
            if (it.kind == TSG_ITEM_PATH) {
                const Pack xo = item_pack<KQ>(it.xo);
                F mxo, mco;
                pk_means<F, W>(q, xo, mxo, mco);
#pragma unroll
                for (int j = 0; j < TSG_EVAL_GROUP; j++) {
                    if (g0 + j < R) {
                        acc[j] += bl * (term_F<F, UNPOL, W>(q, g0 + j, xn, mxn, mcn)
                            - term_F<F, UNPOL, W>(q, g0 + j, xo, mxo, mco));
                    }
                }
            } else {
                const F sb = it.kind == TSG_ITEM_PLUS ? bl : -bl;
#pragma unroll
                for (int j = 0; j < TSG_EVAL_GROUP; j++) {
                    if (g0 + j < R) {
                        acc[j] += sb * term_F<F, UNPOL, W>(q, g0 + j, xn, mxn, mcn);
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < TSG_EVAL_GROUP; j++) {
            if (g0 + j < R) {
                const double v = warp_sum((double) acc[j]);
                if (lane == j) {
                    w.dD[c * R + g0 + j] = v;
                }
            }
        }
    }
}

}  // namespace tsg
