// One arithmetic x polarisation of the item evaluation: the instantiations
// of k_eval_items for every count form and the launcher that picks one.
// Included by a translation unit that defines TSG_EVAL_F (float or double),
// TSG_EVAL_UNPOL (true or false) and TSG_EVAL_NAME (the launcher's name), so
// that the instantiations compile in parallel.
#include "tsg_eval.cuh"

namespace tsg {

void TSG_EVAL_NAME(int form, unsigned grid, cudaStream_t st, const TSView &v,
    const QueryParams &p, const WsDev &w)
{
    switch (form) {
        case 0:
            k_eval_items<TSG_EVAL_F, TSG_EVAL_UNPOL, TSG_ITEM_RMAX, 16, 1><<<grid, 256, 0, st>>>(v, p, w);
            break;
        case 1:
            k_eval_items<TSG_EVAL_F, TSG_EVAL_UNPOL, TSG_ITEM_RMAX, 16, 2><<<grid, 256, 0, st>>>(v, p, w);
            break;
        case 2:
            k_eval_items<TSG_EVAL_F, TSG_EVAL_UNPOL, TSG_ITEM_RMAX, 32, 1><<<grid, 256, 0, st>>>(v, p, w);
            break;
        default:
            k_eval_items<TSG_EVAL_F, TSG_EVAL_UNPOL, TSG_ITEM_RMAX, 32, 2><<<grid, 256, 0, st>>>(v, p, w);
            break;
    }
}

}  // namespace tsg
