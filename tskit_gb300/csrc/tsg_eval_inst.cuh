// One arithmetic x polarisation of the item pipeline: the replay kernel with
// item evaluation for every count form, its launcher and its kernel handle.
// Included by a translation unit that defines TSG_EVAL_F (float or double),
// TSG_EVAL_UNPOL (true or false), TSG_EVAL_NAME (the launcher's name) and
// TSG_EVAL_FN (the handle's name), and TSG_CHUNKS_NAME (the launcher of the
// chunk evaluation after the compact replay), so that the instantiations
// compile in parallel.
#include "tsg_replay_kernel.cuh"

namespace tsg {

TSG_REPLAY_EVAL_FN(TSG_EVAL_FN)
{
    switch (form) {
        case 0: return (void *) k_replay_items<16, 1, uint16_t, TSG_EVAL_F, TSG_EVAL_UNPOL, true>;
        case 1: return (void *) k_replay_items<16, 2, uint16_t, TSG_EVAL_F, TSG_EVAL_UNPOL, true>;
        case 2: return (void *) k_replay_items<32, 1, int32_t, TSG_EVAL_F, TSG_EVAL_UNPOL, true>;
        default: return (void *) k_replay_items<32, 2, int32_t, TSG_EVAL_F, TSG_EVAL_UNPOL, true>;
    }
}

TSG_REPLAY_EVAL_LAUNCHER(TSG_EVAL_NAME)
{
    switch (form) {
        case 0:
            k_replay_items<16, 1, uint16_t, TSG_EVAL_F, TSG_EVAL_UNPOL, true>
                <<<grid, 512, smem, st>>>(v, p, d, w, 0);
            break;
        case 1:
            k_replay_items<16, 2, uint16_t, TSG_EVAL_F, TSG_EVAL_UNPOL, true>
                <<<grid, 512, smem, st>>>(v, p, d, w, 0);
            break;
        case 2:
            k_replay_items<32, 1, int32_t, TSG_EVAL_F, TSG_EVAL_UNPOL, true>
                <<<grid, 512, 0, st>>>(v, p, d, w, slot_bytes);
            break;
        default:
            k_replay_items<32, 2, int32_t, TSG_EVAL_F, TSG_EVAL_UNPOL, true>
                <<<grid, 512, 0, st>>>(v, p, d, w, slot_bytes);
            break;
    }
}

TSG_CHUNK_EVAL_LAUNCHER(TSG_CHUNKS_NAME)
{
    // the replay wrote each item's branch lengths with the item
    const int64_t C = v.num_chunks;
    const int64_t total = (C + TSG_EVAL_BLOCK - 1) / TSG_EVAL_BLOCK * p.gwpb;
    const unsigned ge = (unsigned) std::min<int64_t>((total + 7) / 8, 1 << 20);
    if (kq == 1) {
        k_eval_grouped<TSG_EVAL_F, TSG_EVAL_UNPOL, 1><<<ge, 256, 0, st>>>(v, p, w, total);
    } else {
        k_eval_grouped<TSG_EVAL_F, TSG_EVAL_UNPOL, 2><<<ge, 256, 0, st>>>(v, p, w, total);
    }
}

template <typename F, bool UNPOL, int KQ>
__global__ void __launch_bounds__(256) kb_eval_grouped(const BatchQuery *bq, const int64_t *off,
    int nq)
{
    TSG_BATCH_QUERY();
    const int64_t total = (Q.v.num_chunks + TSG_EVAL_BLOCK - 1) / TSG_EVAL_BLOCK * Q.p.gwpb;
    eval_grouped_body<F, UNPOL, KQ>(Q.v, Q.p, Q.w, total, bid, nb);
}

TSG_CHUNK_EVAL_BATCH_LAUNCHER(TSG_CHUNKS_BATCH_NAME)
{
    if (blocks_eval <= 0) {
        return;
    }
    if (kq == 1) {
        kb_eval_grouped<TSG_EVAL_F, TSG_EVAL_UNPOL, 1><<<(unsigned) blocks_eval, 256, 0, st>>>(
            bq, off_eval, nq);
    } else {
        kb_eval_grouped<TSG_EVAL_F, TSG_EVAL_UNPOL, 2><<<(unsigned) blocks_eval, 256, 0, st>>>(
            bq, off_eval, nq);
    }
}

}  // namespace tsg
