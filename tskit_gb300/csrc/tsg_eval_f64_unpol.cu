// Item replay with evaluation, FP64 per lane, unpolarised.
#define TSG_EVAL_F double
#define TSG_EVAL_UNPOL true
#define TSG_EVAL_NAME launch_replay_eval_f64_unpol
#define TSG_EVAL_FN replay_eval_fn_f64_unpol
#define TSG_CHUNKS_NAME launch_eval_chunks_f64_unpol
#define TSG_CHUNKS_BATCH_NAME launch_eval_chunks_batch_f64_unpol
#include "tsg_eval_inst.cuh"
