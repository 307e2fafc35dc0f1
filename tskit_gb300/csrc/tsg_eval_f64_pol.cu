// Item replay with evaluation, FP64 per lane, polarised.
#define TSG_EVAL_F double
#define TSG_EVAL_UNPOL false
#define TSG_EVAL_NAME launch_replay_eval_f64_pol
#define TSG_EVAL_FN replay_eval_fn_f64_pol
#define TSG_CHUNKS_NAME launch_eval_chunks_f64_pol
#define TSG_CHUNKS_BATCH_NAME launch_eval_chunks_batch_f64_pol
#include "tsg_eval_inst.cuh"
