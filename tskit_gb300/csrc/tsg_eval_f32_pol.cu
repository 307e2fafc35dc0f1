// Item replay with evaluation, FP32 per lane, polarised.
#define TSG_EVAL_F float
#define TSG_EVAL_UNPOL false
#define TSG_EVAL_NAME launch_replay_eval_f32_pol
#define TSG_EVAL_FN replay_eval_fn_f32_pol
#define TSG_CHUNKS_NAME launch_eval_chunks_f32_pol
#define TSG_CHUNKS_BATCH_NAME launch_eval_chunks_batch_f32_pol
#include "tsg_eval_inst.cuh"
