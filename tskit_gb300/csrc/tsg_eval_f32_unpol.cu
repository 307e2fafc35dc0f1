// Item evaluation, FP32 per lane, unpolarised.
#define TSG_EVAL_F float
#define TSG_EVAL_UNPOL true
#define TSG_EVAL_NAME launch_eval_f32_unpol
#include "tsg_eval_inst.cuh"
