// swm_stage_f32_w128.cu -- the FP32 TMA stage kernel with 128 consumer threads.
#define SWM_STAGE_WIDTH 128
#include "swm_stage_f32_width.cuh"
