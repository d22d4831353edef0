// swm_stage_f32_w160.cu -- the FP32 TMA stage kernel with 160 consumer threads.
#define SWM_STAGE_WIDTH 160
#include "swm_stage_f32_width.cuh"
