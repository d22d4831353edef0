// swm_stage_f32_w96.cu -- the FP32 TMA stage kernel with 96 consumer threads.
#define SWM_STAGE_WIDTH 96
#include "swm_stage_f32_width.cuh"
