// swm_stage_f32_w192.cu -- the FP32 TMA stage kernel with 192 consumer threads.
#define SWM_STAGE_WIDTH 192
#include "swm_stage_f32_width.cuh"
