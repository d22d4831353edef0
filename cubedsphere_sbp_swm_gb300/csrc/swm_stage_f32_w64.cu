// swm_stage_f32_w64.cu -- the FP32 TMA stage kernel with 64 consumer threads.
#define SWM_STAGE_WIDTH 64
#include "swm_stage_f32_width.cuh"
