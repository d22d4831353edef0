// swm_stage_f32_width.cuh -- instantiates the FP32 TMA stage kernel of one
// consumer width (SWM_STAGE_WIDTH, defined by the including translation
// unit) for every SBP order, behind the width-specific launchers declared in
// swm_launch.h.  One translation unit per width keeps the builds parallel.
#pragma once

#include "swm_launch.h"
#include "swm_stage_tma.cuh"

namespace swm {

template <>
cudaError_t stage_f32_launch<SWM_STAGE_WIDTH>(int order, bool fixbw, const StageMaps& m,
                                              const InstDev<float>& one, const InstDev<float>* many,
                                              const WorkUnit* units, int nunits, int mode, int boxw,
                                              int grid, int* err, cudaStream_t st) {
  return StageF32Width<SWM_STAGE_WIDTH>::launch(order, fixbw, m, one, many, units, nunits, mode,
                                                boxw, grid, err, st);
}

template <>
int stage_f32_occupancy<SWM_STAGE_WIDTH>(int order, bool fixbw, int boxw) {
  return StageF32Width<SWM_STAGE_WIDTH>::occupancy(order, fixbw, boxw);
}

template <>
cudaError_t stage_f32_prepare<SWM_STAGE_WIDTH>(int order) {
  return StageF32Width<SWM_STAGE_WIDTH>::prepare(order);
}

}  // namespace swm
