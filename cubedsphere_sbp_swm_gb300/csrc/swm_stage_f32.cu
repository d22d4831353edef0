// swm_stage_f32.cu -- float: the dispatch of the TMA-pipelined fused stage
// kernel (swm_stage_tma.cuh) over its consumer widths (instantiated in
// swm_stage_f32_w*.cu) and the cube-edge kernel.
#include "swm_launch.h"
#include "swm_stage_tma.cuh"

namespace swm {

template <>
cudaError_t launch_stage<float>(int order, int cols, bool fixbw, const StageMaps* maps,
                                const InstDev<float>& one, const InstDev<float>* many,
                                const WorkUnit* units, int nunits, int mode, int boxw, int grid,
                                int* err, cudaStream_t st) {
  static const StageMaps kNone{};
  const StageMaps& m = maps ? *maps : kNone;
  switch (cols) {
    case 64: return stage_f32_launch<64>(order, fixbw, m, one, many, units, nunits, mode, boxw, grid, err, st);
    case 96: return stage_f32_launch<96>(order, fixbw, m, one, many, units, nunits, mode, boxw, grid, err, st);
    case 128: return stage_f32_launch<128>(order, fixbw, m, one, many, units, nunits, mode, boxw, grid, err, st);
    case 160: return stage_f32_launch<160>(order, fixbw, m, one, many, units, nunits, mode, boxw, grid, err, st);
    case 192: return stage_f32_launch<192>(order, fixbw, m, one, many, units, nunits, mode, boxw, grid, err, st);
    default: return cudaErrorInvalidValue;
  }
}

template <>
int stage_occupancy<float>(int order, int boxw, int cols, bool fixbw) {
  switch (cols) {
    case 64: return stage_f32_occupancy<64>(order, fixbw, boxw);
    case 96: return stage_f32_occupancy<96>(order, fixbw, boxw);
    case 128: return stage_f32_occupancy<128>(order, fixbw, boxw);
    case 160: return stage_f32_occupancy<160>(order, fixbw, boxw);
    case 192: return stage_f32_occupancy<192>(order, fixbw, boxw);
    default: return 0;
  }
}

template <>
int stage_boxw_max<float>(int cols) {
  switch (cols) {
    case 64: return TmaLayout<float, 42, 64>::BOXW_MAX;
    case 96: return TmaLayout<float, 42, 96>::BOXW_MAX;
    case 128: return TmaLayout<float, 42, 128>::BOXW_MAX;
    case 160: return TmaLayout<float, 42, 160>::BOXW_MAX;
    case 192: return TmaLayout<float, 42, 192>::BOXW_MAX;
    default: return 0;
  }
}

template <>
cudaError_t prepare_stage<float>(int order, StageShape* shape) {
  cudaError_t e = stage_f32_prepare<64>(order);
  if (e == cudaSuccess) e = stage_f32_prepare<96>(order);
  if (e == cudaSuccess) e = stage_f32_prepare<128>(order);
  if (e == cudaSuccess) e = stage_f32_prepare<160>(order);
  if (e == cudaSuccess) e = stage_f32_prepare<192>(order);
  if (e != cudaSuccess) return e;
  shape->cols = TMA_CONS_DEFAULT;
  shape->tma = 1;
  shape->boxw = stage_boxw_max<float>(shape->cols);
  shape->rps = TmaLayout<float, 42, TMA_CONS_DEFAULT>::RPS;
  shape->nf = TmaLayout<float, 42, TMA_CONS_DEFAULT>::NF;
  shape->fixbw = 0;
  shape->ctas_per_sm = stage_occupancy<float>(order, shape->boxw, shape->cols, false);
  return cudaGetLastError();
}

template <>
cudaError_t launch_edge<float>(const InstDev<float>& one, const InstDev<float>* many, int ninst,
                               int max_n, const Topology& tp, int mode, cudaStream_t st) {
  const int nodes = 6 * (4 * max_n - 4);
  dim3 grid((nodes + 127) / 128, ninst);
  edge_kernel<float><<<grid, 128, 0, st>>>(one, many, tp, mode);
  return cudaGetLastError();
}

}  // namespace swm
