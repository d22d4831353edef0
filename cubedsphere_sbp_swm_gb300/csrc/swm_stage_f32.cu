// swm_stage_f32.cu -- float instantiation: the TMA-pipelined fused stage
// kernel (swm_stage_tma.cuh) and the cube-edge kernel.
#include "swm_launch.h"
#include "swm_stage_tma.cuh"

namespace swm {

template <>
cudaError_t launch_stage<float>(int order, const StageMaps* maps, const InstDev<float>& one,
                                const InstDev<float>* many, const WorkUnit* units, int nunits,
                                int mode, int boxw, int grid, int* err, cudaStream_t st) {
  static const StageMaps kNone{};
  const StageMaps& m = maps ? *maps : kNone;
  switch (order) {
    case 21: return launch_stage_tma_ord<float, 21>(m, one, many, units, nunits, mode, boxw, grid, err, st);
    case 42: return launch_stage_tma_ord<float, 42>(m, one, many, units, nunits, mode, boxw, grid, err, st);
    case 43: return launch_stage_tma_ord<float, 43>(m, one, many, units, nunits, mode, boxw, grid, err, st);
    case 63: return launch_stage_tma_ord<float, 63>(m, one, many, units, nunits, mode, boxw, grid, err, st);
    default: return cudaErrorInvalidValue;
  }
}

template <>
int stage_occupancy<float>(int order, int boxw) {
  switch (order) {
    case 21: return stage_tma_occupancy<float, 21>(boxw);
    case 42: return stage_tma_occupancy<float, 42>(boxw);
    case 43: return stage_tma_occupancy<float, 43>(boxw);
    default: return stage_tma_occupancy<float, 63>(boxw);
  }
}

template <>
cudaError_t prepare_stage<float>(int order, StageShape* shape) {
  cudaError_t e;
  switch (order) {
    case 21: e = prepare_stage_tma_ord<float, 21>(); break;
    case 42: e = prepare_stage_tma_ord<float, 42>(); break;
    case 43: e = prepare_stage_tma_ord<float, 43>(); break;
    case 63: e = prepare_stage_tma_ord<float, 63>(); break;
    default: return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  shape->cols = TMA_CONS;
  shape->tma = 1;
  shape->boxw = TmaLayout<float, 42>::BOXW_MAX;
  shape->rps = TmaLayout<float, 42>::RPS;
  shape->nf = TmaLayout<float, 42>::NF;
  shape->ctas_per_sm = stage_occupancy<float>(order, shape->boxw);
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
