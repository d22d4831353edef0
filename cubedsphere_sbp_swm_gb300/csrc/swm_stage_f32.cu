// swm_stage_f32.cu -- float instantiation: the TMA-pipelined fused stage
// kernel (swm_stage_tma.cuh) and the cube-edge kernel.
#include "swm_launch.h"
#include "swm_stage_tma.cuh"

namespace swm {

template <>
cudaError_t launch_stage<float>(int order, const StageMaps* maps, const InstDev<float>& one,
                                const InstDev<float>* many, const WorkUnit* units, int nunits,
                                int mode, int* err, cudaStream_t st) {
  static const StageMaps kNone{};
  const StageMaps& m = maps ? *maps : kNone;
  switch (order) {
    case 21: return launch_stage_tma_ord<float, 21>(m, one, many, units, nunits, mode, err, st);
    case 42: return launch_stage_tma_ord<float, 42>(m, one, many, units, nunits, mode, err, st);
    case 43: return launch_stage_tma_ord<float, 43>(m, one, many, units, nunits, mode, err, st);
    case 63: return launch_stage_tma_ord<float, 63>(m, one, many, units, nunits, mode, err, st);
    default: return cudaErrorInvalidValue;
  }
}

template <>
cudaError_t prepare_stage<float>(int order, StageShape* shape) {
  cudaError_t e;
  switch (order) {
    case 21: e = prepare_stage_tma_ord<float, 21>(&shape->ctas_per_sm); break;
    case 42: e = prepare_stage_tma_ord<float, 42>(&shape->ctas_per_sm); break;
    case 43: e = prepare_stage_tma_ord<float, 43>(&shape->ctas_per_sm); break;
    case 63: e = prepare_stage_tma_ord<float, 63>(&shape->ctas_per_sm); break;
    default: return cudaErrorInvalidValue;
  }
  if (e != cudaSuccess) return e;
  shape->cols = TMA_CONS;
  shape->tma = 1;
  shape->boxw = TmaLayout<float, 42>::BOXW;
  shape->rps = TmaLayout<float, 42>::RPS;
  shape->nf = TmaLayout<float, 42>::NF;
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
