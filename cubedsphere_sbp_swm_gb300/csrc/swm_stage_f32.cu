// swm_stage_f32.cu -- float instantiation: the TMA-pipelined fused stage
// kernel (swm_stage_tma.cuh) and the cube-edge kernel.
#include "swm_launch.h"
#include "swm_stage_tma.cuh"

namespace swm {

constexpr int kRpsF32 = 2;  // rows per pipeline stage
constexpr int kNstF32 = 3;  // pipeline stages

template <>
cudaError_t launch_stage<float>(int order, const StageMaps* maps, const InstDev<float>& one,
                                const InstDev<float>* many, const WorkUnit* units, int nunits,
                                int mode, int* err, cudaStream_t st) {
  static const StageMaps kNone{};
  const StageMaps& m = maps ? *maps : kNone;
  switch (order) {
    case 21: return launch_stage_tma_ord<float, 21, kRpsF32, kNstF32>(m, one, many, units, nunits, mode, err, st);
    case 42: return launch_stage_tma_ord<float, 42, kRpsF32, kNstF32>(m, one, many, units, nunits, mode, err, st);
    case 43: return launch_stage_tma_ord<float, 43, kRpsF32, kNstF32>(m, one, many, units, nunits, mode, err, st);
    case 63: return launch_stage_tma_ord<float, 63, kRpsF32, kNstF32>(m, one, many, units, nunits, mode, err, st);
    default: return cudaErrorInvalidValue;
  }
}

template <>
cudaError_t prepare_stage<float>(int order, StageShape* shape) {
  cudaError_t e = launch_stage<float>(order, nullptr, InstDev<float>{}, nullptr, nullptr, 0,
                                      MODE_APPLY, nullptr, nullptr);
  if (e != cudaSuccess) return e;
  switch (order) {
    case 21: shape->ctas_per_sm = stage_tma_occupancy<float, 21, kRpsF32, kNstF32>(); break;
    case 42: shape->ctas_per_sm = stage_tma_occupancy<float, 42, kRpsF32, kNstF32>(); break;
    case 43: shape->ctas_per_sm = stage_tma_occupancy<float, 43, kRpsF32, kNstF32>(); break;
    default: shape->ctas_per_sm = stage_tma_occupancy<float, 63, kRpsF32, kNstF32>(); break;
  }
  shape->cols = TMA_CONS;
  shape->tma = 1;
  shape->boxw = TmaLayout<float, 42, kRpsF32, kNstF32>::BOXW;
  shape->rps = kRpsF32;
  shape->nf = TmaLayout<float, 42, kRpsF32, kNstF32>::NF;
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
