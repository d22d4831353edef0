// swm_stage_f32.cu -- float instantiation: the TMA-pipelined fused stage
// kernel (swm_stage_tma.cuh) and the cube-edge kernel.
#include "swm_launch.h"
#include "swm_stage_tma.cuh"

namespace swm {

constexpr int kNstF32 = 6;  // pipeline depth (rows in flight per CTA)

template <>
cudaError_t launch_stage<float>(int order, const InstDev<float>& one, const InstDev<float>* many,
                                const WorkUnit* units, int nunits, int mode, int* err,
                                cudaStream_t st) {
  switch (order) {
    case 21: return launch_stage_tma_ord<float, 21, kNstF32>(one, many, units, nunits, mode, err, st);
    case 42: return launch_stage_tma_ord<float, 42, kNstF32>(one, many, units, nunits, mode, err, st);
    case 43: return launch_stage_tma_ord<float, 43, kNstF32>(one, many, units, nunits, mode, err, st);
    case 63: return launch_stage_tma_ord<float, 63, kNstF32>(one, many, units, nunits, mode, err, st);
    default: return cudaErrorInvalidValue;
  }
}

template <>
cudaError_t prepare_stage<float>(int order, int* ctas_per_sm, int* cols) {
  cudaError_t e = launch_stage<float>(order, InstDev<float>{}, nullptr, nullptr, 0, MODE_APPLY,
                                      nullptr, nullptr);
  if (e != cudaSuccess) return e;
  switch (order) {
    case 21: *ctas_per_sm = stage_tma_occupancy<float, 21, kNstF32>(); break;
    case 42: *ctas_per_sm = stage_tma_occupancy<float, 42, kNstF32>(); break;
    case 43: *ctas_per_sm = stage_tma_occupancy<float, 43, kNstF32>(); break;
    default: *ctas_per_sm = stage_tma_occupancy<float, 63, kNstF32>(); break;
  }
  *cols = TMA_CONS;
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
