// swm_stage_f32.cu -- float instantiation of the fused stage and edge kernels.
#include "swm_launch.h"
#include "swm_stage.cuh"

namespace swm {

template <>
cudaError_t launch_stage<float>(int order, const InstDev<float>& one, const InstDev<float>* many,
                               const WorkUnit* units, int nunits, int mode, cudaStream_t st) {
  switch (order) {
    case 21: return launch_stage_ord<float, 21>(one, many, units, nunits, mode, st);
    case 42: return launch_stage_ord<float, 42>(one, many, units, nunits, mode, st);
    case 43: return launch_stage_ord<float, 43>(one, many, units, nunits, mode, st);
    case 63: return launch_stage_ord<float, 63>(one, many, units, nunits, mode, st);
    default: return cudaErrorInvalidValue;
  }
}

template <>
cudaError_t prepare_stage<float>(int order) {
  // set the dynamic shared-memory opt-in once, outside any stream capture
  return launch_stage<float>(order, InstDev<float>{}, nullptr, nullptr, 0, MODE_APPLY, nullptr) ;
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
