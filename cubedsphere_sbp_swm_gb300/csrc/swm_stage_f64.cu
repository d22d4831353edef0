// swm_stage_f64.cu -- double instantiation of the fused stage kernel (plain
// loads; the FP64 path is bound by the GPU's FP64 rate, not by HBM) and the
// cube-edge kernel.
#include "swm_launch.h"
#include "swm_stage.cuh"

namespace swm {

template <>
cudaError_t launch_stage<double>(int order, int cols, bool fixbw, const StageMaps* maps,
                                 const InstDev<double>& one, const InstDev<double>* many,
                                 const WorkUnit* units, int nunits, int mode, int boxw, int grid,
                                 int* err, cudaStream_t st) {
  (void)cols;
  (void)fixbw;
  (void)err;
  (void)grid;
  (void)boxw;
  (void)maps;
  switch (order) {
    case 21: return launch_stage_ord<double, 21>(one, many, units, nunits, mode, st);
    case 42: return launch_stage_ord<double, 42>(one, many, units, nunits, mode, st);
    case 43: return launch_stage_ord<double, 43>(one, many, units, nunits, mode, st);
    case 63: return launch_stage_ord<double, 63>(one, many, units, nunits, mode, st);
    default: return cudaErrorInvalidValue;
  }
}

template <class T, int ORD>
static int v1_occupancy() {
  int blocks = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, stage_kernel<T, ORD>, STAGE_BW,
                                                stage_smem_bytes<T, ORD>());
  return blocks;
}

template <>
cudaError_t prepare_stage<double>(int order, StageShape* shape) {
  cudaError_t e = launch_stage<double>(order, STAGE_BW, false, nullptr, InstDev<double>{}, nullptr, nullptr,
                                       0, MODE_APPLY, 0, 0, nullptr, nullptr);
  int* ctas_per_sm = &shape->ctas_per_sm;
  if (e != cudaSuccess) return e;
  switch (order) {
    case 21: *ctas_per_sm = v1_occupancy<double, 21>(); break;
    case 42: *ctas_per_sm = v1_occupancy<double, 42>(); break;
    case 43: *ctas_per_sm = v1_occupancy<double, 43>(); break;
    default: *ctas_per_sm = v1_occupancy<double, 63>(); break;
  }
  shape->cols = STAGE_BW;
  shape->tma = 0;
  shape->boxw = shape->rps = shape->nf = 0;
  shape->fixbw = 0;
  return cudaGetLastError();
}

template <>
int stage_boxw_max<double>(int cols) {
  (void)cols;
  return 0;
}

template <>
int stage_occupancy<double>(int order, int boxw, int cols, bool fixbw) {
  (void)boxw;
  (void)cols;
  (void)fixbw;
  switch (order) {
    case 21: return v1_occupancy<double, 21>();
    case 42: return v1_occupancy<double, 42>();
    case 43: return v1_occupancy<double, 43>();
    default: return v1_occupancy<double, 63>();
  }
}

template <>
cudaError_t launch_edge<double>(const InstDev<double>& one, const InstDev<double>* many, int ninst,
                                int max_n, const Topology& tp, int mode, cudaStream_t st) {
  const int nodes = 6 * (4 * max_n - 4);
  dim3 grid((nodes + 127) / 128, ninst);
  edge_kernel<double><<<grid, 128, 0, st>>>(one, many, tp, mode);
  return cudaGetLastError();
}

}  // namespace swm
