// swm_launch.h -- host launchers of the fused stage and cube-edge kernels,
// one instantiation per precision (swm_stage_f64.cu / swm_stage_f32.cu).
#pragma once

#include "swm_device.cuh"

namespace swm {

// Fused stage kernel over nunits work units.  maps describes the buffers of
// a one-instance launch to the TMA unit (batched instances carry their own
// maps in InstDev::maps) and boxw is the widest TMA box of the instances
// (TMA kernels only); grid > 0 runs the TMA kernel persistently on that many
// CTAs (0: one CTA per unit); err is the device error flag raised by an
// expired bounded wait.
// cols: the consumer width of the TMA kernel (one of kStageWidths); fixbw:
// the variant whose boxes all have the width's widest box width (boxw must
// then equal stage_boxw_max).
template <class T>
cudaError_t launch_stage(int order, int cols, bool fixbw, const StageMaps* maps, const InstDev<T>& one,
                         const InstDev<T>* many, const WorkUnit* units, int nunits, int mode,
                         int boxw, int grid, int* err, cudaStream_t st);
// Sets the launch attributes of the stage kernels of one SBP order, every
// consumer width (called at context creation, outside any stream capture),
// and returns the default shape.
template <class T>
cudaError_t prepare_stage(int order, StageShape* shape);
// Resident stage-kernel CTAs per SM when the TMA box is boxw columns wide.
template <class T>
int stage_occupancy(int order, int boxw, int cols, bool fixbw);
// Widest TMA box of the kernel of consumer width cols (0: width not built).
template <class T>
int stage_boxw_max(int cols);

// Consumer widths of the FP32 TMA stage kernel; each is instantiated in its
// own translation unit (swm_stage_f32_w<width>.cu).
constexpr int kStageWidths[5] = {64, 96, 128, 160, 192};
template <int CONS>
cudaError_t stage_f32_launch(int order, bool fixbw, const StageMaps& m, const InstDev<float>& one,
                             const InstDev<float>* many, const WorkUnit* units, int nunits,
                             int mode, int boxw, int grid, int* err, cudaStream_t st);
template <int CONS>
int stage_f32_occupancy(int order, bool fixbw, int boxw);
template <int CONS>
cudaError_t stage_f32_prepare(int order);
// Cube-edge kernel over ninst instances whose largest edge has max_n nodes.
template <class T>
cudaError_t launch_edge(const InstDev<T>& one, const InstDev<T>* many, int ninst, int max_n,
                        const Topology& tp, int mode, cudaStream_t st);

}  // namespace swm
