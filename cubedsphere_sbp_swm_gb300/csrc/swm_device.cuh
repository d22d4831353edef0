// swm_device.cuh -- types and tables shared by the CUDA translation units.
//
// Data layout in HBM (one instance = one cubed-sphere state):
//   field  = 6 panels x n rows x P columns of T, n = N+1 nodes per edge,
//            P = n rounded up to a 128-byte multiple (32 floats / 16 doubles),
//            node (p, i, j) at p*n*P + j*P + i; padding columns are zero.
//   state  = 3 consecutive fields (h, u, v), stride fs = 6*n*P.
//   metric = J, Qi1, Qi2, Qi3, f, rJ fields (rJ = 1/(J*hx*a)), FP64-computed.
//   edge   = per panel 4 sides x 4 values (gx, gy, zeta, div) x n, the
//            pre-sync values of every panel-boundary node.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace swm {

// TMA tensor maps of one fused-stage launch.  All are 3-D (column, panel row
// over the 6n rows of all panels, field) over the pitched fields; entries a
// launch does not use hold a copy of a valid map.
struct StageMaps {
  CUtensorMap in;    // stage input state   box {boxw, rps, 3}
  CUtensorMap met;   // metric J, Qi1..3    box {boxw, rps, 4}
  CUtensorMap metf;  // metric f (+rJ)      box {boxw, rps, 1 | 2}
  CUtensorMap base;  // RK base state       box {boxw, rps, 3}
  CUtensorMap acc;   // RK running sum      box {boxw, rps, 3}
  CUtensorMap lo;    // FP32 state low part box {boxw, rps, 3}
  CUtensorMap hs;    // orography           box {boxw, rps, 1}
};

// Launch shape of the fused stage kernel of one precision and SBP order.
struct StageShape {
  int ctas_per_sm;   // resident CTAs per SM
  int cols;          // columns one CTA reads (threads of its consumer warps)
  int tma;           // 1: TMA-pipelined kernel (needs StageMaps)
  int boxw, rps, nf; // TMA box: columns, rows per stage, metric f fields
  int fixbw;         // 1: every box has the width's widest box width
};

constexpr int MAXNE = 6;   // closure rows
constexpr int MAXNW = 9;   // closure width
constexpr int NMETRIC = 6; // J, Qi1, Qi2, Qi3, f, rJ
enum { MJ = 0, MQI1 = 1, MQI2 = 2, MQI3 = 3, MF = 4, MRJ = 5 };
enum { SIDE_L = 0, SIDE_R = 1, SIDE_B = 2, SIDE_T = 3 };
enum { EV_GX = 0, EV_GY = 1, EV_ZETA = 2, EV_DIV = 3 };

// SBP first-derivative operator: left closure block, interior stencil and
// diagonal-norm edge weights (sbp_operators_collection_mod.f90:15-85 in the
// reference; the right block is the sign-flipped mirror, sbp_factory_mod.f90
// :162-165).  Same numbers as the published operators, own layout.
struct SbpC {
  int order, ne, nw, H, rmax, nin, inshift, nA;
  int last[MAXNE];
  double Ql[MAXNE * MAXNW];
  double Qin[7];
  double A[6];
};

// rmax: farthest row any output row reads, = max(H, max_r(last[r]-1-r)).
constexpr double kQ63A1 = 13649.0 / 43200.0, kQ63A2 = 12013.0 / 8640.0,
                 kQ63A3 = 2711.0 / 4320.0, kQ63A4 = 5359.0 / 4320.0,
                 kQ63A5 = 7877.0 / 8640.0, kQ63A6 = 43801.0 / 43200.0;
constexpr double kq56 = 5591070156686698065364559.0 / 7931626489314500743872000.0;
constexpr double kq11 = -1.0 / 2.0;
constexpr double kq12 = -953.0 / 16200.0 + kq56;
constexpr double kq13 = 715489.0 / 259200.0 - (4.0 * kq56);
constexpr double kq14 = -62639.0 / 14400.0 + (6.0 * kq56);
constexpr double kq15 = 147127.0 / 51840.0 - (4.0 * kq56);
constexpr double kq16 = -89387.0 / 129600.0 + kq56;
constexpr double kq23 = -57139.0 / 8640.0 + (10.0 * kq56);
constexpr double kq24 = 745733.0 / 51840.0 - (20.0 * kq56);
constexpr double kq25 = -18343.0 / 1728.0 + (15.0 * kq56);
constexpr double kq26 = 240569.0 / 86400.0 - (4.0 * kq56);
constexpr double kq34 = -176839.0 / 12960.0 + (20.0 * kq56);
constexpr double kq35 = 242111.0 / 17280.0 - (20.0 * kq56);
constexpr double kq36 = -182261.0 / 43200.0 + (6.0 * kq56);
constexpr double kq45 = -165041.0 / 25920.0 + (10.0 * kq56);
constexpr double kq46 = 710473.0 / 259200.0 - (4.0 * kq56);
constexpr double kq47 = 1.0 / 60.0, kq57 = -3.0 / 20.0, kq58 = 1.0 / 60.0;
constexpr double kq67 = 3.0 / 4.0, kq68 = -3.0 / 20.0, kq69 = 1.0 / 60.0;

#define SWM_SBP_TABLES                                                                         \
  {                                                                                            \
    {21, 1, 2, 1, 1, 3, -1, 2, {2, 0, 0, 0, 0, 0},                                             \
     {-1.0, 1.0},                                                                              \
     {-0.5, 0.0, 0.5},                                                                         \
     {0.5, 1.0}},                                                                              \
    {42, 4, 6, 2, 3, 5, -2, 4, {4, 3, 5, 6, 0, 0},                                             \
     {-1.4117647058823528, 1.7352941176470589, -0.2352941176470588, -0.08823529411764705, 0.0, \
      0.0, 0.0, 0.0, 0.0,                                                                      \
      -0.5, 0.0, 0.5, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,                                            \
      0.09302325581395347, -0.686046511627907, 0.0, 0.686046511627907, -0.09302325581395347,   \
      0.0, 0.0, 0.0, 0.0,                                                                      \
      0.030612244897959186, -0.0, -0.6020408163265307, 0.0, 0.653061224489796,                 \
      -0.0816326530612245, 0.0, 0.0, 0.0},                                                     \
     {1.0 / 12.0, -2.0 / 3.0, 0.0, 2.0 / 3.0, -1.0 / 12.0},                                    \
     {17.0 / 48.0, 59.0 / 48.0, 43.0 / 48.0, 49.0 / 48.0}},                                    \
    {43, 4, 6, 2, 5, 5, -2, 4, {6, 6, 6, 6, 0, 0},                                             \
     {-1.8280236842718398, 2.978054584697369, -1.4653148294044123, 0.3078538227474199,         \
      0.008136925288119662, -0.0007068190566565205, 0.0, 0.0, 0.0,                            \
      -0.37814159126691327, -0.31480210500706657, 0.707290999364066, 0.04835554461933453,      \
      -0.06866771096803422, 0.005964863258613564, 0.0, 0.0, 0.0,                               \
      0.1162478575921292, -0.8028500807354999, 0.21558841368737428, 0.5078566674295846,        \
      -0.03231754093993847, -0.004525317033649745, 0.0, 0.0, 0.0,                              \
      -0.010287398573128293, 0.12592344801071614, -0.7341531396449149, 0.04979271660173103,    \
      0.6506171865540596, -0.08189281294846368, 0.0, 0.0, 0.0},                                \
     {1.0 / 12.0, -2.0 / 3.0, 0.0, 2.0 / 3.0, -1.0 / 12.0},                                    \
     {17.0 / 48.0, 59.0 / 48.0, 43.0 / 48.0, 49.0 / 48.0}},                                    \
    {63, 6, 9, 3, 5, 7, -3, 6, {6, 6, 6, 7, 8, 9},                                             \
     {kq11 / kQ63A1, kq12 / kQ63A1, kq13 / kQ63A1, kq14 / kQ63A1, kq15 / kQ63A1,               \
      kq16 / kQ63A1, 0.0, 0.0, 0.0,                                                            \
      -kq12 / kQ63A2, 0.0, kq23 / kQ63A2, kq24 / kQ63A2, kq25 / kQ63A2, kq26 / kQ63A2, 0.0,    \
      0.0, 0.0,                                                                                \
      -kq13 / kQ63A3, -kq23 / kQ63A3, 0.0, kq34 / kQ63A3, kq35 / kQ63A3, kq36 / kQ63A3, 0.0,   \
      0.0, 0.0,                                                                                \
      -kq14 / kQ63A4, -kq24 / kQ63A4, -kq34 / kQ63A4, 0.0, kq45 / kQ63A4, kq46 / kQ63A4,       \
      kq47 / kQ63A4, 0.0, 0.0,                                                                 \
      -kq15 / kQ63A5, -kq25 / kQ63A5, -kq35 / kQ63A5, -kq45 / kQ63A5, 0.0, kq56 / kQ63A5,      \
      kq57 / kQ63A5, kq58 / kQ63A5, 0.0,                                                       \
      -kq16 / kQ63A6, -kq26 / kQ63A6, -kq36 / kQ63A6, -kq46 / kQ63A6, -kq56 / kQ63A6, 0.0,     \
      kq67 / kQ63A6, kq68 / kQ63A6, kq69 / kQ63A6},                                            \
     {-1.0 / 60.0, 3.0 / 20.0, -3.0 / 4.0, 0.0, 3.0 / 4.0, -3.0 / 20.0, 1.0 / 60.0},           \
     {kQ63A1, kQ63A2, kQ63A3, kQ63A4, kQ63A5, kQ63A6}},                                        \
  }

// The closure rows in FP32: the left-end rows rounded once at compile time
// (as a run-time conversion of the double would round them) and the
// right-end rows already negated, so no FP32 kernel converts a coefficient
// at run time (conversions from FP64 run on GB300's narrow FP64 pipe).
struct SbpF {
  float Ql[MAXNE * MAXNW];
  float Qr[MAXNE * MAXNW];   // -Ql
};
constexpr SbpC kSbpTables[4] = SWM_SBP_TABLES;
constexpr SbpF make_sbpf(const SbpC& c) {
  SbpF f{};
  for (int k = 0; k < MAXNE * MAXNW; ++k) {
    f.Ql[k] = float(c.Ql[k]);
    f.Qr[k] = float(-c.Ql[k]);
  }
  return f;
}

#ifdef __CUDACC__
// every translation unit carries its own initialised copy (no -rdc)
static __constant__ SbpC c_sbp[4] = SWM_SBP_TABLES;
static __constant__ SbpF c_sbpf[4] = {make_sbpf(kSbpTables[0]), make_sbpf(kSbpTables[1]),
                                      make_sbpf(kSbpTables[2]), make_sbpf(kSbpTables[3])};

// Closure coefficient m of left-end row k (sbp_ql) and of right-end row k,
// counted from the end, with its sign (sbp_qr = -Ql), in the element type.
template <class T> __device__ __forceinline__ T sbp_ql(int id, int k, int m);
template <class T> __device__ __forceinline__ T sbp_qr(int id, int k, int m);
template <> __device__ __forceinline__ float sbp_ql<float>(int id, int k, int m) {
  return c_sbpf[id].Ql[k * MAXNW + m];
}
template <> __device__ __forceinline__ float sbp_qr<float>(int id, int k, int m) {
  return c_sbpf[id].Qr[k * MAXNW + m];
}
template <> __device__ __forceinline__ double sbp_ql<double>(int id, int k, int m) {
  return c_sbp[id].Ql[k * MAXNW + m];
}
template <> __device__ __forceinline__ double sbp_qr<double>(int id, int k, int m) {
  return -c_sbp[id].Ql[k * MAXNW + m];
}
#endif

// index of an SBP order in the table above
__host__ __device__ inline int sbp_index(int order) {
  return order == 21 ? 0 : order == 42 ? 1 : order == 43 ? 2 : order == 63 ? 3 : -1;
}

// One side of a panel and where its duplicated nodes live on the neighbour:
// the neighbour panel q, the side of q that holds the same physical nodes,
// whether the along-side index runs backwards, and how the neighbour's
// vector components map into this panel's frame (the swap/negation that the
// reference's pack_to_buf_vec applies, parallel/buffer_mod.f90:171-277).
struct EdgeLink {
  int q, side_q, rev;
  int dim_i, istep, jstep;
};
struct Topology {
  EdgeLink link[6][4];
};

// Fused-kernel work unit: a strip of columns x a segment of rows of one panel.
struct WorkUnit {
  int16_t inst, panel;
  int16_t i0, i1, j0, j1;    // own output columns / rows [i0,i1) x [j0,j1)
  int16_t cl0, cl1, rl0, rl1;  // columns / rows the unit reads
};

// Per-instance pointers and constants of one fused stage launch.
template <class T>
struct InstDev {
  int n, P;
  int boxw;                   // TMA box width (columns) of this instance's strips
  long long ps, fs;           // panel stride n*P, field stride 6*n*P
  const T* metric;            // NMETRIC fields
  const double* qw;           // sync weights qb, qt, ql, qr (4*n, FP64)
  const T* hs;                // orography (nullable)
  const T* in;                // stage input state (3 fields)
  T* out;                     // apply: tendency; RK: next stage state
  const T* base;              // RK: v0 (FP64) / S_hi (FP32)
  T* acc;                     // RK: running sum (FP64 w / FP32 dacc)
  T* base_lo;                 // FP32 RK4 final stage: S_lo; S_hi is written via base_out
  T* base_out;                // final stage: new state (FP64 v0 / FP32 S_hi)
  T* edge;                    // edge buffer (6*4*4*n)
  const StageMaps* maps;      // TMA maps of this instance (batched launches; else null)
  T c_in;                     // stage coefficient for the next stage state
  T c_acc;                    // stage coefficient for the running sum
  T ghs;                      // 1 / (hx * a)
  T grav;
};

enum StageMode { MODE_APPLY = 0, MODE_RK1 = 1, MODE_RK2 = 2, MODE_RK3 = 3, MODE_RK4 = 4 };

}  // namespace swm
