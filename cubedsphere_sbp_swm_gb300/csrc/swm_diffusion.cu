// swm_diffusion.cu -- the hyperdiffusion split step on the GPU.
//
// The reference's drivers follow every RK4 step with one explicit Euler step
// of a diffusion operator (ts2_mod.f90:143-146,
// operator_swm_diff_mod.f90:25-46): the biharmonic -(c^4) L(L(h)) of the
// depth and of the three Cartesian components of the velocity, with L the
// narrow-stencil SBP Laplacian of order 4/2, 6/3 or 2/1
// (laplace_Ah_sbp42_narrow_mod.f90:23-763, its 6/3 twin and
// laplace_Ah_sbp21_narrow_mod.f90:23-243).
//
// The narrow second-derivative operators have variable coefficients
// b = J*Qi11 (x) and J*Qi22 (y), which depend on the grid only, so the
// per-node stencil coefficients are built once per context (in FP64, stored
// in the element type): the interior stencil (2*hw+1 coefficients per node
// and direction) as fields, the closure rows (rows x cols per line end) as
// small tables (FP32 contexts form the interior coefficients from the two b
// fields instead).  A Laplacian computes d1x = D1x(f)*J*Qi12 and
// d1y = D1y(f)*J*Qi12 (SBP first derivative of the same order), then the
// narrow D2 in x and y, the cross-derivative boundary fluxes on the panel
// edges, the mixed terms D1y(d1x) + D1x(d1y), division by (hx*a)^2 and by J;
// followed by the Ah scalar edge sync.  FP32: one tiled pass with the first
// derivatives in shared memory (lap_tile_kernel); FP64: two passes with the
// first derivatives in work fields (lap_d1_kernel, lap_main_kernel).  Every
// pass handles nf fields per node so the coefficient and metric loads are
// shared by h and the three Cartesian velocity components.
//
// Element type T: double for FP64 contexts; float for FP32 contexts (the
// tendency is small next to the state, which stays a compensated pair
// updated in FP64).  GB300's FP64 rate bounds the FP64 passes.
#include "swm_narrow_tables.h"
#include "swm_ops.cuh"
#include "swm_stage.cuh"

namespace swm {
namespace {

constexpr int DTPB = 256;
inline int dblk(long long count) { return (int)((count + DTPB - 1) / DTPB); }

// table index of an order: [0] 4/2, [1] 6/3, [2] 2/1
constexpr int narrow_index(int narrow) { return narrow == 63 ? 1 : narrow == 21 ? 2 : 0; }
constexpr NarrowD2 kNarrowAll[3] = {kNarrow42, kNarrow63, kNarrow21};
__constant__ NarrowD2 c_narrow[3] = {kNarrow42, kNarrow63, kNarrow21};

// Interior stencil matrices of the three orders in FP32.
struct NarrowIn32 {
  float v[3][NARROW_MAXW][NARROW_MAXW];
};
constexpr NarrowIn32 make_narrow_in32() {
  NarrowIn32 t{};
  for (int o = 0; o < NARROW_MAXW; ++o)
    for (int q = 0; q < NARROW_MAXW; ++q)
      for (int x = 0; x < 3; ++x) t.v[x][o][q] = float(kNarrowAll[x].in[o][q]);
  return t;
}
__constant__ NarrowIn32 c_in32 = make_narrow_in32();

// Closure row scales and the flux penalty of the three orders in FP32
// (rounded at compile time: the FP32 Laplacian converts no coefficient at run
// time).
struct NarrowScale32 {
  float rowscale[3][NARROW_MAXR];
  float penalty[3];
};
constexpr NarrowScale32 make_narrow_scale32() {
  NarrowScale32 t{};
  for (int x = 0; x < 3; ++x) {
    for (int r = 0; r < NARROW_MAXR; ++r) t.rowscale[x][r] = float(kNarrowAll[x].rowscale[r]);
    t.penalty[x] = float(kNarrowAll[x].penalty);
  }
  return t;
}
__constant__ NarrowScale32 c_scale32 = make_narrow_scale32();

template <int NARROW>
struct NarrowShape {
  static constexpr int ni = narrow_index(NARROW);
  static constexpr int rows = kNarrowAll[ni].rows;
  static constexpr int cols = kNarrowAll[ni].cols;
  static constexpr int nb = kNarrowAll[ni].nb;
  static constexpr int hw = kNarrowAll[ni].hw;
  static constexpr int w = 2 * hw + 1;
  // stencil taps a node keeps: a closure row's cols or the interior's w
  // (2/1: 2 and 3)
  static constexpr int taps = cols > w ? cols : w;
};

// Node kernels run on 2-D tiles of TX columns x TY rows of the (6n)-row
// stack of panels, so a block reuses the rows its y-stencils share.
constexpr int TX = 32, TY = 8, RTPB = TX * TY;
inline dim3 row_grid(const FieldGeom& g) { return dim3((g.n + TX - 1) / TX, (6 * g.n + TY - 1) / TY); }
inline dim3 row_block() { return dim3(TX, TY); }

struct Node {
  int p, i, j;
  long long idx;   // pitched index
};
// false for the threads past the last column or row
__device__ __forceinline__ bool node_here(const FieldGeom& g, Node& r) {
  r.i = blockIdx.x * TX + threadIdx.x;
  const int row = blockIdx.y * TY + threadIdx.y;
  r.p = row / g.n;
  r.j = row - r.p * g.n;
  r.idx = (long long)r.p * g.ps + (long long)r.j * g.P + r.i;
  return r.i < g.n && row < 6 * g.n;
}

// Interior stencil coefficients of both directions (zero at closure nodes):
// cx[o] multiplies f[i+o-hw] of the row, cy[o] f[j+o-hw] of the column.
template <class T, int NARROW>
__global__ void narrow_coef_kernel(FieldGeom g, const double* m, T* cx, T* cy, T* b) {
  using S = NarrowShape<NARROW>;
  Node k;
  if (!node_here(g, k)) return;
  const NarrowD2& D = c_narrow[S::ni];
  const long long pb = (long long)k.p * g.ps;
  const double* J = m + MJ * g.fs + pb;
  const double* Q1 = m + MQI1 * g.fs + pb;
  const double* Q3 = m + MQI3 * g.fs + pb;
  const bool inx = k.i >= S::rows && k.i < g.n - S::rows;
  const bool iny = k.j >= S::rows && k.j < g.n - S::rows;
  const long long a0 = (long long)k.j * g.P + k.i;
  b[k.idx] = T(Q1[a0] * J[a0]);
  b[g.fs + k.idx] = T(Q3[a0] * J[a0]);
  if (!cx) return;
#pragma unroll
  for (int o = 0; o < S::w; ++o) {
    double ax = 0.0, ay = 0.0;
    if (inx)
      for (int q = 0; q < S::w; ++q) {
        const long long a = (long long)k.j * g.P + (k.i + q - S::hw);
        ax += D.in[o][q] * (Q1[a] * J[a]);
      }
    if (iny)
      for (int q = 0; q < S::w; ++q) {
        const long long a = (long long)(k.j + q - S::hw) * g.P + k.i;
        ay += D.in[o][q] * (Q3[a] * J[a]);
      }
    cx[o * g.fs + k.idx] = T(ax);
    cy[o * g.fs + k.idx] = T(ay);
  }
}

// Closure rows of both directions: entry ((((p*n + line)*2 + side)*rows + r)
// *cols + c) holds M[r][c] = sum_q C[r][c][q] b_q for the line's end `side`
// (nodes counted from that end); the row scale is applied after the sum.
template <class T, int NARROW>
__global__ void narrow_closure_kernel(FieldGeom g, const double* m, T* clx, T* cly) {
  using S = NarrowShape<NARROW>;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long per = 6LL * g.n * 2 * S::rows * S::cols;
  if (e >= per) return;
  const int c = (int)(e % S::cols);
  const int r = (int)((e / S::cols) % S::rows);
  const int side = (int)((e / ((long long)S::cols * S::rows)) % 2);
  const long long pl = e / (2LL * S::cols * S::rows);
  const int p = (int)(pl / g.n), line = (int)(pl % g.n);
  const NarrowD2& D = c_narrow[S::ni];
  const long long pb = (long long)p * g.ps;
  const double* J = m + MJ * g.fs + pb;
  const double* Q1 = m + MQI1 * g.fs + pb;
  const double* Q3 = m + MQI3 * g.fs + pb;
  double mx = 0.0, my = 0.0;
  for (int q = 0; q < S::nb; ++q) {
    const int node = side ? g.n - 1 - q : q;
    const long long ax = (long long)line * g.P + node;    // x: along the row `line`
    const long long ay = (long long)node * g.P + line;    // y: along the column `line`
    mx += D.c[r][c][q] * (Q1[ax] * J[ax]);
    my += D.c[r][c][q] * (Q3[ay] * J[ay]);
  }
  clx[e] = T(mx);
  cly[e] = T(my);
}

// FP32 Laplacian tiles: a block of LTX x LTY threads computes the pre-sync
// Laplacian of NF fields on a tile of LTX x LTY nodes of one panel, one node
// per thread (laplace_Ah_sbp42_narrow_mod.f90:23-763 with the division by J
// of lines 52-53).  Tiles start at multiples of the tile size; the last one
// of a line is moved back to end on the panel edge (its nodes overlap the
// previous tile's and get the same values), so a closure node's stencil stays
// inside the tile's region: [a0 - R, a0 + len + R) clipped to the panel,
// widened to the closure columns [0, cols) or [n - cols, n) when the tile
// holds closure nodes.  The block stages in shared memory, for all NF fields
// at once:
//   the fields on the region;
//   d1x = D1x(f)*J*Qi12 on the tile's columns x the region's rows and
//   d1y = D1y(f)*J*Qi12 on the region's columns x the tile's rows
//   (laplace_Ah_sbp42_narrow_mod.f90:60-93);
// together with J and Qi12 on both d1 areas and (FP32) the variable
// coefficients b, and then finishes its nodes from shared memory: the narrow
// D2 in x and y, the cross-derivative boundary fluxes, the mixed terms
// D1y(d1x) + D1x(d1y), the scaling, and the edge values for the sync.
constexpr int LTX = 32, LTY = 8, LTPB = LTX * LTY;

// 4-byte asynchronous copy global -> shared (no register round trip: every
// copy of a thread is in flight at once); cp_async_wait_all waits for this
// thread's copies, a barrier after it for the block's.
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

template <int NARROW, int NF>
struct LapTile {
  using S = NarrowShape<NARROW>;
  static constexpr int H1 = Ord<NARROW>::H;          // first-derivative interior half width
  static constexpr int R = S::hw > H1 ? S::hw : H1;  // interior reach
  // widest region of a tile of length L: L + R on the inner side, and on
  // the outer side R, or the rest of the closure columns when the tile
  // starts inside the closure rows.  A row tile (LTY < rows) can also start
  // inside the closure rows of one end and reach those of the other (small
  // panels): its region is then the whole line, shorter than 2 rows + LTY - 1.
  static constexpr int EXT = R + (R > S::rows - 1 ? R : S::rows - 1);
  static constexpr int RX = LTX + EXT;
  static constexpr int RY = LTY + (EXT > 2 * S::rows - 2 ? EXT : 2 * S::rows - 2);
  // shared-memory arrays, in floats: fields, d1x, d1y, then J and Qi12 on
  // the d1x and d1y areas, then b_x and b_y
  static constexpr int NDX = RY * LTX, NDY = LTY * RX;
  static constexpr int OFS_DX = NF * RY * RX, OFS_DY = OFS_DX + NF * NDX;
  static constexpr int OFS_JX = OFS_DY + NF * NDY, OFS_QX = OFS_JX + NDX;
  static constexpr int OFS_JY = OFS_QX + NDX, OFS_QY = OFS_JY + NDY;
  static constexpr int OFS_BX = OFS_QY + NDY, OFS_BY = OFS_BX + NDY;
  static constexpr size_t bytes = sizeof(float) * (size_t)(OFS_BY + NDX);
};

// region [lo, hi) of a tile [a0, a0 + len) along a line of n nodes
template <int NARROW>
__device__ __forceinline__ void lap_region(int a0, int len, int n, int& lo, int& hi) {
  using S = NarrowShape<NARROW>;
  constexpr int R = LapTile<NARROW, 1>::R;
  lo = max(0, a0 - R);
  hi = min(n, a0 + len + R);
  if (a0 < S::rows) {
    lo = 0;
    hi = max(hi, min(n, S::cols));
  }
  if (a0 + len > n - S::rows) {
    hi = n;
    lo = min(lo, max(0, n - S::cols));
  }
}

// SYNC_IN: Ein is the edge buffer of the kernel that wrote f, whose
// panel-side nodes still need their cube-edge scalar sync: the block applies
// it to the staged values of those nodes (value slot c of Ein for field c),
// the arithmetic of sync_fields_kernel, so the sync launch is not needed.
// (A compile-time switch: the code costs registers in the launches that do
// not need it.)
template <int NARROW, int NF, bool SYNC_IN = false>
__global__ void __launch_bounds__(LTPB, 4) lap_tile_kernel(FieldGeom g, int nty, const float* f,
                                                           const float* clx, const float* cly,
                                                           const float* bco, const float* mt,
                                                           float hs2, float* out, float* E,
                                                           const float* Ein,
                                                           const __grid_constant__ Topology tp) {
  using T = float;
  using S = NarrowShape<NARROW>;
  using LT = LapTile<NARROW, NF>;
  constexpr int RX = LT::RX, RY = LT::RY;
  extern __shared__ __align__(16) unsigned char lap_smem[];
  T* sm = reinterpret_cast<T*>(lap_smem);
  T(*Fs)[RY][RX] = reinterpret_cast<T(*)[RY][RX]>(sm);
  T(*DXs)[RY][LTX] = reinterpret_cast<T(*)[RY][LTX]>(sm + LT::OFS_DX);
  T(*DYs)[LTY][RX] = reinterpret_cast<T(*)[LTY][RX]>(sm + LT::OFS_DY);
  T(*JXs)[LTX] = reinterpret_cast<T(*)[LTX]>(sm + LT::OFS_JX);
  T(*QXs)[LTX] = reinterpret_cast<T(*)[LTX]>(sm + LT::OFS_QX);
  T(*JYs)[RX] = reinterpret_cast<T(*)[RX]>(sm + LT::OFS_JY);
  T(*QYs)[RX] = reinterpret_cast<T(*)[RX]>(sm + LT::OFS_QY);
  T(*BXs)[RX] = reinterpret_cast<T(*)[RX]>(sm + LT::OFS_BX);
  T(*BYs)[LTX] = reinterpret_cast<T(*)[LTX]>(sm + LT::OFS_BY);

  const int n = g.n, P = g.P;
  const int p = blockIdx.y / nty, ty = blockIdx.y - p * nty;
  const int tw = min(LTX, n), th = min(LTY, n);
  const int i0 = min((int)blockIdx.x * LTX, n - tw), j0 = min(ty * LTY, n - th);
  int xlo, xhi, ylo, yhi;
  lap_region<NARROW>(i0, tw, n, xlo, xhi);
  lap_region<NARROW>(j0, th, n, ylo, yhi);
  const int rx = xhi - xlo, ry = yhi - ylo;
  // tiles without closure nodes in a direction take the interior first
  // derivative there without the per-node closure tests
  const bool xin = i0 >= S::rows && i0 + tw <= n - S::rows;
  const bool yin = j0 >= S::rows && j0 + th <= n - S::rows;
  const long long pb = (long long)p * g.ps;
  const int lx = threadIdx.x, ly = threadIdx.y;

  // stage the fields on the region, the metric on the d1 areas and b.
  // Region rows go to thread rows, region columns to lanes.
  const T* MJp = mt + MJ * g.fs + pb;
  const T* MQp = mt + MQI2 * g.fs + pb;
  for (int y = ly; y < ry; y += LTY) {
    const long long rowa = (long long)(ylo + y) * P;
    for (int x = lx; x < rx; x += LTX) {
#pragma unroll
      for (int c = 0; c < NF; ++c) cp_async4(&Fs[c][y][x], f + c * g.fs + pb + rowa + xlo + x);
    }
    if (lx < tw) {
      const long long a = rowa + i0 + lx;
      cp_async4(&JXs[y][lx], MJp + a);
      cp_async4(&QXs[y][lx], MQp + a);
      cp_async4(&BYs[y][lx], bco + g.fs + pb + a);
    }
  }
  if (ly < th) {
    const long long rowa = (long long)(j0 + ly) * P;
    for (int x = lx; x < rx; x += LTX) {
      const long long a = rowa + xlo + x;
      cp_async4(&JYs[ly][x], MJp + a);
      cp_async4(&QYs[ly][x], MQp + a);
      cp_async4(&BXs[ly][x], bco + pb + a);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  if (SYNC_IN && (xlo == 0 || xhi == n || ylo == 0 || yhi == n)) {
    // the region's panel-side nodes: left and right columns, then bottom and
    // top rows without the corners the columns already took
    const EdgeView<float> ev{Ein, n};
    const int tid = ly * LTX + lx;
    for (int e = tid; e < 2 * (rx + ry); e += LTPB) {
      int x, y;
      if (e < ry) {
        if (xlo != 0) continue;
        x = 0; y = e;
      } else if (e < 2 * ry) {
        if (xhi != n) continue;
        x = rx - 1; y = e - ry;
      } else {
        const bool bottom = e < 2 * ry + rx;
        if (bottom ? ylo != 0 : yhi != n) continue;
        x = bottom ? e - 2 * ry : e - 2 * ry - rx;
        y = bottom ? 0 : ry - 1;
        if ((x == 0 && xlo == 0) || (x == rx - 1 && xhi == n)) continue;
      }
#pragma unroll
      for (int c = 0; c < NF; ++c)
        Fs[c][y][x] = sync_scalar_node<float>(ev, tp, p, xlo + x, ylo + y, c, Fs[c][y][x]);
    }
    __syncthreads();
  }

  // d1x on the tile's columns x the region's rows, d1y on the region's
  // columns x the tile's rows
  if (lx < tw) {
    const int i = i0 + lx;
    for (int y = ly; y < ry; y += LTY) {
      const T jq = JXs[y][lx], qq = QXs[y][lx];
#pragma unroll
      for (int c = 0; c < NF; ++c) {
        auto fa = [&](int q) { return Fs[c][y][q - xlo]; };
        const T dx = xin ? d_interior<NARROW, T>([&](int o) { return fa(i + o); })
                         : d_line<NARROW, T>(i, n, fa);
        DXs[c][y][lx] = dx * jq * qq;
      }
    }
  }
  if (ly < th) {
    const int j = j0 + ly;
    for (int x = lx; x < rx; x += LTX) {
      const T jq = JYs[ly][x], qq = QYs[ly][x];
#pragma unroll
      for (int c = 0; c < NF; ++c) {
        auto fa = [&](int q) { return Fs[c][q - ylo][x]; };
        const T dy = yin ? d_interior<NARROW, T>([&](int o) { return fa(j + o); })
                         : d_line<NARROW, T>(j, n, fa);
        DYs[c][ly][x] = dy * jq * qq;
      }
    }
  }
  __syncthreads();
  if (lx >= tw || ly >= th) return;

  const int i = i0 + lx, j = j0 + ly;
  const int yr = j - ylo, xr = i - xlo;
  if (xin && yin) {
    // A tile with no closure node and no panel side (most tiles): the same
    // terms in the same order as below, with every stencil offset known at
    // compile time and no per-node tests.
    T ax[S::w], ay[S::w];
#pragma unroll
    for (int c = 0; c < S::w; ++c) {
      T accx = T(0), accy = T(0);
#pragma unroll
      for (int q = 0; q < S::w; ++q) {
        accx += c_in32.v[S::ni][c][q] * BXs[ly][xr - S::hw + q];
        accy += c_in32.v[S::ni][c][q] * BYs[yr - S::hw + q][lx];
      }
      ax[c] = accx;
      ay[c] = accy;
    }
    const T inv = T(1) / (hs2 * JXs[yr][lx]);
#pragma unroll
    for (int c = 0; c < NF; ++c) {
      T sx = T(0), sy = T(0);
#pragma unroll
      for (int t = 0; t < S::w; ++t) sx += ax[t] * Fs[c][yr][xr - S::hw + t];
#pragma unroll
      for (int t = 0; t < S::w; ++t) sy += ay[t] * Fs[c][yr - S::hw + t][xr];
      const T d2yx = d_interior<NARROW, T>([&](int o) { return DXs[c][yr + o][lx]; });
      const T d2xy = d_interior<NARROW, T>([&](int o) { return DYs[c][ly][xr + o]; });
      T v = sx + sy;
      v = v + d2xy + d2yx;
      out[c * g.fs + pb + (long long)j * P + i] = v * inv;
    }
    return;
  }
  const bool clxn = i < S::rows || i >= n - S::rows;
  const bool clyn = j < S::rows || j >= n - S::rows;
  // stencil of this node in x and y: coefficients and tap offsets in the
  // region; the interior uses the first w taps
  T ax[S::taps], ay[S::taps];
  int x0, xs, y0, ys;
  T rsx = T(1), rsy = T(1);
  if (clxn) {
    const int side = i < S::rows ? 0 : 1, r = side ? n - 1 - i : i;
    const T* M = clx + ((((long long)p * n + j) * 2 + side) * S::rows + r) * S::cols;
#pragma unroll
    for (int c = 0; c < S::cols; ++c) ax[c] = M[c];
    x0 = (side ? n - 1 : 0) - xlo; xs = side ? -1 : 1;
    rsx = c_scale32.rowscale[S::ni][r];
  } else {   // from the variable coefficients along the row
#pragma unroll
    for (int c = 0; c < S::taps; ++c) {
      T acc = T(0);
      if (c < S::w) {
#pragma unroll
        for (int q = 0; q < S::w; ++q) acc += c_in32.v[S::ni][c][q] * BXs[ly][xr - S::hw + q];
      }
      ax[c] = acc;
    }
    x0 = xr - S::hw; xs = 1;
  }
  if (clyn) {
    const int side = j < S::rows ? 0 : 1, r = side ? n - 1 - j : j;
    const T* M = cly + ((((long long)p * n + i) * 2 + side) * S::rows + r) * S::cols;
#pragma unroll
    for (int c = 0; c < S::cols; ++c) ay[c] = M[c];
    y0 = (side ? n - 1 : 0) - ylo; ys = side ? -1 : 1;
    rsy = c_scale32.rowscale[S::ni][r];
  } else {   // from the variable coefficients along the column
#pragma unroll
    for (int c = 0; c < S::taps; ++c) {
      T acc = T(0);
      if (c < S::w) {
#pragma unroll
        for (int q = 0; q < S::w; ++q) acc += c_in32.v[S::ni][c][q] * BYs[yr - S::hw + q][lx];
      }
      ay[c] = acc;
    }
    y0 = yr - S::hw; ys = 1;
  }
  const T J = JXs[yr][lx];
  const T pen = c_scale32.penalty[S::ni];
  // one reciprocal of (hx a)^2 J for the NF divisions of the node
  const T inv = T(1) / (hs2 * J);
#pragma unroll
  for (int c = 0; c < NF; ++c) {
    // the closure rows read cols taps, the interior w (same order)
    T sx = T(0), sy = T(0);
    if (clxn) {
#pragma unroll
      for (int t = 0; t < S::cols; ++t) sx += ax[t] * Fs[c][yr][x0 + xs * t];
    } else {
#pragma unroll
      for (int t = 0; t < S::w; ++t) sx += ax[t] * Fs[c][yr][x0 + t];
    }
    if (clyn) {
#pragma unroll
      for (int t = 0; t < S::cols; ++t) sy += ay[t] * Fs[c][y0 + ys * t][xr];
    } else {
#pragma unroll
      for (int t = 0; t < S::w; ++t) sy += ay[t] * Fs[c][y0 + t][xr];
    }
    T d2x = clxn ? rsx * sx : sx;
    const T d2y = clyn ? rsy * sy : sy;
    const T dxo = DXs[c][yr][lx], dyo = DYs[c][ly][xr];
    if (i == 0) d2x = d2x - T(0.5) * (pen * (T(-2) * dyo));
    if (i == n - 1) d2x = d2x - T(0.5) * (pen * (T(2) * dyo));
    if (j == 0) d2x = d2x - T(0.5) * (pen * (T(-2) * dxo));
    if (j == n - 1) d2x = d2x - T(0.5) * (pen * (T(2) * dxo));
    auto fdx = [&](int q) { return DXs[c][q - ylo][lx]; };
    auto fdy = [&](int q) { return DYs[c][ly][q - xlo]; };
    const T d2yx = yin ? d_interior<NARROW, T>([&](int o) { return fdx(j + o); })
                       : d_line<NARROW, T>(j, n, fdx);
    const T d2xy = xin ? d_interior<NARROW, T>([&](int o) { return fdy(i + o); })
                       : d_line<NARROW, T>(i, n, fdy);
    T v = d2x + d2y;
    v = v + d2xy + d2yx;
    v = v * inv;
    out[c * g.fs + pb + (long long)j * P + i] = v;
    // panel-boundary values also go to value slot c of the edge buffer
    auto put = [&](int side, int q) { E[((long long)(p * 4 + side) * 4 + c) * n + q] = v; };
    if (i == 0) put(SIDE_L, j);
    if (i == n - 1) put(SIDE_R, j);
    if (j == 0) put(SIDE_B, i);
    if (j == n - 1) put(SIDE_T, i);
  }
}

// FP64 Laplacian, two passes of one node per thread.  GB300's FP64 rate
// bounds them, so they compute every first derivative once and keep it in
// work fields rather than recompute the tile halos of the FP32 kernel.
// Pass 1: d1x = D1x(f)*J*Qi12, d1y = D1y(f)*J*Qi12 of NF fields
// (laplace_Ah_sbp42_narrow_mod.f90:60-93).
template <class T, int NARROW, int NF>
__global__ void __launch_bounds__(RTPB) lap_d1_kernel(FieldGeom g, const T* f, const T* mt,
                                                      T* d1x, T* d1y) {
  Node k;
  if (!node_here(g, k)) return;
  const int o = k.j * g.P + k.i;   // offset inside the panel
  const long long pb = (long long)k.p * g.ps;
  const T J = mt[MJ * g.fs + pb + o], Q2 = mt[MQI2 * g.fs + pb + o];
#pragma unroll
  for (int c = 0; c < NF; ++c) {
    const T* F = f + c * g.fs + pb;
    const T dx = d_line<NARROW, T>(k.i, g.n, [&](int q) { return F[k.j * g.P + q]; });
    const T dy = d_line<NARROW, T>(k.j, g.n, [&](int q) { return F[q * g.P + k.i]; });
    d1x[c * g.fs + pb + o] = dx * J * Q2;
    d1y[c * g.fs + pb + o] = dy * J * Q2;
  }
}

// Pass 2: the pre-sync Laplacian of NF fields (laplace_Ah_sbp42_narrow_mod.f90
// :94-763 with the division by J of lines 52-53).
template <class T, int NARROW, int NF>
__global__ void __launch_bounds__(RTPB) lap_main_kernel(FieldGeom g, const T* f, const T* d1x,
                                                        const T* d1y, const T* cx, const T* cy,
                                                        const T* clx, const T* cly, const T* mt,
                                                        double hs, T* out, T* E) {
  using S = NarrowShape<NARROW>;
  Node k;
  if (!node_here(g, k)) return;
  const NarrowD2& D = c_narrow[S::ni];
  const int n = g.n, P = g.P;
  const int o = k.j * P + k.i;
  const long long pb = (long long)k.p * g.ps;
  const bool clxn = k.i < S::rows || k.i >= n - S::rows;
  const bool clyn = k.j < S::rows || k.j >= n - S::rows;
  // stencil of this node in x and y: coefficients and tap offsets (inside
  // the panel); the interior uses the first w taps
  T ax[S::taps], ay[S::taps];
  int x0, xs, y0, ys;
  T rsx = T(1), rsy = T(1);
  if (clxn) {
    const int side = k.i < S::rows ? 0 : 1, r = side ? n - 1 - k.i : k.i;
    const T* M = clx + ((((long long)k.p * n + k.j) * 2 + side) * S::rows + r) * S::cols;
#pragma unroll
    for (int c = 0; c < S::cols; ++c) ax[c] = M[c];
    x0 = k.j * P + (side ? n - 1 : 0); xs = side ? -1 : 1;
    rsx = T(D.rowscale[r]);
  } else {
#pragma unroll
    for (int c = 0; c < S::taps; ++c) ax[c] = c < S::w ? cx[c * g.fs + pb + o] : T(0);
    x0 = o - S::hw; xs = 1;
  }
  if (clyn) {
    const int side = k.j < S::rows ? 0 : 1, r = side ? n - 1 - k.j : k.j;
    const T* M = cly + ((((long long)k.p * n + k.i) * 2 + side) * S::rows + r) * S::cols;
#pragma unroll
    for (int c = 0; c < S::cols; ++c) ay[c] = M[c];
    y0 = (side ? n - 1 : 0) * P + k.i; ys = side ? -P : P;
    rsy = T(D.rowscale[r]);
  } else {
#pragma unroll
    for (int c = 0; c < S::taps; ++c) ay[c] = c < S::w ? cy[c * g.fs + pb + o] : T(0);
    y0 = o - S::hw * P; ys = P;
  }
  const int ntx = clxn ? S::cols : S::w, nty = clyn ? S::cols : S::w;
  const T J = mt[MJ * g.fs + pb + o];
  const T hs2 = T(hs * hs);
  const T pen = T(D.penalty);
#pragma unroll
  for (int c = 0; c < NF; ++c) {
    const T* F = f + c * g.fs + pb;
    T sx = T(0), sy = T(0);
#pragma unroll
    for (int t = 0; t < S::taps; ++t)
      if (t < ntx) sx += ax[t] * F[x0 + xs * t];
#pragma unroll
    for (int t = 0; t < S::taps; ++t)
      if (t < nty) sy += ay[t] * F[y0 + ys * t];
    T d2x = clxn ? rsx * sx : sx;
    const T d2y = clyn ? rsy * sy : sy;
    const T* DX = d1x + c * g.fs + pb;
    const T* DY = d1y + c * g.fs + pb;
    if (k.i == 0) d2x = d2x - T(0.5) * (pen * (T(-2) * DY[o]));
    if (k.i == n - 1) d2x = d2x - T(0.5) * (pen * (T(2) * DY[o]));
    if (k.j == 0) d2x = d2x - T(0.5) * (pen * (T(-2) * DX[o]));
    if (k.j == n - 1) d2x = d2x - T(0.5) * (pen * (T(2) * DX[o]));
    const T d2yx = d_line<NARROW, T>(k.j, n, [&](int q) { return DX[q * P + k.i]; });
    const T d2xy = d_line<NARROW, T>(k.i, n, [&](int q) { return DY[k.j * P + q]; });
    T v = d2x + d2y;
    v = v + d2xy + d2yx;
    v = v / hs2;
    v = v / J;
    out[c * g.fs + pb + o] = v;
    // panel-boundary values also go to value slot c of the edge buffer
    auto put = [&](int side, int q) { E[((long long)(k.p * 4 + side) * 4 + c) * n + q] = v; };
    if (k.i == 0) put(SIDE_L, k.j);
    if (k.i == n - 1) put(SIDE_R, k.j);
    if (k.j == 0) put(SIDE_B, k.i);
    if (k.j == n - 1) put(SIDE_T, k.i);
  }
}

// Cartesian components of the covariant (u, v): b1*u + b2*v
// (vec_math_mod.f90:107-126), and a copy of h into h_out (nullable).
template <class T>
__global__ void to_cart_kernel(FieldGeom g, const T* b, const T* h, const T* u, const T* v, T* h_out,
                               T* cart) {
  Node k;
  if (!node_here(g, k)) return;
  if (h_out) h_out[k.idx] = h[k.idx];
  const T uu = u[k.idx], vv = v[k.idx];
#pragma unroll
  for (int a = 0; a < 3; ++a)
    cart[a * g.fs + k.idx] = b[a * g.fs + k.idx] * uu + b[(3 + a) * g.fs + k.idx] * vv;
}

// Tendencies of (u, v): the projections of c*L (3 Cartesian fields) on b1
// and b2 (vec_math_mod.f90:128-160); and the depth tendency ch*Lh.
template <class T>
__global__ void from_cart_kernel(FieldGeom g, const T* b, T cuv, const T* L, T* tu, T* tv, T ch,
                                 const T* Lh, T* th) {
  Node k;
  if (!node_here(g, k)) return;
  T t[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) t[a] = cuv * L[a * g.fs + k.idx];
  tu[k.idx] = t[0] * b[k.idx] + t[1] * b[g.fs + k.idx] + t[2] * b[2 * g.fs + k.idx];
  tv[k.idx] = t[0] * b[3 * g.fs + k.idx] + t[1] * b[4 * g.fs + k.idx] + t[2] * b[5 * g.fs + k.idx];
  th[k.idx] = ch * Lh[k.idx];
}

// FP32 (hi, lo) pair element k += dt * t: the increment joins the low part,
// then a two-sum renormalises the pair (the compensated update of the RK4
// stage epilogue).
__device__ __forceinline__ void pair_add(float dt, float t, float* hi, float* lo, long long k) {
  const float d = dt * t;
  const float h = hi[k];
  const float tt = lo[k] + d;
  const float sm = h + tt;
  const float bb = sm - h;
  hi[k] = sm;
  lo[k] = (h - (sm - bb)) + (tt - bb);
}

// (hi, lo) pair += dt * t over count elements; FP64 tendencies are added in
// FP64.
template <class T>
__global__ void pair_axpy_kernel(long long count, double dt, const T* t, float* hi, float* lo) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  if constexpr (sizeof(T) == 4) {
    pair_add(float(dt), t[k], hi, lo, k);
  } else {
    const double y = ((double)hi[k] + (double)lo[k]) + dt * (double)t[k];
    const float h = (float)y;
    hi[k] = h;
    lo[k] = (float)(y - (double)h);
  }
}

// The FP32 diffusion step's update of the (hi, lo) state, in two launches
// with the arithmetic of from_cart_kernel, the covariant vector sync and
// pair_axpy_kernel:
//   diff_update_kernel: the tendencies (th, tu, tv) of every node; h and the
//     velocity's inner nodes are added to the pair at once; the velocity's
//     panel-boundary nodes store their tendencies in (tu, tv) and in the
//     edge buffer's GX/GY slots;
//   diff_sync_update_kernel: those nodes' covariant sync
//     (ecs_Ah_vec_sync_mod.f90:62-125), then their pair update.
//
// Ein (nullable): the edge buffer of the Laplacian that wrote Lh and L when
// their panel-side values still need the cube-edge scalar sync (value slot 0
// for Lh, 1..3 for L), applied here as sync_fields_kernel would.
__global__ void diff_update_kernel(FieldGeom g, const float* b, float cuv, const float* L, float ch,
                                   const float* Lh, float dt, float* hi, float* lo, float* tu,
                                   float* tv, float* E, const float* Ein,
                                   const __grid_constant__ Topology tp) {
  Node k;
  if (!node_here(g, k)) return;
  const long long fs = g.fs;
  const int n = g.n;
  const bool side = k.i == 0 || k.i == n - 1 || k.j == 0 || k.j == n - 1;
  float lv[3], lh = Lh[k.idx];
#pragma unroll
  for (int a = 0; a < 3; ++a) lv[a] = L[a * fs + k.idx];
  if (Ein && side) {
    const EdgeView<float> ev{Ein, n};
    lh = sync_scalar_node<float>(ev, tp, k.p, k.i, k.j, 0, lh);
#pragma unroll
    for (int a = 0; a < 3; ++a) lv[a] = sync_scalar_node<float>(ev, tp, k.p, k.i, k.j, 1 + a, lv[a]);
  }
  float t[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) t[a] = cuv * lv[a];
  const float ut = t[0] * b[k.idx] + t[1] * b[fs + k.idx] + t[2] * b[2 * fs + k.idx];
  const float vt = t[0] * b[3 * fs + k.idx] + t[1] * b[4 * fs + k.idx] + t[2] * b[5 * fs + k.idx];
  pair_add(dt, ch * lh, hi, lo, k.idx);
  if (k.i > 0 && k.i < n - 1 && k.j > 0 && k.j < n - 1) {
    pair_add(dt, ut, hi + fs, lo + fs, k.idx);
    pair_add(dt, vt, hi + 2 * fs, lo + 2 * fs, k.idx);
    return;
  }
  tu[k.idx] = ut;
  tv[k.idx] = vt;
  auto put = [&](int side, int q) {
    E[((long long)(k.p * 4 + side) * 4 + EV_GX) * n + q] = ut;
    E[((long long)(k.p * 4 + side) * 4 + EV_GY) * n + q] = vt;
  };
  if (k.i == 0) put(SIDE_L, k.j);
  if (k.i == n - 1) put(SIDE_R, k.j);
  if (k.j == 0) put(SIDE_B, k.i);
  if (k.j == n - 1) put(SIDE_T, k.i);
}

__global__ void diff_sync_update_kernel(FieldGeom g, Topology tp, const double* qw, const float* E,
                                        const float* tu, const float* tv, float dt, float* hi,
                                        float* lo) {
  const int n = g.n, nb = 4 * n - 4;
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6 * nb) return;
  const int p = gi / nb;
  int i, j;
  boundary_node(gi - p * nb, n, i, j);
  const long long x = (long long)p * g.ps + (long long)j * g.P + i;
  const EdgeView<float> ev{E, n};
  float a = tu[x], c = tv[x];
  sync_vector_node<float>(ev, tp, qw, p, i, j, a, c);
  pair_add(dt, a, hi + g.fs, lo + g.fs, x);
  pair_add(dt, c, hi + 2 * g.fs, lo + 2 * g.fs, x);
}

// Ah scalar sync of nf <= 4 fields at once (halo_Ah_scalar_sync_mod.f90:
// 38-93): field c comes from value slot c of the edge buffer, which the
// Laplacian kernel filled with the panel-boundary values.
template <class T>
__global__ void sync_fields_kernel(FieldGeom g, Topology tp, int nf, const T* E, T* f) {
  const int n = g.n, nb = 4 * n - 4;
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6 * nb) return;
  const int p = gi / nb;
  int i, j;
  boundary_node(gi - p * nb, n, i, j);
  const long long x = (long long)p * g.ps + (long long)j * g.P + i;
  const EdgeView<T> ev{E, n};
  for (int c = 0; c < nf; ++c) f[c * g.fs + x] = sync_scalar_node<T>(ev, tp, p, i, j, c, f[c * g.fs + x]);
}

__global__ void to_f32_kernel(long long count, const double* s, float* d) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < count) d[k] = (float)s[k];
}

}  // namespace

int narrow_rows(int narrow) { return kNarrowAll[narrow_index(narrow)].rows; }
int narrow_cols(int narrow) { return kNarrowAll[narrow_index(narrow)].cols; }
int narrow_width(int narrow) { return 2 * kNarrowAll[narrow_index(narrow)].hw + 1; }
long long narrow_closure_count(int narrow, int n) {
  return 6LL * n * 2 * narrow_rows(narrow) * narrow_cols(narrow);
}

template <class T, int NARROW, int NF>
cudaError_t laplace_nf(const FieldGeom& g, const Topology& tp, const NarrowTables<T>& t, const T* f,
                       const T* mt, double hs, T* d1x, T* d1y, T* out, T* edge, const T* edge_in,
                       cudaStream_t st) {
  if constexpr (sizeof(T) == 4) {
    const int nty = (g.n + LTY - 1) / LTY;
    const dim3 grid((g.n + LTX - 1) / LTX, 6 * nty), block(LTX, LTY);
    // (hx a)^2 rounded to FP32 once, as the kernel would round it
    if constexpr (NARROW == 42 && NF == 4) {
      if (edge_in) {
        lap_tile_kernel<NARROW, NF, true><<<grid, block, LapTile<NARROW, NF>::bytes, st>>>(
            g, nty, f, t.clx, t.cly, t.b, mt, float(hs * hs), out, edge, edge_in, tp);
        return cudaGetLastError();
      }
    } else if (edge_in) {
      return cudaErrorInvalidValue;
    }
      lap_tile_kernel<NARROW, NF><<<grid, block, LapTile<NARROW, NF>::bytes, st>>>(
          g, nty, f, t.clx, t.cly, t.b, mt, float(hs * hs), out, edge, nullptr, tp);
  } else {
    if (edge_in) return cudaErrorInvalidValue;   // FP64 inputs are synced by their own launch
    if (!d1x || !d1y) return cudaErrorInvalidValue;
    lap_d1_kernel<T, NARROW, NF><<<row_grid(g), row_block(), 0, st>>>(g, f, mt, d1x, d1y);
    lap_main_kernel<T, NARROW, NF><<<row_grid(g), row_block(), 0, st>>>(
        g, f, d1x, d1y, t.cx, t.cy, t.clx, t.cly, mt, hs, out, edge);
  }
  return cudaGetLastError();
}

// Shared memory above the default 48 KB for the FP32 Laplacian tiles of one
// order (set outside any stream capture).
template <int NARROW>
cudaError_t prepare_laplace_order() {
  cudaError_t e = cudaFuncSetAttribute(lap_tile_kernel<NARROW, 1>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)LapTile<NARROW, 1>::bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(lap_tile_kernel<NARROW, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)LapTile<NARROW, 3>::bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(lap_tile_kernel<NARROW, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)LapTile<NARROW, 4>::bytes);
  if constexpr (NARROW == 42) {   // the folded-sync form serves the 4/2 order only
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(lap_tile_kernel<NARROW, 4, true>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LapTile<NARROW, 4>::bytes);
  }
  return e;
}

template <class T>
cudaError_t launch_narrow_tables(const FieldGeom& g, const NarrowTables<T>& t, const double* m,
                                 cudaStream_t st) {
  const long long ncl = narrow_closure_count(t.narrow, g.n);
  if constexpr (sizeof(T) == 4) {
    cudaError_t e = t.narrow == 63   ? prepare_laplace_order<63>()
                    : t.narrow == 21 ? prepare_laplace_order<21>()
                                     : prepare_laplace_order<42>();
    if (e != cudaSuccess) return e;
  }
  if (t.narrow == 63) {
    narrow_coef_kernel<T, 63><<<row_grid(g), row_block(), 0, st>>>(g, m, t.cx, t.cy, t.b);
    narrow_closure_kernel<T, 63><<<dblk(ncl), DTPB, 0, st>>>(g, m, t.clx, t.cly);
  } else if (t.narrow == 21) {
    narrow_coef_kernel<T, 21><<<row_grid(g), row_block(), 0, st>>>(g, m, t.cx, t.cy, t.b);
    narrow_closure_kernel<T, 21><<<dblk(ncl), DTPB, 0, st>>>(g, m, t.clx, t.cly);
  } else {
    narrow_coef_kernel<T, 42><<<row_grid(g), row_block(), 0, st>>>(g, m, t.cx, t.cy, t.b);
    narrow_closure_kernel<T, 42><<<dblk(ncl), DTPB, 0, st>>>(g, m, t.clx, t.cly);
  }
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_laplace(const FieldGeom& g, const Topology& tp, const NarrowTables<T>& t, int nf,
                           const T* f, const T* mt, double hs, T* d1x, T* d1y, T* out, T* edge,
                           cudaStream_t st) {
  if (nf != 1 && nf != 3 && nf != 4) return cudaErrorInvalidValue;
  cudaError_t e;
  if (t.narrow == 63) {
    if (nf == 1) e = laplace_nf<T, 63, 1>(g, tp, t, f, mt, hs, d1x, d1y, out, edge, nullptr, st);
    else if (nf == 3) e = laplace_nf<T, 63, 3>(g, tp, t, f, mt, hs, d1x, d1y, out, edge, nullptr, st);
    else e = laplace_nf<T, 63, 4>(g, tp, t, f, mt, hs, d1x, d1y, out, edge, nullptr, st);
  } else if (t.narrow == 21) {
    if (nf == 1) e = laplace_nf<T, 21, 1>(g, tp, t, f, mt, hs, d1x, d1y, out, edge, nullptr, st);
    else if (nf == 3) e = laplace_nf<T, 21, 3>(g, tp, t, f, mt, hs, d1x, d1y, out, edge, nullptr, st);
    else e = laplace_nf<T, 21, 4>(g, tp, t, f, mt, hs, d1x, d1y, out, edge, nullptr, st);
  } else {
    if (nf == 1) e = laplace_nf<T, 42, 1>(g, tp, t, f, mt, hs, d1x, d1y, out, edge, nullptr, st);
    else if (nf == 3) e = laplace_nf<T, 42, 3>(g, tp, t, f, mt, hs, d1x, d1y, out, edge, nullptr, st);
    else e = laplace_nf<T, 42, 4>(g, tp, t, f, mt, hs, d1x, d1y, out, edge, nullptr, st);
  }
  if (e != cudaSuccess) return e;
  const int nb = 6 * (4 * g.n - 4);
  sync_fields_kernel<T><<<dblk(nb), DTPB, 0, st>>>(g, tp, nf, edge, out);
  return cudaGetLastError();
}

// The biharmonic operator's two FP32 Laplacians of the 4 fields
// [h, x, y, z] without sync launches: f -> L (panel-side values also to
// edge_a), then L -> f, whose staging syncs L's panel-side values from
// edge_a and which writes its own to edge_b.  f's panel-side nodes are left
// unsynced: the consumer syncs them from edge_b (launch_diff_update_f32).
// The 4/2 order only: measured on GB300, it saves 2.8% of the FP32
// diffusion step at N=384 d42, while for 6/3 the folded staging's register
// spills cost more than the two sync launches (0.77 -> 0.80 ms at N=1024).
cudaError_t launch_biharmonic_f32(const FieldGeom& g, const Topology& tp,
                                  const NarrowTables<float>& t, float* f, float* L, const float* mt,
                                  double hs, float* edge_a, float* edge_b, cudaStream_t st) {
  if (t.narrow != 42) return cudaErrorInvalidValue;
  cudaError_t e = laplace_nf<float, 42, 4>(g, tp, t, f, mt, hs, nullptr, nullptr, L, edge_a, nullptr, st);
  if (e == cudaSuccess)
    e = laplace_nf<float, 42, 4>(g, tp, t, L, mt, hs, nullptr, nullptr, f, edge_b, edge_a, st);
  return e;
}

template <class T>
cudaError_t launch_to_cart(const FieldGeom& g, const T* b12, const T* h, const T* u, const T* v,
                           T* h_out, T* cart, cudaStream_t st) {
  to_cart_kernel<T><<<row_grid(g), row_block(), 0, st>>>(g, b12, h, u, v, h_out, cart);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_diff_tendency(const FieldGeom& g, const T* b12, double cuv, const T* L, T* tu,
                                 T* tv, double ch, const T* Lh, T* th, cudaStream_t st) {
  from_cart_kernel<T><<<row_grid(g), row_block(), 0, st>>>(g, b12, T(cuv), L, tu, tv, T(ch), Lh,
                                                              th);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_pair_axpy(long long count, double dt, const T* t, float* hi, float* lo,
                             cudaStream_t st) {
  pair_axpy_kernel<T><<<dblk(count), DTPB, 0, st>>>(count, dt, t, hi, lo);
  return cudaGetLastError();
}

cudaError_t launch_diff_update_f32(const FieldGeom& g, const Topology& tp, const double* qw,
                                   const float* b12, double cuv, const float* L, double ch,
                                   const float* Lh, double dt, float* hi, float* lo, float* tu,
                                   float* tv, float* edge, const float* edge_in, cudaStream_t st) {
  // dt enters the FP32 increment rounded to FP32 (once, here)
  diff_update_kernel<<<row_grid(g), row_block(), 0, st>>>(g, b12, float(cuv), L, float(ch), Lh,
                                                            float(dt), hi, lo, tu, tv, edge, edge_in,
                                                            tp);
  const int nb = 6 * (4 * g.n - 4);
  diff_sync_update_kernel<<<dblk(nb), DTPB, 0, st>>>(g, tp, qw, edge, tu, tv, float(dt), hi, lo);
  return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(long long count, const double* s, float* d, cudaStream_t st) {
  to_f32_kernel<<<dblk(count), DTPB, 0, st>>>(count, s, d);
  return cudaGetLastError();
}

#define SWM_DIFF_INSTANTIATE(T)                                                                  \
  template cudaError_t launch_narrow_tables<T>(const FieldGeom&, const NarrowTables<T>&,         \
                                               const double*, cudaStream_t);                     \
  template cudaError_t launch_laplace<T>(const FieldGeom&, const Topology&, const NarrowTables<T>&,\
                                         int, const T*, const T*, double, T*, T*, T*, T*,        \
                                         cudaStream_t);                                          \
  template cudaError_t launch_to_cart<T>(const FieldGeom&, const T*, const T*, const T*, const T*,\
                                         T*, T*, cudaStream_t);                                  \
  template cudaError_t launch_diff_tendency<T>(const FieldGeom&, const T*, double, const T*, T*, \
                                               T*, double, const T*, T*, cudaStream_t);          \
  template cudaError_t launch_pair_axpy<T>(long long, double, const T*, float*, float*,          \
                                           cudaStream_t);
SWM_DIFF_INSTANTIATE(float)
SWM_DIFF_INSTANTIATE(double)

}  // namespace swm
