// swm_diffusion.cu -- the hyperdiffusion split step on the GPU (FP64).
//
// The reference's drivers follow every RK4 step with one explicit Euler step
// of a diffusion operator (ts2_mod.f90:143-146,
// operator_swm_diff_mod.f90:25-46): the biharmonic -(c^4) L(L(h)) of the
// depth and of the three Cartesian components of the velocity, with L the
// narrow-stencil SBP Laplacian of order 4/2 or 6/3
// (laplace_Ah_sbp42_narrow_mod.f90:23-763 and its 6/3 twin).
//
// The narrow second-derivative operators have variable coefficients
// b = J*Qi11 (x) and J*Qi22 (y), which depend on the grid only, so the
// per-node stencil coefficients are built once per context: the interior
// stencil (2*hw+1 coefficients per node and direction) as fields, the
// closure rows (rows x cols per line end) as small tables.  A Laplacian is
// then two passes over the fields it is applied to:
//   1. d1x = D1x(f)*J*Qi12, d1y = D1y(f)*J*Qi12 (SBP first derivative of the
//      same order);
//   2. the narrow D2 in x and y from the precomputed coefficients, the
//      cross-derivative boundary fluxes on the panel edges, the mixed terms
//      D1y(d1x) + D1x(d1y), division by (hx*a)^2 and by J;
// followed by the Ah scalar edge sync.  Every pass handles nf fields per
// node so the coefficient loads are shared by h and the three Cartesian
// velocity components.
#include "swm_narrow_tables.h"
#include "swm_ops.cuh"

namespace swm {
namespace {

constexpr int DTPB = 256;
inline int dblk(long long count) { return (int)((count + DTPB - 1) / DTPB); }

__constant__ NarrowD2 c_narrow[2] = {kNarrow42, kNarrow63};

template <int NARROW>
struct NarrowShape {
  static constexpr int ni = NARROW == 63 ? 1 : 0;
  static constexpr int rows = NARROW == 63 ? kNarrow63.rows : kNarrow42.rows;
  static constexpr int cols = NARROW == 63 ? kNarrow63.cols : kNarrow42.cols;
  static constexpr int nb = NARROW == 63 ? kNarrow63.nb : kNarrow42.nb;
  static constexpr int hw = NARROW == 63 ? kNarrow63.hw : kNarrow42.hw;
  static constexpr int w = 2 * hw + 1;
  static constexpr int sbp = NARROW == 63 ? 3 : 1;   // index of the D1 operator in c_sbp
};

struct Node {
  int p, i, j;
  long long idx;   // pitched index
};
__device__ __forceinline__ Node node_at(const FieldGeom& g, long long gi) {
  Node r;
  const long long nn = (long long)g.n * g.n;
  r.p = (int)(gi / nn);
  const long long rem = gi - (long long)r.p * nn;
  r.j = (int)(rem / g.n);
  r.i = (int)(rem - (long long)r.j * g.n);
  r.idx = (long long)r.p * g.ps + (long long)r.j * g.P + r.i;
  return r;
}

// SBP first derivative at k of a line read through fa (sbp_operator_mod.f90:
// 152-228: left closure, interior, mirrored right closure).
template <class FA>
__device__ __forceinline__ double d1_line(int id, int k, int n, FA fa) {
  const SbpC& s = c_sbp[id];
  double acc = 0.0;
  if (k < s.ne) {
    for (int m = 0; m < s.last[k]; ++m) acc += s.Ql[k * MAXNW + m] * fa(m);
  } else if (k >= n - s.ne) {
    const int r = n - 1 - k;
    for (int m = s.last[r] - 1; m >= 0; --m) acc += (-s.Ql[r * MAXNW + m]) * fa(n - 1 - m);
  } else {
    for (int t = 0; t < s.nin; ++t) acc += s.Qin[t] * fa(k + s.inshift + t);
  }
  return acc;
}

// Interior stencil coefficients of both directions (zero at closure nodes):
// cx[o] multiplies f[i+o-hw] of the row, cy[o] f[j+o-hw] of the column.
template <int NARROW>
__global__ void narrow_coef_kernel(FieldGeom g, const double* m, double* cx, double* cy) {
  using S = NarrowShape<NARROW>;
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const Node k = node_at(g, gi);
  const NarrowD2& T = c_narrow[S::ni];
  const long long pb = (long long)k.p * g.ps;
  const double* J = m + MJ * g.fs + pb;
  const double* Q1 = m + MQI1 * g.fs + pb;
  const double* Q3 = m + MQI3 * g.fs + pb;
  const bool inx = k.i >= S::rows && k.i < g.n - S::rows;
  const bool iny = k.j >= S::rows && k.j < g.n - S::rows;
#pragma unroll
  for (int o = 0; o < S::w; ++o) {
    double ax = 0.0, ay = 0.0;
    if (inx)
      for (int q = 0; q < S::w; ++q) {
        const long long a = (long long)k.j * g.P + (k.i + q - S::hw);
        ax += T.in[o][q] * (Q1[a] * J[a]);
      }
    if (iny)
      for (int q = 0; q < S::w; ++q) {
        const long long a = (long long)(k.j + q - S::hw) * g.P + k.i;
        ay += T.in[o][q] * (Q3[a] * J[a]);
      }
    cx[o * g.fs + k.idx] = ax;
    cy[o * g.fs + k.idx] = ay;
  }
}

// Closure rows of both directions: entry ((((p*n + line)*2 + side)*rows + r)
// *cols + c) holds M[r][c] = sum_q C[r][c][q] b_q for the line's end `side`
// (nodes counted from that end).
template <int NARROW>
__global__ void narrow_closure_kernel(FieldGeom g, const double* m, double* clx, double* cly) {
  using S = NarrowShape<NARROW>;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long per = 6LL * g.n * 2 * S::rows * S::cols;
  if (e >= per) return;
  const int c = (int)(e % S::cols);
  const int r = (int)((e / S::cols) % S::rows);
  const int side = (int)((e / ((long long)S::cols * S::rows)) % 2);
  const long long pl = e / (2LL * S::cols * S::rows);
  const int p = (int)(pl / g.n), line = (int)(pl % g.n);
  const NarrowD2& T = c_narrow[S::ni];
  const long long pb = (long long)p * g.ps;
  const double* J = m + MJ * g.fs + pb;
  const double* Q1 = m + MQI1 * g.fs + pb;
  const double* Q3 = m + MQI3 * g.fs + pb;
  double mx = 0.0, my = 0.0;
  for (int q = 0; q < S::nb; ++q) {
    const int node = side ? g.n - 1 - q : q;
    const long long ax = (long long)line * g.P + node;    // x: along the row `line`
    const long long ay = (long long)node * g.P + line;    // y: along the column `line`
    mx += T.c[r][c][q] * (Q1[ax] * J[ax]);
    my += T.c[r][c][q] * (Q3[ay] * J[ay]);
  }
  clx[e] = mx;
  cly[e] = my;
}

// Pass 1: d1x = D1x(f)*J*Qi12, d1y = D1y(f)*J*Qi12 of nf fields
// (laplace_Ah_sbp42_narrow_mod.f90:60-93).
template <int NARROW>
__global__ void lap_d1_kernel(FieldGeom g, int nf, const double* f, long long fstride,
                              const double* m, double* d1x, double* d1y) {
  using S = NarrowShape<NARROW>;
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const Node k = node_at(g, gi);
  const double J = m[MJ * g.fs + k.idx], Q2 = m[MQI2 * g.fs + k.idx];
  for (int c = 0; c < nf; ++c) {
    const double* F = f + c * fstride + (long long)k.p * g.ps;
    const double dx = d1_line(S::sbp, k.i, g.n, [&](int q) { return F[(long long)k.j * g.P + q]; });
    const double dy = d1_line(S::sbp, k.j, g.n, [&](int q) { return F[(long long)q * g.P + k.i]; });
    d1x[c * g.fs + k.idx] = dx * J * Q2;
    d1y[c * g.fs + k.idx] = dy * J * Q2;
  }
}

// Pass 2: the pre-sync Laplacian of nf fields (laplace_Ah_sbp42_narrow_mod.f90
// :94-763 with the division by J of lines 52-53).
template <int NARROW>
__global__ void lap_main_kernel(FieldGeom g, int nf, const double* f, long long fstride,
                                const double* d1x, const double* d1y, const double* cx,
                                const double* cy, const double* clx, const double* cly,
                                const double* m, double hs, double* out) {
  using S = NarrowShape<NARROW>;
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const Node k = node_at(g, gi);
  const NarrowD2& T = c_narrow[S::ni];
  const int n = g.n;
  const bool clxn = k.i < S::rows || k.i >= n - S::rows;
  const bool clyn = k.j < S::rows || k.j >= n - S::rows;
  // stencil of this node in x and y: coefficients, first tap, tap step
  double ax[S::cols], ay[S::cols];
  int x0, xs, y0, ys;
  double rsx = 1.0, rsy = 1.0;
  if (clxn) {
    const int side = k.i < S::rows ? 0 : 1, r = side ? n - 1 - k.i : k.i;
    const double* M = clx + ((((long long)k.p * n + k.j) * 2 + side) * S::rows + r) * S::cols;
#pragma unroll
    for (int c = 0; c < S::cols; ++c) ax[c] = M[c];
    x0 = side ? n - 1 : 0; xs = side ? -1 : 1;
    rsx = T.rowscale[r];
  } else {
#pragma unroll
    for (int c = 0; c < S::cols; ++c) ax[c] = c < S::w ? cx[c * g.fs + k.idx] : 0.0;
    x0 = k.i - S::hw; xs = 1;
  }
  if (clyn) {
    const int side = k.j < S::rows ? 0 : 1, r = side ? n - 1 - k.j : k.j;
    const double* M = cly + ((((long long)k.p * n + k.i) * 2 + side) * S::rows + r) * S::cols;
#pragma unroll
    for (int c = 0; c < S::cols; ++c) ay[c] = M[c];
    y0 = side ? n - 1 : 0; ys = side ? -1 : 1;
    rsy = T.rowscale[r];
  } else {
#pragma unroll
    for (int c = 0; c < S::cols; ++c) ay[c] = c < S::w ? cy[c * g.fs + k.idx] : 0.0;
    y0 = k.j - S::hw; ys = 1;
  }
  const int ntx = clxn ? S::cols : S::w, nty = clyn ? S::cols : S::w;
  const double J = m[MJ * g.fs + k.idx];
  const double hs2 = hs * hs;
  const long long pb = (long long)k.p * g.ps;
  for (int c = 0; c < nf; ++c) {
    const double* F = f + c * fstride + pb;
    double sx = 0.0, sy = 0.0;
#pragma unroll
    for (int t = 0; t < S::cols; ++t)
      if (t < ntx) sx += ax[t] * F[(long long)k.j * g.P + (x0 + xs * t)];
#pragma unroll
    for (int t = 0; t < S::cols; ++t)
      if (t < nty) sy += ay[t] * F[(long long)(y0 + ys * t) * g.P + k.i];
    double d2x = clxn ? rsx * sx : sx;
    const double d2y = clyn ? rsy * sy : sy;
    const double* DX = d1x + c * g.fs + pb;
    const double* DY = d1y + c * g.fs + pb;
    const long long o = (long long)k.j * g.P + k.i;
    if (k.i == 0) d2x = d2x - 0.5 * (T.penalty * (-2.0 * DY[o]));
    if (k.i == n - 1) d2x = d2x - 0.5 * (T.penalty * (2.0 * DY[o]));
    if (k.j == 0) d2x = d2x - 0.5 * (T.penalty * (-2.0 * DX[o]));
    if (k.j == n - 1) d2x = d2x - 0.5 * (T.penalty * (2.0 * DX[o]));
    const double d2yx = d1_line(S::sbp, k.j, n, [&](int q) { return DX[(long long)q * g.P + k.i]; });
    const double d2xy = d1_line(S::sbp, k.i, n, [&](int q) { return DY[(long long)k.j * g.P + q]; });
    double v = 1.0 * d2x + 1.0 * d2y;
    v = v + 1.0 * d2xy + 1.0 * d2yx;
    v = v / hs2;
    out[c * g.fs + k.idx] = v / J;
  }
}

// Cartesian components of the covariant (u, v): b1*u + b2*v
// (vec_math_mod.f90:107-126).
__global__ void to_cart_kernel(FieldGeom g, const double* b, const double* u, const double* v,
                               double* cart) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const Node k = node_at(g, gi);
  const double uu = u[k.idx], vv = v[k.idx];
#pragma unroll
  for (int a = 0; a < 3; ++a)
    cart[a * g.fs + k.idx] = b[a * g.fs + k.idx] * uu + b[(3 + a) * g.fs + k.idx] * vv;
}

// Tendencies of (u, v): the projections of c*L (3 Cartesian fields) on b1
// and b2 (vec_math_mod.f90:128-160); and, with th != nullptr, the depth
// tendency ch*Lh.
__global__ void from_cart_kernel(FieldGeom g, const double* b, double cuv, const double* L,
                                 double* tu, double* tv, double ch, const double* Lh,
                                 double* th) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const Node k = node_at(g, gi);
  if (tu) {
    double t[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) t[a] = cuv * L[a * g.fs + k.idx];
    tu[k.idx] = t[0] * b[k.idx] + t[1] * b[g.fs + k.idx] + t[2] * b[2 * g.fs + k.idx];
    tv[k.idx] = t[0] * b[3 * g.fs + k.idx] + t[1] * b[4 * g.fs + k.idx] + t[2] * b[5 * g.fs + k.idx];
  }
  if (th) th[k.idx] = ch * Lh[k.idx];
}

// FP32 (hi, lo) pair += dt * t (t FP64), summed in FP64 and split again.
__global__ void pair_axpy_kernel(long long count, double dt, const double* t, float* hi,
                                 float* lo) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const double y = ((double)hi[k] + (double)lo[k]) + dt * t[k];
  const float h = (float)y;
  hi[k] = h;
  lo[k] = (float)(y - (double)h);
}

}  // namespace

int narrow_rows(int narrow) { return narrow == 63 ? kNarrow63.rows : kNarrow42.rows; }
int narrow_cols(int narrow) { return narrow == 63 ? kNarrow63.cols : kNarrow42.cols; }
int narrow_width(int narrow) { return narrow == 63 ? 2 * kNarrow63.hw + 1 : 2 * kNarrow42.hw + 1; }
long long narrow_closure_count(int narrow, int n) {
  return 6LL * n * 2 * narrow_rows(narrow) * narrow_cols(narrow);
}

cudaError_t launch_narrow_tables(const FieldGeom& g, const NarrowTables& t, const double* m,
                                 cudaStream_t st) {
  const long long nodes = 6LL * g.n * g.n, ncl = narrow_closure_count(t.narrow, g.n);
  if (t.narrow == 63) {
    narrow_coef_kernel<63><<<dblk(nodes), DTPB, 0, st>>>(g, m, t.cx, t.cy);
    narrow_closure_kernel<63><<<dblk(ncl), DTPB, 0, st>>>(g, m, t.clx, t.cly);
  } else {
    narrow_coef_kernel<42><<<dblk(nodes), DTPB, 0, st>>>(g, m, t.cx, t.cy);
    narrow_closure_kernel<42><<<dblk(ncl), DTPB, 0, st>>>(g, m, t.clx, t.cly);
  }
  return cudaGetLastError();
}

cudaError_t launch_laplace_presync(const FieldGeom& g, const NarrowTables& t, int nf,
                                   const double* f, long long fstride, const double* m, double hs,
                                   double* d1x, double* d1y, double* out, cudaStream_t st) {
  const long long nodes = 6LL * g.n * g.n;
  if (t.narrow == 63) {
    lap_d1_kernel<63><<<dblk(nodes), DTPB, 0, st>>>(g, nf, f, fstride, m, d1x, d1y);
    lap_main_kernel<63><<<dblk(nodes), DTPB, 0, st>>>(g, nf, f, fstride, d1x, d1y, t.cx, t.cy,
                                                      t.clx, t.cly, m, hs, out);
  } else {
    lap_d1_kernel<42><<<dblk(nodes), DTPB, 0, st>>>(g, nf, f, fstride, m, d1x, d1y);
    lap_main_kernel<42><<<dblk(nodes), DTPB, 0, st>>>(g, nf, f, fstride, d1x, d1y, t.cx, t.cy,
                                                      t.clx, t.cly, m, hs, out);
  }
  return cudaGetLastError();
}

cudaError_t launch_to_cart(const FieldGeom& g, const double* b12, const double* u, const double* v,
                           double* cart, cudaStream_t st) {
  to_cart_kernel<<<dblk(6LL * g.n * g.n), DTPB, 0, st>>>(g, b12, u, v, cart);
  return cudaGetLastError();
}

cudaError_t launch_diff_tendency(const FieldGeom& g, const double* b12, double cuv, const double* L,
                                 double* tu, double* tv, double ch, const double* Lh, double* th,
                                 cudaStream_t st) {
  from_cart_kernel<<<dblk(6LL * g.n * g.n), DTPB, 0, st>>>(g, b12, cuv, L, tu, tv, ch, Lh, th);
  return cudaGetLastError();
}

cudaError_t launch_pair_axpy(long long count, double dt, const double* t, float* hi, float* lo,
                             cudaStream_t st) {
  pair_axpy_kernel<<<dblk(count), DTPB, 0, st>>>(count, dt, t, hi, lo);
  return cudaGetLastError();
}

}  // namespace swm
