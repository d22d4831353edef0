// swm_cgrid.cu -- the C-grid SBP vector-invariant shallow-water operator on
// the GPU (FP64 and the FP32 form): metric of the four staggered meshes,
// cross-halo tables, the six passes of one right-hand side, the RK4 stage
// epilogue, the SBP_C quadrature, the hyperdiffusion and the ECS halos of the
// cell centres.
//
// One right-hand side (operator_swm_mod.f90:61-113 with the C-grid operators)
// is six passes over the panels:
//   centre_a  p points   J Qi12 times the other covariant component
//                        interpolated to the centres (co2contra, first half)
//   faces_a   u, v       contravariant components, mass fluxes h*u^i, J*flux
//                        and the kinetic-energy densities J u u^i / 2
//   curl      q points   staggered differences + SAT penalties
//   w2uv      u          the curl, with its Ah-type edge / corner average
//                        taken as it is read, interpolated to the x-faces
//   centre_b  p points   kinetic energy + g (h + hs), the divergence with its
//                        SAT penalties (h tendency), the Coriolis terms
//   faces_b   u, v       gradient with its SAT penalties + the Coriolis term
//                        interpolated back (u, v tendencies)
// The neighbours' points the SBP-SAT operators read across a panel edge come
// straight from the neighbouring panel through a precomputed table (one GPU
// holds all six panels, so the reference's halo exchange becomes an indexed
// load).
#include "swm_cgrid.h"
#include "swm_cube.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <initializer_list>
#include <vector>

namespace swm {

namespace {

constexpr double kPiC = 3.141592653589793238462643383279502884;
constexpr int kHaloDepth = 5;  // 3 for the SBP operators, 5 for the ECS_O corner formulas
constexpr int kMassBlocks = 256;
constexpr int kMassThreads = 256;

// Staggered 1-D SBP operator (sbp_operator_mod.f90:12-38, sbp_apply
// 152-228): left closure rows Ql[r*nw + m] over inputs m < last[r]; the
// right block mirrors them (times rsign); interior stencil Qin over inputs
// k+inshift .. k+inshift+w-1.  dnx = outputs - inputs.
template <class T>
struct StagOpT {
  int ne, nw, inshift, dnx;
  T rsign;
  int last[4];
  T Ql[24];
  T Qin[4];
};

// The operators and SAT constants of one SBP order, in the arithmetic type
// of the kernels (FP32 copies rounded once on the host).
template <class T>
struct COpsT {
  StagOpT<T> wc2i, wi2c, dc2i, di2c;
  int np;      // boundary projection length
  T proj[3];   // boundary projection (left)
  T pen_c[3];  // proj / A_centres: penalty of the divergence (at_center)
  T a_i0;      // A_interfaces(1): penalty weight of the curl
  T sq1;       // the gradient's first interface weight (7/18 at 4/2)
};
using StagOp = StagOpT<double>;
using COps = COpsT<double>;

template <class T>
StagOpT<T> stag_cast(const StagOp& s) {
  StagOpT<T> r{};
  r.ne = s.ne; r.nw = s.nw; r.inshift = s.inshift; r.dnx = s.dnx; r.rsign = T(s.rsign);
  for (int k = 0; k < 4; ++k) { r.last[k] = s.last[k]; r.Qin[k] = T(s.Qin[k]); }
  for (int k = 0; k < 24; ++k) r.Ql[k] = T(s.Ql[k]);
  return r;
}

template <class T>
COpsT<T> ops_cast(const COps& o) {
  COpsT<T> r{};
  r.wc2i = stag_cast<T>(o.wc2i); r.wi2c = stag_cast<T>(o.wi2c);
  r.dc2i = stag_cast<T>(o.dc2i); r.di2c = stag_cast<T>(o.di2c);
  r.np = o.np;
  for (int k = 0; k < 3; ++k) { r.proj[k] = T(o.proj[k]); r.pen_c[k] = T(o.pen_c[k]); }
  r.a_i0 = T(o.a_i0); r.sq1 = T(o.sq1);
  return r;
}

// Tables of the staggered operators (sbp_operators_collection_mod.f90:88-193
// and sbp_factory_mod.f90:38-179): the same numbers as the reference.
void fill_ops(int order, COps& o) {
  auto set = [](StagOp& s, int ne, int nw, std::initializer_list<double> q, std::initializer_list<int> last,
                std::initializer_list<double> in, int inshift, int dnx, double rsign) {
    s = StagOp{};
    s.ne = ne; s.nw = nw; s.inshift = inshift; s.dnx = dnx; s.rsign = rsign;
    int k = 0;
    for (double x : q) s.Ql[k++] = x;
    k = 0;
    for (int x : last) s.last[k++] = x;
    k = 0;
    for (double x : in) s.Qin[k++] = x;
  };
  o = COps{};
  if (order == 42) {
    set(o.wc2i, 4, 5,
        {1.3630402181345285, -0.17804474904273135, -0.23303115631809243, 0.048035687226327554, 0.0,
         0.46340770044238916, 0.4765661872892848, 0.15664452409426372, -0.09661841182593758, 0.0,
         0.07545241951434666, 0.44794495248229815, 0.37775283649236274, 0.09884979151099299, 0.0,
         -0.04413695843145285, -0.04040344754874627, 0.649837488701711, 0.4980831989686297, -0.06338028169014084},
        {4, 4, 4, 5}, {-1.0 / 16.0, 9.0 / 16.0, 9.0 / 16.0, -1.0 / 16.0}, -2, 1, 1.0);
    set(o.wi2c, 4, 6,
        {0.4892964885611128, 0.48123107353632727, 0.0696483872440123, -0.040175949341450676, 0.0, 0.0,
         -0.07913099957454726, 0.6127279550862234, 0.5119370885511979, -0.045534044062872786, 0.0, 0.0,
         -0.0869982983587545, 0.1691760860218048, 0.3626427230326682, 0.6151794893042863, -0.06, 0.0,
         0.018680545032460714, -0.10869571330417979, 0.09884979151099299, 0.4911653767607321, 0.5625, -0.0625},
        {4, 4, 5, 6}, {-1.0 / 16.0, 9.0 / 16.0, 9.0 / 16.0, -1.0 / 16.0}, -1, -1, 1.0);
    set(o.dc2i, 4, 5,
        {-2.0, 3.0, -1.0, 0.0, 0.0, -1.0, 1.0, 0.0, 0.0, 0.0, 1.0 / 24.0, -9.0 / 8.0, 9.0 / 8.0, -1.0 / 24.0, 0.0,
         -1.0 / 71.0, 6.0 / 71.0, -83.0 / 71.0, 81.0 / 71.0, -3.0 / 71.0},
        {3, 2, 4, 5}, {1.0 / 24.0, -9.0 / 8.0, 9.0 / 8.0, -1.0 / 24.0}, -2, 1, -1.0);
    set(o.di2c, 3, 5,
        {-79.0 / 78.0, 27.0 / 26.0, -1.0 / 26.0, 1.0 / 78.0, 0.0, 2.0 / 21.0, -9.0 / 7.0, 9.0 / 7.0, -2.0 / 21.0, 0.0,
         1.0 / 75.0, 0.0, -27.0 / 25.0, 83.0 / 75.0, -1.0 / 25.0},
        {4, 4, 5}, {1.0 / 24.0, -9.0 / 8.0, 9.0 / 8.0, -1.0 / 24.0}, -1, -1, -1.0);
    o.np = 3;
    const double proj[3] = {15.0 / 8.0, -5.0 / 4.0, 3.0 / 8.0};
    const double ac[3] = {13.0 / 12.0, 7.0 / 8.0, 25.0 / 24.0};
    for (int k = 0; k < 3; ++k) { o.proj[k] = proj[k]; o.pen_c[k] = proj[k] / ac[k]; }
    o.a_i0 = 7.0 / 18.0;
    o.sq1 = 7.0 / 18.0;
  } else {
    set(o.wc2i, 1, 1, {1.0}, {1}, {0.5, 0.5}, -1, 1, 1.0);
    set(o.wi2c, 1, 2, {0.5, 0.5}, {2}, {0.5, 0.5}, 0, -1, 1.0);
    set(o.dc2i, 1, 2, {-1.0, 1.0}, {2}, {-1.0, 1.0}, -1, 1, -1.0);
    set(o.di2c, 1, 2, {-1.0, 1.0}, {2}, {-1.0, 1.0}, 0, -1, -1.0);
    o.np = 2;
    o.proj[0] = 1.5; o.proj[1] = -0.5;
    o.pen_c[0] = 1.5 / 1.0; o.pen_c[1] = -0.5 / 1.0;
    o.a_i0 = 0.5;
    o.sq1 = 0.5;
  }
}

// Metric fields (one pitched field each) and work fields of one context.
// GB300's FP64 pipe is narrow, so the divisions of the operators are taken
// once on the host: reciprocal fields 1/J and 1/(J hx a), and J Qi12.  The
// covariant metric (J Q12, Q11, Q22) and 1/(J hx a) on the faces serve the
// contra2co transform and grad_perp of the hyperdiffusion.
enum { M_JP = 0, M_QI2P, M_FP, M_RJP, M_RJPHA, M_JQI2P,  // centres
       M_JU, M_QI1U, M_RJU,                              // x-faces
       M_JV, M_QI3V, M_RJV,                              // y-faces
       M_JQ, M_RJQHA,                                    // corners
       M_JQ2P, M_Q1U, M_Q3V, M_RJUHA, M_RJVHA,           // covariant metric, face 1/(J hx a)
       M_COUNT };
constexpr int kMetricMesh[M_COUNT] = {0, 0, 0, 0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 0, 1, 2, 1, 2};
enum { W_AP = 0, W_BP, W_UT, W_VT, W_HU, W_HV, W_GU, W_GV, W_KEU, W_KEV, W_CURL, W_FU, W_KE,
       W_CUP, W_CVP, W_COUNT };

// kernel flags
enum : int {
  F_CO = 1,        // faces_a: contravariant components from the covariant ones
  F_MF = 2,        // faces_a: mass fluxes
  F_G = 4,         // faces_a: J * mass flux
  F_KE = 8,        // faces_a: kinetic-energy densities; centre_b: kinetic energy
  F_ADDGH = 16,    // centre_b: + g h + g hs
  F_DIV = 32,      // centre_b: divergence
  F_COR = 64,      // centre_b: Coriolis terms at the centres; faces_b: back to the faces
  F_GRAD = 128,    // faces_b: gradient
  F_SEP = 256,     // centre_b / faces_b: write the operator's own output, not a tendency
  F_WUT = 512,     // faces_a: store the contravariant components (unfused co2contra)
  F_WFLUX = 1024,  // faces_a: store the mass fluxes (unfused massflux; the 2/1 divergence)
  F_QSYNC = 2048,  // w2uv: the curl is unsynced; average its edge and corner copies as it is read
};

template <class T>
struct CArgsT {
  FieldGeom g;
  int N, L, flags;
  int ord;  // SBP order of ops (21 or 42): the kernels' template argument
  T grav;
  T dx1;  // 1 / (a hx), the gradient's scale
  COpsT<T> ops;
  const T *Jp, *fp, *rJp, *rJpha, *JQi2p, *Ju, *Qi1u, *rJu, *Jv, *Qi3v, *rJv, *rJqha, *rJuha, *rJvha;
  const int* halo;
  // ECS_O halo: cubic weights [row 0..1][position -1..N+2][4], stencil bases, hx a
  const double* ecs_w;
  const int* ecs_ind;
  double hxa;
  // ecs_A_vec: the maps [edge][depth][position][4]; J on the first ring
  // beyond each edge [edge][position] (bottom, top, left, right)
  const double* ecs_tm;
  const double* ecs_jr;
  // ECS_xy: cubic weights [row 0..kXyRows-1][position 1-kXyRows..n+kXyRows][4], bases
  const double* xy_w;
  const int* xy_ind;
  double hx0, rad;  // hx and the radius
  // inputs
  const T *h, *u, *v, *hs, *ut_in, *vt_in, *hu_in, *hv_in, *ke_in, *curl_in;
  // intermediate and unfused outputs
  T *Ap, *Bp, *ut, *vt, *hu, *hv, *Gu, *Gv, *KEu, *KEv, *curl, *fu, *KE, *cup, *cvp;
  T *o1, *o2;  // unfused outputs of centre_b (div) / faces_b (gx|cor_u, gy|cor_v)
  // RK4 stage epilogue: mode 0 writes the tendency to tend, 1..4 the stages
  // of rk4_mod.f90:20-42 (y0, Y, Kb, acc: 3 fields each, fs apart; FP32:
  // y0 / lo the state pair, acc the running increment, no Kb)
  int mode;
  T hdt, dt, c3, c6;
  T *tend, *y0, *Y, *Kb, *acc, *lo;
};

// element offset within a field (fields stay below 2^31 elements)
__device__ __forceinline__ int at(const FieldGeom& g, int p, int i, int j) {
  return p * (int)g.ps + j * g.P + i;
}

// sbp_apply for output k of nout outputs over a line read through F(m)
template <int W, class T, class Fn>
__device__ __forceinline__ T stag_at_f(const StagOpT<T>& s, Fn F, int nout, int k) {
  T acc = T(0.0);
  if (k >= s.ne && k < nout - s.ne) {
#pragma unroll
    for (int t = 0; t < W; ++t) acc += s.Qin[t] * F(k + s.inshift + t);
  } else if (k < s.ne) {
    for (int m = 0; m < s.last[k]; ++m) acc += s.Ql[k * s.nw + m] * F(m);
  } else {
    const int nin = nout - s.dnx, r = nout - 1 - k;
    for (int m = s.last[r] - 1; m >= 0; --m) acc += (s.rsign * s.Ql[r * s.nw + m]) * F(nin - 1 - m);
  }
  return acc;
}

// sbp_apply for output k of nout outputs over a line f with stride st
template <int W, class T>
__device__ __forceinline__ T stag_at(const StagOpT<T>& s, const T* __restrict__ f, int st, int nout,
                                          int k) {
  T acc = T(0.0);
  if (k >= s.ne && k < nout - s.ne) {
    const T* b = f + (k + s.inshift) * st;
#pragma unroll
    for (int t = 0; t < W; ++t) acc += s.Qin[t] * b[t * st];
  } else if (k < s.ne) {
    for (int m = 0; m < s.last[k]; ++m) acc += s.Ql[k * s.nw + m] * f[m * st];
  } else {
    const int nin = nout - s.dnx, r = nout - 1 - k;
    for (int m = s.last[r] - 1; m >= 0; --m) acc += (s.rsign * s.Ql[r * s.nw + m]) * f[(nin - 1 - m) * st];
  }
  return acc;
}

// value of a neighbour's point in the cross halo: mesh 0 o, 1 u, 2 v, 3 q; side 0
// left, 1 right, 2 bottom, 3 top; depth d >= 1; k along the side.  f is the
// field of the mesh, g the other component of a C vector.
template <class T>
__device__ __forceinline__ T halo_at(const CArgsT<T>& a, int mesh, int side, int p, int d, int k,
                                          const T* __restrict__ f, const T* __restrict__ g) {
  const int c = __ldg(&a.halo[((((mesh * 4 + side) * 6 + p) * kHaloDepth + (d - 1)) * a.L) + k]);
  const T x = ((c & 2) ? g : f)[c >> 2];
  return (c & 1) ? -x : x;
}

template <class T>
__device__ __forceinline__ void rk_put(const CArgsT<T>& a, int comp, int e, T k) {
  const int o = comp * (int)a.g.fs + e;
  if constexpr (sizeof(T) == 8) {
    // FP64: the reference's order, y = 1*y0 + c k and
    // y0 = (y0 + dt/6 k1 + dt/3 k2) + dt/3 k3 + dt/6 k4
    switch (a.mode) {
      case 0: a.tend[o] = k; break;
      case 1: a.Kb[o] = k; a.Y[o] = T(1.0) * a.y0[o] + a.hdt * k; break;
      case 2: a.acc[o] = (a.y0[o] + a.c6 * a.Kb[o]) + a.c3 * k; a.Y[o] = T(1.0) * a.y0[o] + a.hdt * k; break;
      case 3: a.Kb[o] = k; a.Y[o] = T(1.0) * a.y0[o] + a.dt * k; break;
      default: a.y0[o] = (a.acc[o] + a.c3 * a.Kb[o]) + a.c6 * k; break;
    }
  } else {
    // FP32 compensated form (as on the Ah grid): the stage increments add up
    // apart from the state, and the last stage adds them to the (hi, lo)
    // state pair with an exact two-sum
    switch (a.mode) {
      case 0: a.tend[o] = k; break;
      case 1: a.Y[o] = a.y0[o] + a.hdt * k; a.acc[o] = a.c6 * k; break;
      case 2: a.Y[o] = a.y0[o] + a.hdt * k; a.acc[o] = a.acc[o] + a.c3 * k; break;
      case 3: a.Y[o] = a.y0[o] + a.dt * k; a.acc[o] = a.acc[o] + a.c3 * k; break;
      default: {
        const T d = a.acc[o] + a.c6 * k;
        const T hi = a.y0[o], lo = a.lo[o];
        const T t = lo + d;
        const T s = hi + t;
        const T bb = s - hi;
        a.y0[o] = s;
        a.lo[o] = (hi - (s - bb)) + (t - bb);
        break;
      }
    }
  }
}

#define SWM_C_INDEX(nx_, ny_)                                  \
  const int i = blockIdx.x * blockDim.x + threadIdx.x;        \
  const int j = blockIdx.y * blockDim.y + threadIdx.y;        \
  const int p = blockIdx.z;                                   \
  if (i >= (nx_) || j >= (ny_)) return;

// co2contra_c_sbp (co2contra_Cgrid_mod.f90:292-437), first half: the other
// covariant component interpolated to the centres times J Qi12 there.
template <int ORD, class T>
__global__ void __launch_bounds__(256) centre_a_kernel(const __grid_constant__ CArgsT<T> a) {
  constexpr int W = ORD == 42 ? 4 : 2;
  const int N = a.N;
  SWM_C_INDEX(N, N)
  const FieldGeom& g = a.g;
  const int e = at(g, p, i, j);
  const T jq = a.JQi2p[e];
  a.Ap[e] = jq * stag_at<W, T>(a.ops.wi2c, a.v + at(g, p, i, 0), g.P, N, j);
  a.Bp[e] = jq * stag_at<W, T>(a.ops.wi2c, a.u + at(g, p, 0, j), 1, N, i);
}

// co2contra second half, massflux_c_sbp (massflux_Cgrid_mod.f90:298-358),
// J * flux (div_c_sbp42_mod.f90:109-143, coriolis_Cgrid_mod.f90:83-97) and
// the kinetic-energy densities (KE_Cgrid_mod.f90:41-58) on the faces.
template <int ORD, class T>
__global__ void __launch_bounds__(256) faces_a_kernel(const __grid_constant__ CArgsT<T> a) {
  constexpr int W = ORD == 42 ? 4 : 2;
  const int N = a.N;
  SWM_C_INDEX(N + 1, N + 1)
  const FieldGeom& g = a.g;
  const int e = at(g, p, i, j);
  if (j < N) {  // u point
    T ut;
    if (a.flags & F_CO) {
      const T t = stag_at<W, T>(a.ops.wc2i, a.Ap + at(g, p, 0, j), 1, N + 1, i);
      ut = a.Qi1u[e] * a.u[e] + t * a.rJu[e];
      if (a.flags & F_WUT) a.ut[e] = ut;
    } else {
      ut = a.ut_in ? a.ut_in[e] : T(0.0);
    }
    if (a.flags & F_MF) {
      const T hu = ut * stag_at<W, T>(a.ops.wc2i, a.h + at(g, p, 0, j), 1, N + 1, i);
      if (a.flags & F_WFLUX) a.hu[e] = hu;
      if (a.flags & F_G) a.Gu[e] = hu * a.Ju[e];
    } else if (a.flags & F_G) {
      a.Gu[e] = a.hu_in[e] * a.Ju[e];
    }
    if (a.flags & F_KE) a.KEu[e] = a.Ju[e] * (a.u[e] * ut) * T(0.5);
  }
  if (i < N) {  // v point
    T vt;
    if (a.flags & F_CO) {
      const T t = stag_at<W, T>(a.ops.wc2i, a.Bp + at(g, p, i, 0), g.P, N + 1, j);
      vt = a.Qi3v[e] * a.v[e] + t * a.rJv[e];
      if (a.flags & F_WUT) a.vt[e] = vt;
    } else {
      vt = a.vt_in ? a.vt_in[e] : T(0.0);
    }
    if (a.flags & F_MF) {
      const T hv = vt * stag_at<W, T>(a.ops.wc2i, a.h + at(g, p, i, 0), g.P, N + 1, j);
      if (a.flags & F_WFLUX) a.hv[e] = hv;
      if (a.flags & F_G) a.Gv[e] = hv * a.Jv[e];
    } else if (a.flags & F_G) {
      a.Gv[e] = a.hv_in[e] * a.Jv[e];
    }
    if (a.flags & F_KE) a.KEv[e] = a.Jv[e] * (a.v[e] * vt) * T(0.5);
  }
}

// curl_c_sbp (curl/curl_c_sbp_mod.f90:44-127) before the corner sync: the
// staggered differences of the covariant components onto the corners, with
// the SAT penalties on their jumps across the panel edges.
template <int ORD, class T>
__global__ void __launch_bounds__(256) curl_kernel(const __grid_constant__ CArgsT<T> a) {
  constexpr int W = ORD == 42 ? 4 : 2;
  const int N = a.N;
  SWM_C_INDEX(N + 1, N + 1)
  const FieldGeom& g = a.g;
  const COpsT<T>& o = a.ops;
  const T* vrow = a.v + at(g, p, 0, j);
  const T* ucol = a.u + at(g, p, i, 0);
  T dvx = stag_at<W, T>(o.dc2i, vrow, 1, N + 1, i);
  if (i == 0) {
    T dv = T(0.0);
    for (int m = 0; m < o.np; ++m) dv = dv + o.proj[m] * (vrow[m] - halo_at(a, 2, 0, p, m + 1, j, a.v, a.u));
    dvx = dvx + T(0.5) * dv / o.a_i0;
  }
  if (i == N) {
    T dv = T(0.0);
    for (int m = 0; m < o.np; ++m) dv = dv + o.proj[m] * (halo_at(a, 2, 1, p, m + 1, j, a.v, a.u) - vrow[N - 1 - m]);
    dvx = dvx + T(0.5) * dv / o.a_i0;
  }
  T duy = stag_at<W, T>(o.dc2i, ucol, g.P, N + 1, j);
  if (j == 0) {
    T du = T(0.0);
    for (int m = 0; m < o.np; ++m) du = du + o.proj[m] * (ucol[m * g.P] - halo_at(a, 1, 2, p, m + 1, i, a.u, a.v));
    duy = duy + T(0.5) * du / o.a_i0;
  }
  if (j == N) {
    T du = T(0.0);
    for (int m = 0; m < o.np; ++m)
      du = du + o.proj[m] * (halo_at(a, 1, 3, p, m + 1, i, a.u, a.v) - ucol[(N - 1 - m) * g.P]);
    duy = duy + T(0.5) * du / o.a_i0;
  }
  const int e = at(g, p, i, j);
  a.curl[e] = (dvx - duy) * a.rJqha[e];
}

// interp_w2h, first half (interpolator_w2h_mod.f90:25-67): the corner field
// interpolated along y to the u points.  The reference averages two
// tensor-product interpolations to the centres, x after y and y after x;
// the 1-D operators act on different indices, so both are the same linear
// map and one of them is evaluated (the results agree to round-off).
//
// With F_QSYNC the curl comes straight from curl_kernel, unsynced, and its
// edge and corner points are averaged with the neighbours' copies here, as
// they are read: the Ah-type sync of the corner mesh
// (halo/halo_Ah_scalar_sync_mod.f90:38-93, in the order of the sync kernel),
// with the copies from the corner mesh's cross-halo table.  That saves the
// sync's two launches per stage in the fused step, where this pass is the
// curl's only reader.
template <class T>
__device__ __forceinline__ T curl_synced(const CArgsT<T>& a, int p, int i, int j) {
  const int N = a.N;
  const T* c = a.curl_in;
  const T own = c[at(a.g, p, i, j)];
  if (i > 0 && i < N && j > 0 && j < N) return own;
  auto H = [&](int side, int k) { return halo_at(a, 3, side, p, 1, k, c, c); };
  if (i == 0 && j == 0) return (own + H(0, 0) + H(2, 0)) / T(3.0);
  if (i == N && j == 0) return (own + H(1, 0) + H(2, N)) / T(3.0);
  if (i == 0 && j == N) return (own + H(0, N) + H(3, 0)) / T(3.0);
  if (i == N && j == N) return (own + H(1, N) + H(3, N)) / T(3.0);
  if (i == 0) return T(0.5) * (H(0, j) + own);
  if (i == N) return T(0.5) * (own + H(1, j));
  if (j == 0) return T(0.5) * (own + H(2, i));
  return T(0.5) * (own + H(3, i));
}

template <int ORD, class T>
__global__ void __launch_bounds__(256) w2uv_kernel(const __grid_constant__ CArgsT<T> a) {
  constexpr int W = ORD == 42 ? 4 : 2;
  const int N = a.N;
  SWM_C_INDEX(N + 1, N)
  const FieldGeom& g = a.g;
  if (a.flags & F_QSYNC)
    a.fu[at(g, p, i, j)] = stag_at_f<W, T>(a.ops.wi2c, [&](int m) { return curl_synced(a, p, i, m); }, N, j);
  else
    a.fu[at(g, p, i, j)] = stag_at<W, T>(a.ops.wi2c, a.curl_in + at(g, p, i, 0), g.P, N, j);
}

// grad_perp_c_sbp (grad_perp/grad_perp_c_sbp_mod.f90:20-95): the staggered
// differences of the corner field w along y onto the x-faces and along x onto
// the y-faces, each with the "at_center" SAT penalty on the jump between the
// panel's edge point and the neighbour's copy of it
// (sbp_operator_mod.f90:343-391); gu = -(.) / (J a hx), gv = (.) / (J a hx).
template <int ORD, class T>
__global__ void __launch_bounds__(256) gperp_kernel(const __grid_constant__ CArgsT<T> a) {
  constexpr int W = ORD == 42 ? 4 : 2;
  const int N = a.N;
  SWM_C_INDEX(N + 1, N + 1)
  const FieldGeom& g = a.g;
  const COpsT<T>& o = a.ops;
  const T* w = a.curl_in;
  const int e = at(g, p, i, j);
  if (j < N) {  // x-face: along the column i
    const T* col = w + at(g, p, i, 0);
    T s = stag_at<W, T>(o.di2c, col, g.P, N, j);
    if (j < o.np) s = s + T(0.5) * o.pen_c[j] * (col[0] - halo_at(a, 3, 2, p, 1, i, w, w));
    if (j >= N - o.np) s = s + T(0.5) * o.pen_c[N - 1 - j] * (halo_at(a, 3, 3, p, 1, i, w, w) - col[N * g.P]);
    a.o1[e] = -s * a.rJuha[e];
  }
  if (i < N) {  // y-face: along the row j
    const T* row = w + at(g, p, 0, j);
    T s = stag_at<W, T>(o.di2c, row, 1, N, i);
    if (i < o.np) s = s + T(0.5) * o.pen_c[i] * (row[0] - halo_at(a, 3, 0, p, 1, j, w, w));
    if (i >= N - o.np) s = s + T(0.5) * o.pen_c[N - 1 - i] * (halo_at(a, 3, 1, p, 1, j, w, w) - row[N]);
    a.o2[e] = s * a.rJvha[e];
  }
}

// Last pass of the hyperdiffusion (hordiff_Cgrid_mod.f90:59-140,
// hordiff_scalar_mod.f90:33-53): th = c4h L(L(h)); (tu, tv) = c4uv A +
// 1.0 (c4uv B), A the curl part, B the divergence part (parts 1 B only, 2 A
// only, 3 both).  mode 0 stores the tendency, 1 the explicit Euler step
// y + dt t (explicit_Eul1_mod.f90:20-30) in place, 2 the same step on an
// FP32 (hi, lo) state pair with an exact two-sum.
template <class T>
__global__ void __launch_bounds__(256) diff_combine_kernel(FieldGeom g, int N, int parts, T c4uv, T c4h,
                                                           const T* __restrict__ Lh, const T* __restrict__ Au,
                                                           const T* __restrict__ Av, const T* __restrict__ Bu,
                                                           const T* __restrict__ Bv, int mode, double dt, T* out,
                                                           float* lo) {
  SWM_C_INDEX(N + 1, N + 1)
  const int e = at(g, p, i, j);
  auto put = [&](int comp, T t) {
    const long long o = comp * g.fs + e;
    if (mode == 0) {
      out[o] = t;
    } else if (mode == 1) {
      out[o] = out[o] + T(dt) * t;
    } else {
      // the increment joins the low part, then an exact FP32 two-sum
      // renormalises the pair (FP64 arithmetic here would make this pass
      // bound by GB300's narrow FP64 pipe)
      const float d = float(dt) * float(t);
      const float h = float(out[o]);
      const float tt = lo[o] + d;
      const float sm = h + tt;
      const float bb = sm - h;
      out[o] = T(sm);
      lo[o] = (h - (sm - bb)) + (tt - bb);
    }
  };
  auto mix = [&](T A, T B) {
    if (parts == 1) return c4uv * B;
    if (parts == 2) return c4uv * A;
    return c4uv * A + T(1.0) * (c4uv * B);
  };
  if (i < N && j < N) put(0, c4h * Lh[e]);
  if (j < N) put(1, mix(Au[e], Bu[e]));
  if (i < N) put(2, mix(Av[e], Bv[e]));
}

// ------------------------------------------------------------------ ECS_O
// The ECS_O scalar halo of a cell-centre field (equiang_cs/ecs_halo_mod.f90:
// 95-475), evaluated where it is read instead of stored: (i1, j1) are the
// reference's 1-based tile indices, a halo point lies within two rows of the
// panel.  ecs_x is the neighbour's value the 'full' o-point exchange places
// there (exactly one of i1, j1 outside [1, N]).
__device__ __forceinline__ double ecs_x(const CArgsT<double>& a, const double* f, int p, int i1, int j1) {
  const int N = a.N;
  if (i1 >= 1 && i1 <= N && j1 >= 1 && j1 <= N) return f[at(a.g, p, i1 - 1, j1 - 1)];
  int side, d, k;
  if (i1 < 1) { side = 0; d = 1 - i1; k = j1 - 1; }
  else if (i1 > N) { side = 1; d = i1 - N; k = j1 - 1; }
  else if (j1 < 1) { side = 2; d = 1 - j1; k = i1 - 1; }
  else { side = 3; d = j1 - N; k = i1 - 1; }
  const int c = __ldg(&a.halo[(((0 * 4 + side) * 6 + p) * kHaloDepth + (d - 1)) * a.L + k]);
  return f[c >> 2];
}

__device__ __forceinline__ double ecs_wt(const CArgsT<double>& a, int m, int i, int r) {
  return __ldg(&a.ecs_w[((r - 1) * (a.N + 4) + (i + 1)) * 4 + (m + 1)]);
}

// The six corner values of corner c (1 at (0,0), 2 at (N+1,0), 3 at
// (N+1,N+1), 4 at (0,N+1)) from ecs_halo_1corner (ecs_halo_mod.f90:179-260):
// k = 0..5 at the corner-relative points (0,1), (1,0), (0,0), (-1,0), (0,-1),
// (-1,-1), the last three for width 2 only.
template <class XF>
__device__ double ecs_corner(const CArgsT<double>& a, XF X, int c, int k) {
  const int N = a.N;
  const int ist = (c == 1 || c == 2) ? N + 1 : 0, jst = c >= 2 ? N + 1 : 0;
  const int idr = (c == 1 || c == 2) ? -1 : 1, jdr = c >= 2 ? -1 : 1;
  auto fc = [&](int i, int j) { return X(ist + idr * i, jst + jdr * j); };
  // the weights of corner 1, mirrored for the corners at i = N+1
  auto pw = [&](int m, int i, int r) { return idr == 1 ? ecs_wt(a, m, i, r) : ecs_wt(a, 1 - m, N + 1 - i, r); };
  const double zw = pw(-1, 1, 1), zw2 = zw * zw, zw3 = zw2 * zw;
  const double z0 = pw(0, 1, 1), z1 = pw(1, 1, 1), z2 = pw(2, 1, 1);
  double zx = z0 * fc(0, 1) + z1 * fc(0, 2) + z2 * fc(0, 3);
  double zy = z0 * fc(1, 0) + z1 * fc(1, -1) + z2 * fc(1, -2);
  double zz = z0 * fc(1, 1) + z1 * fc(2, 1) + z2 * fc(3, 1);
  if (k == 0) return (zx + zw * zy + zw2 * zz) / (1.0 - zw3);
  const double zfy1 = (zy + zw * zz + zw2 * zx) / (1.0 - zw3);
  zx = z0 * fc(1, 0) + z1 * fc(2, 0) + z2 * fc(3, 0);
  zy = z0 * fc(0, 1) + z1 * fc(-1, 1) + z2 * fc(-2, 1);
  zz = z0 * fc(1, 1) + z1 * fc(1, 2) + z2 * fc(1, 3);
  if (k == 1) return (zx + zw * zy + zw2 * zz) / (1.0 - zw3);
  const double zfy2 = (zy + zw * zz + zw2 * zx) / (1.0 - zw3);
  if (k == 2) {
    const double zff1 = pw(-1, 1, 2) * fc(2, 0) + pw(0, 1, 2) * fc(2, -1) + pw(1, 1, 2) * fc(2, -2) + pw(2, 1, 2) * fc(2, -3);
    const double zff2 = pw(-1, 1, 2) * fc(0, 2) + pw(0, 1, 2) * fc(-1, 2) + pw(1, 1, 2) * fc(-2, 2) + pw(2, 1, 2) * fc(-3, 2);
    return 0.5 * (pw(-1, 0, 1) * zff1 + pw(0, 0, 1) * zfy1 + pw(1, 0, 1) * fc(0, 1) + pw(2, 0, 1) * fc(0, 2) +
                  pw(-1, 0, 1) * zff2 + pw(0, 0, 1) * zfy2 + pw(1, 0, 1) * fc(1, 0) + pw(2, 0, 1) * fc(2, 0));
  }
  const double zff1 = pw(-1, 2, 1) * fc(1, 0) + pw(0, 2, 1) * fc(1, -1) + pw(1, 2, 1) * fc(1, -2) + pw(2, 2, 1) * fc(1, -3);
  const double zff2 = pw(-1, 2, 1) * fc(0, 1) + pw(0, 2, 1) * fc(-1, 1) + pw(1, 2, 1) * fc(-2, 1) + pw(2, 2, 1) * fc(-3, 1);
  if (k == 3) return pw(-1, 0, 2) * zff1 + pw(0, 0, 2) * fc(-1, 1) + pw(1, 0, 2) * fc(-1, 2) + pw(2, 0, 2) * fc(-1, 3);
  if (k == 4) return pw(-1, 0, 2) * zff2 + pw(0, 0, 2) * fc(1, -1) + pw(1, 0, 2) * fc(2, -1) + pw(2, 0, 2) * fc(3, -1);
  const double zff11 = pw(-1, 2, 2) * fc(2, -1) + pw(0, 2, 2) * fc(2, -2) + pw(1, 2, 2) * fc(2, -3) + pw(2, 2, 2) * fc(2, -4);
  const double zff22 = pw(-1, 2, 2) * fc(-1, 2) + pw(0, 2, 2) * fc(-2, 2) + pw(1, 2, 2) * fc(-3, 2) + pw(2, 2, 2) * fc(-4, 2);
  return 0.5 * (pw(-1, -1, 2) * zff11 + pw(0, -1, 2) * zff1 + pw(1, -1, 2) * fc(-1, 1) + pw(2, -1, 2) * fc(-1, 2) +
                pw(-1, -1, 2) * zff22 + pw(0, -1, 2) * zff2 + pw(1, -1, 2) * fc(1, -1) + pw(2, -1, 2) * fc(2, -1));
}

// The ECS_O value at the halo point (i1, j1) of a halo of width hw (1 or 2):
// a corner value where the point is one of its corner's special points, else
// the cubic interpolation along the edge (ecs_ext_halo_1e) of row r.  X(i1,
// j1) gives the exchanged values (the vector halo passes its mapped
// components).
template <class XF>
__device__ double ecs_o_at_x(const CArgsT<double>& a, XF X, int i1, int j1, int hw) {
  const int N = a.N;
  const int ci[6] = {0, 1, 0, -1, 0, -1}, cj[6] = {1, 0, 0, 0, -1, -1};
  for (int c = 0; c < 4; ++c) {
    const int ist = (c == 1 || c == 2) ? N + 1 : 0, jst = c >= 2 ? N + 1 : 0;
    const int idr = (c == 1 || c == 2) ? -1 : 1, jdr = c >= 2 ? -1 : 1;
    const int ri = idr * (i1 - ist), rj = jdr * (j1 - jst);
    for (int k = 0; k < (hw > 1 ? 6 : 3); ++k)
      if (ri == ci[k] && rj == cj[k]) return ecs_corner(a, X, c, k);
  }
  int r, pos;
  bool along_i;
  if (j1 < 1) { r = 1 - j1; pos = i1; along_i = true; }
  else if (j1 > N) { r = j1 - N; pos = i1; along_i = true; }
  else if (i1 < 1) { r = 1 - i1; pos = j1; along_i = false; }
  else { r = i1 - N; pos = j1; along_i = false; }
  const int b = __ldg(&a.ecs_ind[(r - 1) * (N + 4) + (pos + 1)]);
  auto G = [&](int k) { return along_i ? X(k, j1) : X(i1, k); };
  double s = ecs_wt(a, -1, pos, r) * G(b - 1);
  s = s + ecs_wt(a, 0, pos, r) * G(b);
  s = s + ecs_wt(a, 1, pos, r) * G(b + 1);
  s = s + ecs_wt(a, 2, pos, r) * G(b + 2);
  return s;
}

__device__ __forceinline__ double ecs_o_at(const CArgsT<double>& a, const double* f, int p, int i1, int j1, int hw) {
  return ecs_o_at_x(a, [&](int x, int y) { return ecs_x(a, f, p, x, y); }, i1, j1, hw);
}

// The A-grid vector halo's exchanged component c (0 u, 1 v) at (i1, j1): the
// 'full' vector exchange (the neighbour's components turned to this panel's
// axes, tables 4 and 5), then the map TM of its edge, depth and position
// (ecs_halo_vec_a_mod.f90:55-156).  Contravariant components.
__device__ __forceinline__ double ecs_vx(const CArgsT<double>& a, const double* u, const double* v, int p, int c,
                                         int i1, int j1) {
  const int N = a.N;
  if (i1 >= 1 && i1 <= N && j1 >= 1 && j1 <= N) return (c == 0 ? u : v)[at(a.g, p, i1 - 1, j1 - 1)];
  int e, d, k;
  if (j1 < 1) { e = 0; d = 1 - j1; k = i1; }
  else if (j1 > N) { e = 1; d = j1 - N; k = i1; }
  else if (i1 < 1) { e = 2; d = 1 - i1; k = j1; }
  else { e = 3; d = i1 - N; k = j1; }
  const int side = e == 0 ? 2 : e == 1 ? 3 : e == 2 ? 0 : 1;
  const double eu = halo_at(a, 4, side, p, d, k - 1, u, v);
  const double ev = halo_at(a, 5, side, p, d, k - 1, v, u);
  const double* T = a.ecs_tm + (((e * kHaloDepth) + (d - 1)) * N + (k - 1)) * 4;
  return c == 0 ? __ldg(T) * eu + __ldg(T + 1) * ev : __ldg(T + 2) * eu + __ldg(T + 3) * ev;
}

__device__ __forceinline__ double ecs_v_at(const CArgsT<double>& a, const double* u, const double* v, int p, int c,
                                           int i1, int j1, int hw) {
  return ecs_o_at_x(a, [&](int x, int y) { return ecs_vx(a, u, v, p, c, x, y); }, i1, j1, hw);
}

// gradient_a2_ecs (gradient/grad_a2_mod.f90:19-69): the central difference of
// the cell values with the ECS_O halo of width 1 at the panel edges, gx, gy
// covariant at the centres.
__global__ void __launch_bounds__(256) grad_a2_kernel(const __grid_constant__ CArgsT<double> a) {
  const int N = a.N;
  SWM_C_INDEX(N, N)
  const double* f = a.ke_in;
  auto E = [&](int i1, int j1) {
    return (i1 >= 1 && i1 <= N && j1 >= 1 && j1 <= N) ? f[at(a.g, p, i1 - 1, j1 - 1)] : ecs_o_at(a, f, p, i1, j1, 1);
  };
  const int i1 = i + 1, j1 = j + 1, e = at(a.g, p, i, j);
  a.o1[e] = 0.5 * (E(i1 + 1, j1) - E(i1 - 1, j1)) / a.hxa;
  a.o2[e] = 0.5 * (E(i1, j1 + 1) - E(i1, j1 - 1)) / a.hxa;
}

// gradient_c2_ecs (gradient/grad_c2_ecs_mod.f90:95-144): the first
// differences of the cell values onto the faces, with the ECS_O halo of width
// 1 beyond the panel edges; gx on the x-faces, gy on the y-faces.
__global__ void __launch_bounds__(256) grad_c2_kernel(const __grid_constant__ CArgsT<double> a) {
  const int N = a.N;
  SWM_C_INDEX(N + 1, N + 1)
  const double* f = a.ke_in;
  auto E = [&](int i1, int j1) {
    return (i1 >= 1 && i1 <= N && j1 >= 1 && j1 <= N) ? f[at(a.g, p, i1 - 1, j1 - 1)] : ecs_o_at(a, f, p, i1, j1, 1);
  };
  const int i1 = i + 1, j1 = j + 1, e = at(a.g, p, i, j);
  if (j < N) a.o1[e] = (E(i1, j1) - E(i1 - 1, j1)) / a.hxa;
  if (i < N) a.o2[e] = (E(i1, j1) - E(i1, j1 - 1)) / a.hxa;
}

// The extended tiles of the ECS_O halo of width hw: ext[p][j][i] for the
// 1-based (i - hw + 1, j - hw + 1), width N + 2 hw.
__global__ void __launch_bounds__(256) ecs_ext_kernel(const __grid_constant__ CArgsT<double> a, int hw,
                                                      double* ext) {
  const int N = a.N, W = N + 2 * hw;
  SWM_C_INDEX(W, W)
  const int i1 = i + 1 - hw, j1 = j + 1 - hw;
  const double* f = a.ke_in;
  const double v = (i1 >= 1 && i1 <= N && j1 >= 1 && j1 <= N) ? f[at(a.g, p, i1 - 1, j1 - 1)]
                                                              : ecs_o_at(a, f, p, i1, j1, hw);
  ext[((long long)p * W + j) * W + i] = v;
}

// divergence_a2_ecs (divergence/div_a2_mod.f90:19-72): the ecs_A_vec halo of
// width 1, then (J u(i+1) - J u(i-1) + J v(j+1) - J v(j-1)) / (2 J hx a) with
// J on the extended grid lines beyond the edges.
__global__ void __launch_bounds__(256) div_a2_kernel(const __grid_constant__ CArgsT<double> a) {
  const int N = a.N;
  SWM_C_INDEX(N, N)
  const double *u = a.u, *v = a.v;
  const int i1 = i + 1, j1 = j + 1;
  auto in = [&](int x, int y) { return x >= 1 && x <= N && y >= 1 && y <= N; };
  auto J = [&](int x, int y) {
    if (in(x, y)) return a.Jp[at(a.g, p, x - 1, y - 1)];
    const int e = y < 1 ? 0 : y > N ? 1 : x < 1 ? 2 : 3;
    return __ldg(&a.ecs_jr[e * N + ((e < 2 ? x : y) - 1)]);
  };
  auto U = [&](int x, int y) { return in(x, y) ? u[at(a.g, p, x - 1, y - 1)] : ecs_v_at(a, u, v, p, 0, x, y, 1); };
  auto V = [&](int x, int y) { return in(x, y) ? v[at(a.g, p, x - 1, y - 1)] : ecs_v_at(a, u, v, p, 1, x, y, 1); };
  a.o1[at(a.g, p, i, j)] = (J(i1 + 1, j1) * U(i1 + 1, j1) - J(i1 - 1, j1) * U(i1 - 1, j1) +
                            J(i1, j1 + 1) * V(i1, j1 + 1) - J(i1, j1 - 1) * V(i1, j1 - 1)) /
                           (2.0 * J(i1, j1) * a.hxa);
}

// The extended tiles of the ecs_A_vec halo of width hw (both components).
__global__ void __launch_bounds__(256) ecs_vec_ext_kernel(const __grid_constant__ CArgsT<double> a, int hw,
                                                          double* eu, double* ev) {
  const int N = a.N, W = N + 2 * hw;
  SWM_C_INDEX(W, W)
  const int i1 = i + 1 - hw, j1 = j + 1 - hw;
  const bool in = i1 >= 1 && i1 <= N && j1 >= 1 && j1 <= N;
  const long long o = ((long long)p * W + j) * W + i;
  eu[o] = in ? a.u[at(a.g, p, i1 - 1, j1 - 1)] : ecs_v_at(a, a.u, a.v, p, 0, i1, j1, hw);
  ev[o] = in ? a.v[at(a.g, p, i1 - 1, j1 - 1)] : ecs_v_at(a, a.u, a.v, p, 1, i1, j1, hw);
}

// ------------------------------------------------------------------ ECS_xy
// The ECS_xy halo of the corner (node) mesh, the Ah grid's points
// (equiang_cs/ecs_halo_xy_mod.f90:38-217): n = N+1 nodes a side; the
// exchange places the neighbour's copy of the shared edge row in the first
// halo layer, so halo row r comes from the neighbour's row r+1 layers out.
// The reference works in place; each value is restated from the exchanged
// values here (the same steps as the oracle's ecs_xy_panel).
constexpr int kXyRows = kHaloDepth - 1;

__device__ __forceinline__ double xy_x(const CArgsT<double>& a, const double* f, int p, int i1, int j1) {
  const int n = a.N + 1;
  if (i1 >= 1 && i1 <= n && j1 >= 1 && j1 <= n) return f[at(a.g, p, i1 - 1, j1 - 1)];
  int side, d, k;
  if (i1 < 1) { side = 0; d = 1 - i1; k = j1 - 1; }
  else if (i1 > n) { side = 1; d = i1 - n; k = j1 - 1; }
  else if (j1 < 1) { side = 2; d = 1 - j1; k = i1 - 1; }
  else { side = 3; d = j1 - n; k = i1 - 1; }
  return halo_at(a, 3, side, p, d, k, f, f);
}

// The extended value at (i1, j1) of the ECS_xy halo of width hw: the panel's
// edge nodes averaged with their copies (three at the cube corners), the
// corner diagonals from the two strips beyond the duplicates, and the halo
// rows interpolated from the neighbour's rows with the diagonals at their ends.
__device__ double xy_at(const CArgsT<double>& a, const double* f, int p, int i1, int j1, int hw) {
  const int n = a.N + 1, ni = n + 2 * kXyRows;
  auto X = [&](int x, int y) { return xy_x(a, f, p, x, y); };
  const bool in_i = i1 >= 1 && i1 <= n, in_j = j1 >= 1 && j1 <= n;
  if (in_i && in_j) {
    const bool ei = i1 == 1 || i1 == n, ej = j1 == 1 || j1 == n;
    if (!ei && !ej) return X(i1, j1);
    if (i1 == 1 && j1 == 1) return (X(1, 1) + X(1, 0) + X(0, 1)) / 3.0;
    if (i1 == n && j1 == 1) return (X(n, 1) + X(n, 0) + X(n + 1, 1)) / 3.0;
    if (i1 == n && j1 == n) return (X(n, n) + X(n, n + 1) + X(n + 1, n)) / 3.0;
    if (i1 == 1 && j1 == n) return (X(1, n) + X(0, n) + X(1, n + 1)) / 3.0;
    if (j1 == 1) return 0.5 * (X(i1, 1) + X(i1, 0));
    if (j1 == n) return 0.5 * (X(i1, n) + X(i1, n + 1));
    if (i1 == 1) return 0.5 * (X(1, j1) + X(0, j1));
    return 0.5 * (X(n, j1) + X(n + 1, j1));
  }
  auto D = [&](int c, int r) {
    if (c == 0) return 0.5 * (X(-r, 1) + X(1, -r));
    if (c == 1) return 0.5 * (X(n + r + 1, 1) + X(n, -r));
    if (c == 2) return 0.5 * (X(n + r + 1, n) + X(n, n + r + 1));
    return 0.5 * (X(1, n + r + 1) + X(-r, n));
  };
  for (int r = 1; r <= hw; ++r) {
    if (i1 == 1 - r && j1 == 1 - r) return D(0, r);
    if (i1 == n + r && j1 == 1 - r) return D(1, r);
    if (i1 == n + r && j1 == n + r) return D(2, r);
    if (i1 == 1 - r && j1 == n + r) return D(3, r);
  }
  auto lo = [&](int r) { return max(1 - hw, 2 - r); };
  auto hi = [&](int r) { return min(n + hw, n + r - 1); };
  auto itp = [&](int r, int k, auto S) {
    const int b = __ldg(&a.xy_ind[(r - 1) * ni + (k - 1 + kXyRows)]);
    const double* w = a.xy_w + ((r - 1) * ni + (k - 1 + kXyRows)) * 4;
    double s = __ldg(w) * S(b - 1);
    s = s + __ldg(w + 1) * S(b);
    s = s + __ldg(w + 2) * S(b + 1);
    s = s + __ldg(w + 3) * S(b + 2);
    return s;
  };
  if (j1 < 1 && i1 >= lo(1 - j1) && i1 <= hi(1 - j1)) {
    const int r = 1 - j1;
    return itp(r, i1, [&](int k) { return k == 1 ? D(0, r) : k == n ? D(1, r) : X(k, -r); });
  }
  if (j1 > n && i1 >= lo(j1 - n) && i1 <= hi(j1 - n)) {
    const int r = j1 - n;
    return itp(r, i1, [&](int k) { return k == 1 ? D(3, r) : k == n ? D(2, r) : X(k, n + r + 1); });
  }
  if (i1 < 1) {
    const int r = 1 - i1;
    return itp(r, j1, [&](int k) { return k == 1 ? D(0, r) : k == n ? D(3, r) : X(-r, k); });
  }
  const int r = i1 - n;
  return itp(r, j1, [&](int k) { return k == 1 ? D(1, r) : k == n ? D(2, r) : X(n + r + 1, k); });
}

// The extended tiles of the ECS_xy halo of width hw (W = n + 2 hw).
__global__ void __launch_bounds__(256) xy_ext_kernel(const __grid_constant__ CArgsT<double> a, int hw, double* ext) {
  const int n = a.N + 1, W = n + 2 * hw;
  SWM_C_INDEX(W, W)
  ext[((long long)p * W + j) * W + i] = xy_at(a, a.ke_in, p, i + 1 - hw, j + 1 - hw, hw);
}

// laplace_ch_halo2 / laplace_ch_halo4 (laplace/laplace_ch_halo_mod.f90:15-179)
// on the extended tiles of the ECS_xy halo (width 1 / 3), before the edge
// sync.  mt holds the ECS metric (J, Qi11, Qi12, Qi22) of the extended node
// grid at the nodes, at (i+1/2, j) and at (i, j+1/2): three tables of
// (n + 2 kXyRows)^2 points, panel-independent.
template <int ORDER>
__global__ void __launch_bounds__(256) laplace_ch_kernel(const __grid_constant__ CArgsT<double> a, const double* ext,
                                                         const double* mt, double* out) {
  constexpr int hw = ORDER == 2 ? 1 : 3;
  const int n = a.N + 1, W = n + 2 * hw, M = n + 2 * kXyRows;
  SWM_C_INDEX(n, n)
  const double hx = a.hx0, sc = a.rad;
  const double* E = ext + (long long)p * W * W;
  auto F = [&](int x, int y) { return E[(y - 1 + hw) * W + (x - 1 + hw)]; };
  auto T = [&](int t, int x, int y, int c) { return __ldg(&mt[(((long long)t * M + (y - 1 + kXyRows)) * M + (x - 1 + kXyRows)) * 4 + c]); };
  auto Jxy = [&](int x, int y) { return T(0, x, y, 0); };
  auto Q2xy = [&](int x, int y) { return T(0, x, y, 2); };
  auto Jy = [&](int x, int y) { return T(1, x, y, 0); };    // mesh_y: (i+1/2, j)
  auto Q1y = [&](int x, int y) { return T(1, x, y, 1); };
  auto Jx = [&](int x, int y) { return T(2, x, y, 0); };    // mesh_x: (i, j+1/2)
  auto Q3x = [&](int x, int y) { return T(2, x, y, 3); };
  const int i1 = i + 1, j1 = j + 1;
  double v;
  if (ORDER == 2) {
    auto gx = [&](int x, int y) { return (F(x + 1, y) - F(x, y)) / (hx * sc); };
    auto gy = [&](int x, int y) { return (F(x, y + 1) - F(x, y)) / (hx * sc); };
    auto gxt = [&](int x, int y) {
      const double gh0 = 0.5 * (gy(x, y - 1) + gy(x, y)) * Q2xy(x, y) * Jxy(x, y);
      const double gh1 = 0.5 * (gy(x + 1, y - 1) + gy(x + 1, y)) * Q2xy(x + 1, y) * Jxy(x + 1, y);
      return Q1y(x, y) * gx(x, y) + 0.5 * (gh0 + gh1) / Jy(x, y);
    };
    // the reference's pairing: Qi12 at (i+1, j) with J at (i, j+1)
    // (laplace_ch_halo_mod.f90:87), kept for parity
    auto gyt = [&](int x, int y) {
      const double gh0 = 0.5 * (gx(x - 1, y) + gx(x, y)) * Q2xy(x, y) * Jxy(x, y);
      const double gh1 = 0.5 * (gx(x - 1, y + 1) + gx(x, y + 1)) * Q2xy(x + 1, y) * Jxy(x, y + 1);
      return Q3x(x, y) * gy(x, y) + 0.5 * (gh0 + gh1) / Jx(x, y);
    };
    v = (Jy(i1, j1) * gxt(i1, j1) - Jy(i1 - 1, j1) * gxt(i1 - 1, j1) + Jx(i1, j1) * gyt(i1, j1) -
         Jx(i1, j1 - 1) * gyt(i1, j1 - 1)) /
        (Jxy(i1, j1) * hx * sc);
  } else {
    auto gx = [&](int x, int y) {
      return (-F(x + 2, y) + 27.0 * F(x + 1, y) - 27.0 * F(x, y) + F(x - 1, y)) / (24.0 * hx * sc);
    };
    auto gy = [&](int x, int y) {
      return (-F(x, y + 2) + 27.0 * F(x, y + 1) - 27.0 * F(x, y) + F(x, y - 1)) / (24.0 * hx * sc);
    };
    auto gxh = [&](int x, int y) {
      return (-gx(x - 2, y) + 9.0 * gx(x - 1, y) + 9.0 * gx(x, y) - gx(x + 1, y)) / 16.0 * Q2xy(x, y) * Jxy(x, y);
    };
    auto gyh = [&](int x, int y) {
      return (-gy(x, y - 2) + 9.0 * gy(x, y - 1) + 9.0 * gy(x, y) - gy(x, y + 1)) / 16.0 * Q2xy(x, y) * Jxy(x, y);
    };
    auto gxt = [&](int x, int y) {
      return Q1y(x, y) * gx(x, y) + (-gyh(x + 2, y) + 9.0 * gyh(x + 1, y) + 9.0 * gyh(x, y) - gyh(x - 1, y)) / (16.0 * Jy(x, y));
    };
    auto gyt = [&](int x, int y) {
      return Q3x(x, y) * gy(x, y) + (-gxh(x, y + 2) + 9.0 * gxh(x, y + 1) + 9.0 * gxh(x, y) - gxh(x, y - 1)) / (16.0 * Jx(x, y));
    };
    const double dx = (-Jy(i1 + 1, j1) * gxt(i1 + 1, j1) + 27.0 * Jy(i1, j1) * gxt(i1, j1) -
                       27.0 * Jy(i1 - 1, j1) * gxt(i1 - 1, j1) + Jy(i1 - 2, j1) * gxt(i1 - 2, j1)) /
                      24.0;
    const double dy = (-Jx(i1, j1 + 1) * gyt(i1, j1 + 1) + 27.0 * Jx(i1, j1) * gyt(i1, j1) -
                       27.0 * Jx(i1, j1 - 1) * gyt(i1, j1 - 1) + Jx(i1, j1 - 2) * gyt(i1, j1 - 2)) /
                      24.0;
    v = (dx / hx + dy / hx) / (Jxy(i1, j1) * sc);
  }
  out[at(a.g, p, i, j)] = v;
}

// Centre pass: the kinetic energy (KE_Cgrid_mod.f90:60-75) plus g (h + hs)
// (operator_swm_mod.f90:84-85), the divergence (div_c_sbp42_mod.f90:67-107,
// div_c2_mod.f90:97-177) and the Coriolis terms at the centres
// (coriolis_Cgrid_mod.f90:98-118).
template <int ORD, class T>
__global__ void __launch_bounds__(256) centre_b_kernel(const __grid_constant__ CArgsT<T> a) {
  constexpr int W = ORD == 42 ? 4 : 2;
  const int N = a.N;
  SWM_C_INDEX(N, N)
  const FieldGeom& g = a.g;
  const COpsT<T>& o = a.ops;
  const int e = at(g, p, i, j);
  const int row = at(g, p, 0, j), col = at(g, p, i, 0);
  // h of this point, read before the RK epilogue of stages 2 and 3 writes
  // the new h in place over it
  const T hh = (a.flags & (F_ADDGH | F_COR)) ? a.h[e] : T(0.0);
  if (a.flags & F_KE) {
    T ke = (stag_at<W, T>(o.wi2c, a.KEu + row, 1, N, i) + stag_at<W, T>(o.wi2c, a.KEv + col, g.P, N, j)) * a.rJp[e];
    if (a.flags & F_ADDGH) ke = ke + a.grav * hh + a.grav * (a.hs ? a.hs[e] : T(0.0));
    a.KE[e] = ke;
  }
  if (a.flags & F_DIV) {
    T dx, dy;
    if (ORD == 21) {
      const T* hu = a.hu_in;
      const T* hv = a.hv_in;
      auto u = [&](int ii) { return ii < 0 ? halo_at(a, 1, 0, p, 1, j, hu, hv)
                                            : ii > N ? halo_at(a, 1, 1, p, 1, j, hu, hv) : hu[row + ii]; };
      auto v = [&](int jj) { return jj < 0 ? halo_at(a, 2, 2, p, 1, i, hv, hu)
                                            : jj > N ? halo_at(a, 2, 3, p, 1, i, hv, hu) : hv[col + jj * g.P]; };
      auto Ju = [&](int ii) { return a.Ju[row + ii]; };
      auto Jv = [&](int jj) { return a.Jv[col + jj * g.P]; };
      if (i == 0) dx = Ju(1) * u(1) - Ju(0) * (T(0.25) * u(0) + T(0.75) * u(-1));
      else if (i == 1) dx = Ju(2) * u(2) - Ju(1) * u(1) - T(0.25) * Ju(0) * (u(0) - u(-1));
      else if (i == N - 2) dx = Ju(N - 1) * u(N - 1) - Ju(N - 2) * u(N - 2) + T(0.25) * Ju(N) * (u(N) - u(N + 1));
      else if (i == N - 1) dx = Ju(N) * (T(0.75) * u(N + 1) + T(0.25) * u(N)) - Ju(N - 1) * u(N - 1);
      else dx = Ju(i + 1) * u(i + 1) - Ju(i) * u(i);
      if (j == 0) dy = Jv(1) * v(1) - Jv(0) * (T(0.25) * v(0) + T(0.75) * v(-1));
      else if (j == 1) dy = Jv(2) * v(2) - Jv(1) * v(1) - T(0.25) * Jv(0) * (v(0) - v(-1));
      else if (j == N - 2) dy = Jv(N - 1) * v(N - 1) - Jv(N - 2) * v(N - 2) + T(0.25) * Jv(N) * (v(N) - v(N + 1));
      else if (j == N - 1) dy = Jv(N) * (T(0.75) * v(N + 1) + T(0.25) * v(N)) - Jv(N - 1) * v(N - 1);
      else dy = Jv(j + 1) * v(j + 1) - Jv(j) * v(j);
    } else {
      const T* gu = a.Gu;
      const T* gv = a.Gv;
      dx = stag_at<W, T>(o.di2c, gu + row, 1, N, i);
      dy = stag_at<W, T>(o.di2c, gv + col, g.P, N, j);
      if (i < o.np) dx = dx + T(0.5) * o.pen_c[i] * (gu[row] - halo_at(a, 1, 0, p, 1, j, gu, gv));
      if (i >= N - o.np) dx = dx + T(0.5) * o.pen_c[N - 1 - i] * (halo_at(a, 1, 1, p, 1, j, gu, gv) - gu[row + N]);
      if (j < o.np) dy = dy + T(0.5) * o.pen_c[j] * (gv[col] - halo_at(a, 2, 2, p, 1, i, gv, gu));
      if (j >= N - o.np)
        dy = dy + T(0.5) * o.pen_c[N - 1 - j] * (halo_at(a, 2, 3, p, 1, i, gv, gu) - gv[col + N * g.P]);
    }
    const T dv = (dx + dy) * a.rJpha[e];
    if (a.flags & F_SEP) a.o1[e] = dv;
    else rk_put(a, 0, e, -T(1.0) * dv);
  }
  if (a.flags & F_COR) {
    const T gup = stag_at<W, T>(o.wi2c, a.Gu + row, 1, N, i);
    const T gvp = stag_at<W, T>(o.wi2c, a.Gv + col, g.P, N, j);
    const T cp = stag_at<W, T>(o.wi2c, a.fu + row, 1, N, i);  // the curl at the centre
    const T q = (a.fp[e] + cp) / hh;  // one division per point
    a.cup[e] = q * gvp;
    a.cvp[e] = -q * gup;
  }
}

// covariant gradient of the centre field f at face i (gradient_c_sbp42,
// grad_c_sbp42_mod.f90:44-139; gradient_c_sbp21, grad_c2_ecs_mod.f90:234-293)
// along a line: F(k) for 0 <= k < N from the panel, else the o halo.
template <int ORD, class T, class Fn>
__device__ __forceinline__ T grad_line(const CArgsT<T>& a, int N, int i, Fn F) {
  const COpsT<T>& o = a.ops;
  if (ORD == 21) {
    const T dx1 = a.dx1;
    if (i == 0) return (T(0.5) * F(1) + T(0.5) * F(0) - T(1.5) * F(-1) + T(0.5) * F(-2)) * dx1;
    if (i == N) return (-T(0.5) * F(N - 2) - T(0.5) * F(N - 1) + T(1.5) * F(N) - T(0.5) * F(N + 1)) * dx1;
    return (F(i) - F(i - 1)) * dx1;
  } else {
    const StagOpT<T>& D = o.dc2i;
    const T dx1 = a.dx1;
    if (i <= 3) {
      T s = T(0.0);
      for (int m = 0; m < D.last[i]; ++m) s += D.Ql[i * D.nw + m] * F(m);
      T gv = s * dx1;
      if (i == 0) {
        const T dh =
            (o.proj[0] * (F(0) - F(-1)) + o.proj[1] * (F(1) - F(-2)) + o.proj[2] * (F(2) - F(-3))) * dx1;
        gv = gv + T(0.5) * dh / o.sq1;
      }
      return gv;
    }
    if (i <= N - 4) {
      T s = T(0.0);
#pragma unroll
      for (int t = 0; t < 4; ++t) s += F(i - 2 + t) * D.Qin[t];
      return s * dx1;
    }
    const int r = N - i;
    T s = T(0.0);
    for (int m = 0; m < D.last[r]; ++m) s += D.Ql[r * D.nw + m] * F(N - 1 - m);
    T gv = -s * dx1;
    if (i == N) {
      const T dh =
          (o.proj[0] * (F(N) - F(N - 1)) + o.proj[1] * (F(N + 1) - F(N - 2)) + o.proj[2] * (F(N + 2) - F(N - 3))) * dx1;
      gv = gv + T(0.5) * dh / o.sq1;
    }
    return gv;
  }
}

// The gradient at an interior face (4 <= i <= N-4 at 4/2, 1 <= i <= N-1 at
// 2/1), f0 pointing at the centre value F(i), st the stride along the line:
// the interior rows of grad_line with direct loads, in the same order.
template <int ORD, class T>
__device__ __forceinline__ bool grad_interior(int N, int i) {
  return ORD == 21 ? (i >= 1 && i <= N - 1) : (i >= 4 && i <= N - 4);
}
template <int ORD, class T>
__device__ __forceinline__ T grad_in(const CArgsT<T>& a, const T* __restrict__ f0, int st) {
  if (ORD == 21) return (f0[0] - f0[-st]) * a.dx1;
  const T* q = a.ops.dc2i.Qin;
  T s = T(0.0);
  s += f0[-2 * st] * q[0];
  s += f0[-st] * q[1];
  s += f0[0] * q[2];
  s += f0[st] * q[3];
  return s * a.dx1;
}

// Face pass: the gradient of the kinetic energy and the Coriolis term
// interpolated from the centres (interpolator_p2uv_mod.f90:98-115), combined
// into the u, v tendencies (operator_swm_mod.f90:95-96).
template <int ORD, class T>
__global__ void __launch_bounds__(256) faces_b_kernel(const __grid_constant__ CArgsT<T> a) {
  constexpr int W = ORD == 42 ? 4 : 2;
  const int N = a.N;
  SWM_C_INDEX(N + 1, N + 1)
  const FieldGeom& g = a.g;
  const int e = at(g, p, i, j);
  const T* f = a.ke_in;
  if (j < N) {  // u point
    T gx = T(0.0), cu = T(0.0);
    if (a.flags & F_GRAD) {
      const T* rowp = f + at(g, p, 0, j);
      if (grad_interior<ORD, T>(N, i))
        gx = grad_in<ORD, T>(a, rowp + i, 1);
      else
        gx = grad_line<ORD, T>(a, N, i, [&](int k) {
          return k < 0 ? halo_at(a, 0, 0, p, -k, j, f, f) : k >= N ? halo_at(a, 0, 1, p, k - N + 1, j, f, f) : rowp[k];
        });
    }
    if (a.flags & F_COR) cu = stag_at<W, T>(a.ops.wc2i, a.cup + at(g, p, 0, j), 1, N + 1, i);
    if (a.flags & F_SEP) a.o1[e] = (a.flags & F_GRAD) ? gx : cu;
    else rk_put(a, 1, e, -T(1.0) * gx + T(1.0) * cu);
  }
  if (i < N) {  // v point
    T gy = T(0.0), cv = T(0.0);
    if (a.flags & F_GRAD) {
      const T* colp = f + at(g, p, i, 0);
      if (grad_interior<ORD, T>(N, j))
        gy = grad_in<ORD, T>(a, colp + j * g.P, g.P);
      else
        gy = grad_line<ORD, T>(a, N, j, [&](int k) {
          return k < 0 ? halo_at(a, 0, 2, p, -k, i, f, f)
                       : k >= N ? halo_at(a, 0, 3, p, k - N + 1, i, f, f) : colp[k * g.P];
        });
    }
    if (a.flags & F_COR) cv = stag_at<W, T>(a.ops.wc2i, a.cvp + at(g, p, i, 0), g.P, N + 1, j);
    if (a.flags & F_SEP) a.o2[e] = (a.flags & F_GRAD) ? gy : cv;
    else rk_put(a, 2, e, -T(1.0) * gy + T(1.0) * cv);
  }
}

// SBP_C quadrature (quadrature_factory_mod.f90:90-160, sbp_quadrature_mod.f90:
// 21-40): sum of f J hx^2 Ax(i) Ay(j) over a mesh, in fixed-order partials.
__global__ void __launch_bounds__(kMassThreads) mass_partial_kernel(FieldGeom g, int nx, int ny, const double* f,
                                                                     const double* J, const double* ax,
                                                                     const double* ay, double hx2, double* part) {
  __shared__ double sh[kMassThreads];
  const long long total = 6LL * nx * ny;
  double acc = 0.0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k % nx);
    const long long r = k / nx;
    const int j = (int)(r % ny), p = (int)(r / ny);
    const long long e = (long long)p * g.ps + (long long)j * g.P + i;
    acc += f[e] * J[e] * hx2 * ax[i] * ay[j];
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// A mesh field in the dense host layout (i fastest, then j, then panel) to
// or from its pitched device field: FP64, or split into / joined from the
// FP32 (hi, lo) pair as the Ah-grid transfers do.
__global__ void cunpack_kernel(FieldGeom g, int nx, int ny, const double* __restrict__ src, double* d64,
                               float* hi, float* lo) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 6LL * nx * ny) return;
  const int i = (int)(k % nx);
  const long long r = k / nx;
  const int j = (int)(r % ny), p = (int)(r / ny);
  const long long e = (long long)p * g.ps + (long long)j * g.P + i;
  const double x = src[k];
  if (lo) {
    const float h = (float)x;
    hi[e] = h;
    lo[e] = (float)(x - (double)h);
  } else {
    d64[e] = x;
  }
}

__global__ void cpack_kernel(FieldGeom g, int nx, int ny, const double* __restrict__ d64, const float* hi,
                             const float* lo, double* __restrict__ dst) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 6LL * nx * ny) return;
  const int i = (int)(k % nx);
  const long long r = k / nx;
  const int j = (int)(r % ny), p = (int)(r / ny);
  const long long e = (long long)p * g.ps + (long long)j * g.P + i;
  dst[k] = lo ? (double)hi[e] + (double)lo[e] : d64[e];
}

__global__ void mass_final_kernel(const double* part, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < n; ++k) s += part[k];
    *out = s;
  }
}

}  // namespace

struct CGrid {
  FieldGeom g{};
  int N = 0, order = 42, L = 0;
  double hx = 0.0, radius = 1.0, grav = 9.80616;
  COps ops{};
  COpsT<float> ops32{};
  COps ops21{};             // the 2/1 operators of the hyperdiffusion (any order)
  COpsT<float> ops21_32{};
  double* met = nullptr;   // M_COUNT fields
  float* met32 = nullptr;  // their FP32 copies (contexts of the FP32 form)
  double* wk = nullptr;    // W_COUNT fields
  double* rk = nullptr;    // Y, Kb, acc: 3 fields each
  // hyperdiffusion (allocated on first use): kDiffFields work fields, the two
  // side streams of its branches and the fork / join events
  double* dw = nullptr;
  cudaStream_t bs[2] = {nullptr, nullptr};
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  int* halo = nullptr;
  double* ecs_w = nullptr;  // ECS_O weights [2][N+4][4]
  int* ecs_ind = nullptr;   // ECS_O stencil bases [2][N+4]
  double* ecs_tm = nullptr;  // ecs_A_vec maps [4][kHaloDepth][N][4]
  double* ecs_jr = nullptr;  // J on the first ring beyond each edge [4][N]
  double* ext = nullptr;    // extended tiles of the halo entry points (allocated on first use)
  int ext_hw = 0;
  double* xy_w = nullptr;   // ECS_xy weights [kXyRows][n + 2 kXyRows][4]
  int* xy_ind = nullptr;    // ECS_xy stencil bases
  double* xy_ext = nullptr; // ECS_xy extended tiles (width up to kXyRows, on first use)
  double* xy_mt = nullptr;  // metric tables of laplace_ch (on first use)
  double* wts = nullptr;   // quadrature weights: centres (N), interfaces (N+1)
  double* part = nullptr;  // kMassBlocks partial sums
  double* metric(int k) const { return met + (long long)k * g.fs; }
  double* work(int k) const { return wk + (long long)k * g.fs; }
};

namespace {

template <class T>
const T* metric_t(const CGrid* c, int k) {
  if constexpr (sizeof(T) == 8) return c->met ? c->metric(k) : nullptr;
  else return c->met32 ? c->met32 + (long long)k * c->g.fs : nullptr;
}

// Kernel arguments in precision T: FP64 metric and work fields, or the
// FP32 metric copies and the same work buffers read as floats.  ord 0: the
// operators of the context's order; 21: the 2/1 ones.
template <class T>
CArgsT<T> base_args(const CGrid* c, int ord = 0) {
  CArgsT<T> a{};
  a.g = c->g; a.N = c->N; a.L = c->L;
  a.grav = T(c->grav);
  a.ord = ord ? ord : c->order;
  const bool o21 = a.ord == 21;
  if constexpr (sizeof(T) == 8) a.ops = o21 ? c->ops21 : c->ops;
  else a.ops = o21 ? c->ops21_32 : c->ops32;
  a.dx1 = T(1.0 / (c->radius * c->hx));
  auto M = [&](int k) { return metric_t<T>(c, k); };
  auto Wk = [&](int k) { return c->wk ? reinterpret_cast<T*>(c->work(k)) : nullptr; };
  a.Jp = M(M_JP); a.fp = M(M_FP); a.rJp = M(M_RJP);
  a.rJpha = M(M_RJPHA); a.JQi2p = M(M_JQI2P);
  a.Ju = M(M_JU); a.Qi1u = M(M_QI1U); a.rJu = M(M_RJU);
  a.Jv = M(M_JV); a.Qi3v = M(M_QI3V); a.rJv = M(M_RJV);
  a.rJqha = M(M_RJQHA); a.rJuha = M(M_RJUHA); a.rJvha = M(M_RJVHA);
  a.halo = c->halo;
  a.ecs_w = c->ecs_w; a.ecs_ind = c->ecs_ind; a.hxa = c->hx * c->radius;
  a.ecs_tm = c->ecs_tm; a.ecs_jr = c->ecs_jr;
  a.xy_w = c->xy_w; a.xy_ind = c->xy_ind; a.hx0 = c->hx; a.rad = c->radius;
  a.Ap = Wk(W_AP); a.Bp = Wk(W_BP); a.ut = Wk(W_UT); a.vt = Wk(W_VT);
  a.hu = Wk(W_HU); a.hv = Wk(W_HV); a.Gu = Wk(W_GU); a.Gv = Wk(W_GV);
  a.KEu = Wk(W_KEU); a.KEv = Wk(W_KEV); a.curl = Wk(W_CURL);
  a.fu = Wk(W_FU); a.KE = Wk(W_KE);
  a.cup = Wk(W_CUP); a.cvp = Wk(W_CVP);
  return a;
}

dim3 grid_for(int nx, int ny) { return dim3((nx + 31) / 32, (ny + 7) / 8, 6); }
const dim3 kBlock(32, 8, 1);

#define SWM_C_LAUNCH(name, kern, nx, ny)                                                              \
  template <class T>                                                                                   \
  cudaError_t name(const CGrid* c, const CArgsT<T>& a, cudaStream_t st) {                             \
    if (a.ord == 42) kern<42, T><<<grid_for(nx, ny), kBlock, 0, st>>>(a);                             \
    else kern<21, T><<<grid_for(nx, ny), kBlock, 0, st>>>(a);                                         \
    return cudaGetLastError();                                                                         \
  }
SWM_C_LAUNCH(run_centre_a, centre_a_kernel, c->N, c->N)
SWM_C_LAUNCH(run_faces_a, faces_a_kernel, c->N + 1, c->N + 1)
SWM_C_LAUNCH(run_curl, curl_kernel, c->N + 1, c->N + 1)
SWM_C_LAUNCH(run_w2uv, w2uv_kernel, c->N + 1, c->N)
SWM_C_LAUNCH(run_centre_b, centre_b_kernel, c->N, c->N)
SWM_C_LAUNCH(run_faces_b, faces_b_kernel, c->N + 1, c->N + 1)
SWM_C_LAUNCH(run_gperp, gperp_kernel, c->N + 1, c->N + 1)
#undef SWM_C_LAUNCH

#define CKE(call)                               \
  do {                                          \
    cudaError_t e_ = (call);                    \
    if (e_ != cudaSuccess) return e_;           \
  } while (0)

// One right-hand side of the state (h, u, v) with the epilogue of a.mode.
template <class T>
cudaError_t rhs(const CGrid* c, CArgsT<T> a, const T* in, cudaStream_t st) {
  const long long fs = c->g.fs;
  a.h = in; a.u = in + fs; a.v = in + 2 * fs;
  a.flags = F_CO | F_MF | F_G | F_KE | (c->order == 21 ? F_WFLUX : 0);
  CKE(run_centre_a(c, a, st));
  CKE(run_faces_a(c, a, st));
  CKE(run_curl(c, a, st));
  // the corner sync of the curl rides in w2uv's reads (its only reader here)
  a.curl_in = a.curl;
  a.flags = F_QSYNC;
  CKE(run_w2uv(c, a, st));
  a.hu_in = a.hu; a.hv_in = a.hv;
  a.flags = F_KE | F_ADDGH | F_DIV | F_COR;
  CKE(run_centre_b(c, a, st));
  a.ke_in = a.KE;
  a.flags = F_GRAD | F_COR;
  return run_faces_b(c, a, st);
}

// ------------------------------------------------------------------ host
// ECS metric on the prototype face (ecs_metric_mod.f90:326-478) and the
// panel frame (ecs_proto2realface with the identity rotation).
struct MetricAt {
  double J, qi1, qi2, qi3, q1, q2, q3;
};
MetricAt metric_at(double al, double be) {
  const double ta = std::tan(al), tb = std::tan(be);
  const double sg = std::sqrt(1.0 + ta * ta + tb * tb);
  const double s4 = sg * sg * sg * sg;
  MetricAt m;
  m.J = (1.0 + ta * ta) * (1.0 + tb * tb) / (sg * sg * sg);
  m.qi1 = sg * sg / (1.0 + ta * ta);
  m.qi2 = sg * sg * ta * tb / ((1.0 + ta * ta) * (1.0 + tb * tb));
  m.qi3 = sg * sg / (1.0 + tb * tb);
  // the covariant metric tensor (ecs_Q, ecs_metric_mod.f90:401-419)
  m.q1 = (1.0 + ta * ta) * (1.0 + ta * ta) * (1.0 + tb * tb) / s4;
  m.q2 = -(1.0 + ta * ta) * (1.0 + tb * tb) * ta * tb / s4;
  m.q3 = (1.0 + ta * ta) * (1.0 + tb * tb) * (1.0 + tb * tb) / s4;
  return m;
}

double coriolis_at(int p, double al, double be, double omega, const double ax[3]) {
  const double ta = std::tan(al), tb = std::tan(be);
  const double d = std::sqrt(1.0 + ta * ta + tb * tb);
  const double v[3] = {ta / d, tb / d, 1.0 / d};
  double w[3];
  for (int k = 0; k < 3; ++k) w[k] = cube::kEX[p][k] * v[0] + cube::kEY[p][k] * v[1] - cube::kN[p][k] * v[2];
  const double nn = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  const double pr = (ax[0] * w[0] + ax[1] * w[1] + ax[2] * w[2]) / nn;
  return 2.0 * omega * pr;  // calc_coriolis_parameter (coriolis_factory_mod.f90:151-172)
}

// Cross-halo table of mesh T (0 o, 1 u, 2 v, 3 q): create_o_points_halo_
// exchange, create_symm_halo_vec_exchange_U/V_points and create_xy_points_
// halo_exchange (exchange_factory_mod.f90:13-156, 317-617) with the component
// swap and signs of buffer_mod.f90:278-475, for the halo points the C-grid
// SBP operators read: left / right layers along the panel rows, bottom / top
// layers along the columns, depth 1..3.  The neighbour's points are placed
// with the receiving mesh's point counts, so the duplicated edge faces of u
// (v) fill the first x (y) layer and the duplicated edge points of q its
// first layers.
// Tables 4 and 5 are the u and v components of an A-grid vector, both on the
// centres (the 'full' vector exchange of create_o_points_halo_exchange, with
// the same component swap and signs).
constexpr int kHaloMeshes = 6;
bool build_halo(int N, const FieldGeom& g, std::vector<int>& tab, std::string& why) {
  const int L = N + 1;
  const int dims[kHaloMeshes][2] = {{N, N}, {N + 1, N}, {N, N + 1}, {N + 1, N + 1}, {N, N}, {N, N}};
  tab.assign((size_t)kHaloMeshes * 4 * 6 * kHaloDepth * L, -1);
  for (int T = 0; T < kHaloMeshes; ++T) {
    const int nx = dims[T][0], ny = dims[T][1];
    for (int p = 0; p < 6; ++p)
      for (int q = 0; q < 6; ++q) {
        if (q == p) continue;
        int istep, jstep, dim_i;
        cube::orientation(p, q, istep, jstep, dim_i);  // (receiver, sender)
        const bool vec = T == 1 || T == 2 || T == 4 || T == 5;
        const bool first = T == 1 || T == 4;  // the u component
        const bool swap = vec && !dim_i;
        const int S = !swap ? T : T == 1 ? 2 : T == 2 ? 1 : T == 4 ? 5 : 4;
        int sign = 1;
        if (vec) sign = first ? (dim_i ? istep : jstep) : (dim_i ? jstep : istep);
        const int snx = dims[S][0], sny = dims[S][1];
        for (int js = 1; js <= sny; ++js)
          for (int is = 1; is <= snx; ++is) {
            int it, jt;
            cube::map_index(q, is, js, p, nx, ny, it, jt);
            int s = -1, d = 0, k = 0;
            if (it <= 0 && it > -kHaloDepth && jt >= 1 && jt <= ny) { s = 0; d = 1 - it; k = jt - 1; }
            else if (it > nx && it <= nx + kHaloDepth && jt >= 1 && jt <= ny) { s = 1; d = it - nx; k = jt - 1; }
            else if (jt <= 0 && jt > -kHaloDepth && it >= 1 && it <= nx) { s = 2; d = 1 - jt; k = it - 1; }
            else if (jt > ny && jt <= ny + kHaloDepth && it >= 1 && it <= nx) { s = 3; d = jt - ny; k = it - 1; }
            if (s < 0) continue;
            const long long src = (long long)q * g.ps + (long long)(js - 1) * g.P + (is - 1);
            if (src * 4 + 3 > INT32_MAX) { why = "C-grid halo table: field too large"; return false; }
            tab[((((size_t)T * 4 + s) * 6 + p) * kHaloDepth + (d - 1)) * L + k] =
                (int)(src * 4 + (swap ? 2 : 0) + (sign < 0 ? 1 : 0));
          }
      }
    for (int p = 0; p < 6; ++p)
      for (int s = 0; s < 4; ++s)
        for (int d = 1; d <= kHaloDepth; ++d)
          for (int k = 0; k < (s < 2 ? ny : nx); ++k)
            if (tab[((((size_t)T * 4 + s) * 6 + p) * kHaloDepth + (d - 1)) * L + k] < 0) {
              why = "C-grid halo table: a halo point without a sender";
              return false;
            }
  }
  return true;
}

// co2contra (to_co false) or the contra2co transform of co2contra_c_sbp*_new
// (to_co true, co2contra_Cgrid_mod.f90:135-203): the same two passes, with
// the covariant metric J Q12, Q11, Q22 in place of the inverse one.
template <class T>
cudaError_t transform(const CGrid* c, CArgsT<T> a, const T* x, const T* y, T* xo, T* yo, bool to_co,
                      cudaStream_t st) {
  if (to_co) {
    a.JQi2p = metric_t<T>(c, M_JQ2P);
    a.Qi1u = metric_t<T>(c, M_Q1U);
    a.Qi3v = metric_t<T>(c, M_Q3V);
  }
  a.u = x; a.v = y; a.ut = xo; a.vt = yo;
  a.flags = F_CO | F_WUT;
  CKE(run_centre_a(c, a, st));
  return run_faces_a(c, a, st);
}

// Work fields of the hyperdiffusion: the results L(L(h)), the curl part
// (u, v) and the divergence part (u, v), then per branch (curl, divergence,
// h) the centre scratch of the transforms (2), two face pairs (4) and one
// centre or corner field.
constexpr int kDiffResults = 5, kDiffBranch = 7, kDiffFields = kDiffResults + 3 * kDiffBranch;

// The C-grid hyperdiffusion of operator_swm_diff_t (operator_swm_diff_mod.f90
// :25-46) with the 2/1 operators the factory uses at any order
// (hordiff_factory_mod.f90:53-139, 196-247), on the state in (h, u, v):
//   curl part  contra2co grad_perp curl contra2co grad_perp curl (u, v)
//   div part   grad div co2contra grad div co2contra (u, v)
//   h          L(L(h)), L = div co2contra grad
// The three chains are independent: they run as three branches (the
// context stream and two side streams, forked and joined with events, so a
// captured step becomes a three-branch graph), each on its own work fields.
// Then the combine pass on the context stream (mode 0 tendency into out, 1 /
// 2 Euler step on out = the state, 2 with the FP32 low part lo).
template <class T>
cudaError_t diffusion(const CGrid* c, const Topology& tp, T* edge, int parts, double c4uv, double c4h, const T* in,
                      T* out, float* lo, double dt, int mode, cudaStream_t st) {
  if (!c->dw) return cudaErrorInvalidValue;  // cgrid_diffusion_prepare first
  const long long fs = c->g.fs;
  auto F = [&](int k) { return reinterpret_cast<T*>(c->dw + (long long)k * fs); };
  T *TH = F(0), *TU = F(1), *TV = F(2), *U3 = F(3), *V3 = F(4);
  const T *h = in, *u = in + fs, *v = in + 2 * fs;
  struct Branch {
    CArgsT<T> a;  // with this branch's transform scratch
    T *X1, *Y1, *X2, *Y2, *S;
    cudaStream_t st;
  };
  const cudaStream_t side[2] = {c->bs[0], c->bs[1]};
  auto branch = [&](int b) {
    const int o = kDiffResults + kDiffBranch * b;
    Branch r{base_args<T>(c, 21), F(o + 2), F(o + 3), F(o + 4), F(o + 5), F(o + 6), b ? side[b - 1] : st};
    r.a.Ap = F(o);
    r.a.Bp = F(o + 1);
    return r;
  };
  auto div = [&](const Branch& B, const T* x, const T* y, T* o) {
    CArgsT<T> b = B.a;
    b.hu_in = x; b.hv_in = y; b.o1 = o;
    b.flags = F_DIV | F_SEP;
    return run_centre_b(c, b, B.st);
  };
  auto grad = [&](const Branch& B, const T* f, T* gx, T* gy) {
    CArgsT<T> b = B.a;
    b.ke_in = f; b.o1 = gx; b.o2 = gy;
    b.flags = F_GRAD | F_SEP;
    return run_faces_b(c, b, B.st);
  };
  auto curl = [&](const Branch& B, const T* x, const T* y, T* q) {
    CArgsT<T> b = B.a;
    b.u = x; b.v = y; b.curl = q;
    CKE(run_curl(c, b, B.st));
    return launch_sync_scalar_t<T>(c->g, tp, q, edge, B.st);
  };
  auto gperp = [&](const Branch& B, const T* q, T* gu, T* gv) {
    CArgsT<T> b = B.a;
    b.curl_in = q; b.o1 = gu; b.o2 = gv;
    return run_gperp(c, b, B.st);
  };
  auto xf = [&](const Branch& B, const T* x, const T* y, T* xo, T* yo, bool to_co) {
    return transform(c, B.a, x, y, xo, yo, to_co, B.st);
  };
  const Branch bc = branch(0), bd = branch(1), bh = branch(2);
  CKE(cudaEventRecord(c->ev[0], st));
  CKE(cudaStreamWaitEvent(bd.st, c->ev[0], 0));
  CKE(cudaStreamWaitEvent(bh.st, c->ev[0], 0));
  if (parts & 2) {
    CKE(curl(bc, u, v, bc.S));
    CKE(gperp(bc, bc.S, bc.X1, bc.Y1));
    CKE(xf(bc, bc.X1, bc.Y1, bc.X2, bc.Y2, true));
    CKE(curl(bc, bc.X2, bc.Y2, bc.S));
    CKE(gperp(bc, bc.S, bc.X1, bc.Y1));
    CKE(xf(bc, bc.X1, bc.Y1, TU, TV, true));
  }
  if (parts & 1) {
    CKE(xf(bd, u, v, bd.X1, bd.Y1, false));
    CKE(div(bd, bd.X1, bd.Y1, bd.S));
    CKE(grad(bd, bd.S, bd.X2, bd.Y2));
    CKE(xf(bd, bd.X2, bd.Y2, bd.X1, bd.Y1, false));
    CKE(div(bd, bd.X1, bd.Y1, bd.S));
    CKE(grad(bd, bd.S, U3, V3));
  }
  const T* f = h;
  for (int rep = 0; rep < 2; ++rep) {
    CKE(grad(bh, f, bh.X1, bh.Y1));
    CKE(xf(bh, bh.X1, bh.Y1, bh.X2, bh.Y2, false));
    CKE(div(bh, bh.X2, bh.Y2, rep ? TH : bh.S));
    f = bh.S;
  }
  CKE(cudaEventRecord(c->ev[1], bd.st));
  CKE(cudaEventRecord(c->ev[2], bh.st));
  CKE(cudaStreamWaitEvent(st, c->ev[1], 0));
  CKE(cudaStreamWaitEvent(st, c->ev[2], 0));
  diff_combine_kernel<T><<<grid_for(c->N + 1, c->N + 1), kBlock, 0, st>>>(
      c->g, c->N, parts, T(c4uv), T(c4h), TH, TU, TV, U3, V3, mode, dt, out, lo);
  return cudaGetLastError();
}

// Weights of the ECS_O halo (equiang_cs/ecs_halo_factory_mod.f90:164-196,
// init_halo_interp) for rows 1, 2 and positions -1..N+2: the virtual point's
// angle on the neighbour's grid line, atan(tan(alpha_i) / tan(pi/4 +
// (r - 1/2) hx)), its stencil base and the four cubic Lagrange weights.
// False if a stencil the edges use would leave the panel.
bool build_ecs_weights(int N, double hx, std::vector<double>& w, std::vector<int>& ind) {
  const int ni = N + 4;
  w.assign((size_t)2 * ni * 4, 0.0);
  ind.assign((size_t)2 * ni, 0);
  for (int r = 1; r <= 2; ++r)
    for (int i = -1; i <= N + 2; ++i) {
      const double zb = 0.25 * kPiC + (r - 0.5) * hx;
      double za = -0.25 * kPiC + (i - 0.5) * hx;
      za = std::atan(std::tan(za) / std::tan(zb));
      const int b = (int)std::floor((za + 0.25 * kPiC - 0.5 * hx) / hx) + 1;
      const double x = (za + 0.25 * kPiC) / hx - (b - 0.5);
      double* q = &w[((size_t)(r - 1) * ni + (i + 1)) * 4];
      q[0] = -x * (x - 1.0) * (x - 2.0) / 6.0;
      q[1] = (x + 1.0) * (x - 1.0) * (x - 2.0) / 2.0;
      q[2] = -(x + 1.0) * x * (x - 2.0) / 2.0;
      q[3] = (x + 1.0) * x * (x - 1.0) / 6.0;
      ind[(size_t)(r - 1) * ni + (i + 1)] = b;
      const bool used = r == 1 ? (i >= 2 && i <= N - 1) : (i >= 1 && i <= N);
      if (used && (b - 1 < 1 || b + 2 > N)) return false;
    }
  return true;
}

// The equiangular gnomonic map on the prototype face: the point r = (X, Y,
// 1) / sigma with X = tan(alpha), Y = tan(beta), sigma^2 = 1 + X^2 + Y^2, the
// covariant basis a1 = dr/dalpha, a2 = dr/dbeta and the contravariant basis
// b1, b2 from the inverse metric (the same geometry as ecs_metric_mod.f90:
// 326-478).
struct EcsFrame {
  double r[3], a1[3], a2[3], b1[3], b2[3];
};
EcsFrame ecs_frame(double al, double be) {
  const double X = std::tan(al), Y = std::tan(be);
  const double s2 = 1.0 + X * X + Y * Y, sg = std::sqrt(s2), s3 = s2 * sg;
  const double ca = (1.0 + X * X) / s3, cb = (1.0 + Y * Y) / s3;
  const double qi1 = s2 / (1.0 + X * X), qi2 = s2 * X * Y / ((1.0 + X * X) * (1.0 + Y * Y)), qi3 = s2 / (1.0 + Y * Y);
  EcsFrame f;
  const double r[3] = {X / sg, Y / sg, 1.0 / sg};
  const double a1[3] = {ca * (1.0 + Y * Y), -ca * X * Y, -ca * X};
  const double a2[3] = {-cb * X * Y, cb * (1.0 + X * X), -cb * Y};
  for (int k = 0; k < 3; ++k) {
    f.r[k] = r[k]; f.a1[k] = a1[k]; f.a2[k] = a2[k];
    f.b1[k] = qi1 * a1[k] + qi2 * a2[k];
    f.b2[k] = qi2 * a1[k] + qi3 * a2[k];
  }
  return f;
}

// The maps of the A-grid vector halo (ecs_halo_vec_a_factory_mod.f90:108-170):
// for edge e (bottom, top, left, right), depth d and position i, the
// neighbour's point in the canonical placement across that edge (a rotation
// of the prototype face about a coordinate axis), its covariant basis turned
// into this face's frame, projected on this face's contravariant basis at the
// same point of the extended grid.  Also J on the first ring beyond each edge.
void build_ecs_vec_tables(int N, double hx, std::vector<double>& tm, std::vector<double>& jr) {
  tm.assign((size_t)4 * kHaloDepth * N * 4, 0.0);
  jr.assign((size_t)4 * N, 0.0);
  const int ab_shift[4] = {0, 0, 1, 1}, b_sign[4] = {1, -1, 1, -1};
  auto rot = [](int e, const double* v, double* o) {
    switch (e) {
      case 0: o[0] = v[0]; o[1] = -v[2]; o[2] = v[1]; break;   // about x, edge 1
      case 1: o[0] = v[0]; o[1] = v[2]; o[2] = -v[1]; break;   // about x, edge 2
      case 2: o[0] = -v[2]; o[1] = v[1]; o[2] = v[0]; break;   // about y, edge 3
      default: o[0] = v[2]; o[1] = v[1]; o[2] = -v[0]; break;  // about y, edge 4
    }
  };
  auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
  for (int e = 0; e < 4; ++e)
    for (int d = 1; d <= kHaloDepth; ++d)
      for (int i = 1; i <= N; ++i) {
        const double al = -0.25 * kPiC + (i - 0.5) * hx;
        const double be = b_sign[e] * (0.25 * kPiC - (d - 0.5) * hx);
        const EcsFrame S = ab_shift[e] ? ecs_frame(be, al) : ecs_frame(al, be);
        double a1s[3], a2s[3], r[3];
        rot(e, S.a1, a1s);
        rot(e, S.a2, a2s);
        rot(e, S.r, r);
        const EcsFrame T = ecs_frame(std::atan(r[0] / r[2]), std::atan(r[1] / r[2]));
        double* q = &tm[(((size_t)e * kHaloDepth + (d - 1)) * N + (i - 1)) * 4];
        q[0] = dot(a1s, T.b1); q[1] = dot(a2s, T.b1); q[2] = dot(a1s, T.b2); q[3] = dot(a2s, T.b2);
      }
  for (int k = 1; k <= N; ++k) {
    const double in = -0.25 * kPiC + ((k - 1) + 0.5) * hx;
    const double lo = -0.25 * kPiC + (-1 + 0.5) * hx, hi = -0.25 * kPiC + (N + 0.5) * hx;
    jr[0 * N + (k - 1)] = metric_at(in, lo).J;
    jr[1 * N + (k - 1)] = metric_at(in, hi).J;
    jr[2 * N + (k - 1)] = metric_at(lo, in).J;
    jr[3 * N + (k - 1)] = metric_at(hi, in).J;
  }
}

// Weights of the ECS_xy halo (ecs_halo_factory_mod.f90:198-228,
// init_halo_xy_interp) for rows 1..kXyRows and positions 1-kXyRows ..
// n+kXyRows: the node's angle on the neighbour's grid line r layers out, the
// stencil base clamped to [2, n-2] and the cubic Lagrange weights.
void build_xy_weights(int N, double hx, std::vector<double>& w, std::vector<int>& ind) {
  const int n = N + 1, ni = n + 2 * kXyRows;
  w.assign((size_t)kXyRows * ni * 4, 0.0);
  ind.assign((size_t)kXyRows * ni, 0);
  for (int r = 1; r <= kXyRows; ++r)
    for (int i = 1 - kXyRows; i <= n + kXyRows; ++i) {
      const double zb = 0.25 * kPiC + r * hx;
      double za = -0.25 * kPiC + (i - 1.0) * hx;
      za = std::atan(std::tan(za) / std::tan(zb));
      const int b = std::min(std::max(2, (int)std::floor((za + 0.25 * kPiC) / hx) + 1), n - 2);
      const double x = (za + 0.25 * kPiC) / hx - (b - 1.0);
      double* q = &w[((size_t)(r - 1) * ni + (i - 1 + kXyRows)) * 4];
      q[0] = -x * (x - 1.0) * (x - 2.0) / 6.0;
      q[1] = (x + 1.0) * (x - 1.0) * (x - 2.0) / 2.0;
      q[2] = -(x + 1.0) * x * (x - 2.0) / 2.0;
      q[3] = (x + 1.0) * x * (x - 1.0) / 6.0;
      ind[(size_t)(r - 1) * ni + (i - 1 + kXyRows)] = b;
    }
}

}  // namespace

namespace {

// tables_only: the cross-halo tables and ECS weights alone (no metric, work
// or RK fields), for the ECS halos of another grid's context.
int create_impl(const FieldGeom& g, int N, int order, double radius, double grav, double omega, const double axis[3],
                bool fp32, bool tables_only, cudaStream_t st, CGrid** out, std::string& why) {
  *out = nullptr;
  if (order != 21 && order != 42) { why = "C-grid SBP order must be 21 or 42"; return 1; }
  if (N < 12) { why = "C grid needs N >= 12"; return 1; }
  CGrid* c = new CGrid;
  c->g = g; c->N = N; c->order = order; c->L = N + 1;
  c->hx = (0.25 * kPiC - (-0.25 * kPiC)) / (double)N;
  c->radius = radius; c->grav = grav;
  fill_ops(order, c->ops);
  c->ops32 = ops_cast<float>(c->ops);
  fill_ops(21, c->ops21);
  c->ops21_32 = ops_cast<float>(c->ops21);
  const double an = std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
  const double ax[3] = {axis[0] / an, axis[1] / an, axis[2] / an};
  std::vector<int> tab;
  if (!build_halo(N, g, tab, why)) { delete c; return 1; }
  std::vector<double> ew;
  std::vector<int> eind;
  if (!build_ecs_weights(N, c->hx, ew, eind)) { why = "ECS_O halo stencils leave the panel"; delete c; return 1; }
  std::vector<double> etm, ejr;
  build_ecs_vec_tables(N, c->hx, etm, ejr);
  std::vector<double> xyw;
  std::vector<int> xyind;
  build_xy_weights(N, c->hx, xyw, xyind);
  std::vector<double> w(2 * (size_t)N + 1, 1.0);
  {
    // SBP_C42 / SBP_C21 edge weights (D42_A_centers / _interfaces, D21_*)
    const std::vector<double> ec = order == 42 ? std::vector<double>{13.0 / 12.0, 7.0 / 8.0, 25.0 / 24.0, 1.0}
                                               : std::vector<double>{1.0, 1.0};
    const std::vector<double> ei = order == 42 ? std::vector<double>{7.0 / 18.0, 9.0 / 8.0, 1.0, 71.0 / 72.0, 1.0}
                                               : std::vector<double>{0.5, 1.0};
    auto fill = [](double* a, int n, const std::vector<double>& e) {
      const int ne = (int)e.size();
      for (int k = 0; k < std::min(ne, n); ++k) a[k] = e[k];
      for (int k = std::max(n - ne, 0); k < n; ++k) a[k] = e[n - 1 - k];
    };
    fill(w.data(), N, ec);
    fill(w.data() + N, N + 1, ei);
  }
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t x) { if (e == cudaSuccess) e = x; return e == cudaSuccess; };
  const size_t fb = sizeof(double) * g.fs;
  if (!tables_only) {
    ok(cudaMalloc(&c->met, M_COUNT * fb));
    ok(cudaMalloc(&c->wk, W_COUNT * fb));
    ok(cudaMalloc(&c->rk, 9 * fb));
  }
  ok(cudaMalloc(&c->halo, sizeof(int) * tab.size()));
  ok(cudaMalloc(&c->ecs_w, sizeof(double) * ew.size()));
  ok(cudaMalloc(&c->ecs_ind, sizeof(int) * eind.size()));
  ok(cudaMalloc(&c->ecs_tm, sizeof(double) * etm.size()));
  ok(cudaMalloc(&c->ecs_jr, sizeof(double) * ejr.size()));
  ok(cudaMalloc(&c->xy_w, sizeof(double) * xyw.size()));
  ok(cudaMalloc(&c->xy_ind, sizeof(int) * xyind.size()));
  ok(cudaMalloc(&c->wts, sizeof(double) * w.size()));
  ok(cudaMalloc(&c->part, sizeof(double) * kMassBlocks));
  if (e == cudaSuccess) {
    // metric of the four meshes (mesh_factory_mod.f90:25-133: alpha =
    // alpha0 + (i - 1 + shift_i) hx, shift 1/2 at centres, 0 on faces and
    // corners), one field at a time through a host buffer
    std::vector<double> hm(tables_only ? 0 : g.fs, 0.0);
    for (int k = 0; k < (tables_only ? 0 : M_COUNT) && e == cudaSuccess; ++k) {
      std::fill(hm.begin(), hm.end(), 0.0);
      const int mesh = kMetricMesh[k];
      const bool ci = mesh == 0 || mesh == 2;  // centred in alpha
      const bool cj = mesh == 0 || mesh == 1;  // centred in beta
      const int nx = ci ? N : N + 1, ny = cj ? N : N + 1;
      for (int p = 0; p < 6; ++p)
        for (int j = 0; j < ny; ++j)
          for (int i = 0; i < nx; ++i) {
            const double al = -0.25 * kPiC + (i + (ci ? 0.5 : 0.0)) * c->hx;
            const double be = -0.25 * kPiC + (j + (cj ? 0.5 : 0.0)) * c->hx;
            const MetricAt m = metric_at(al, be);
            const double J = m.J, jha = J * c->hx * radius;
            double x;
            switch (k) {
              case M_QI2P: x = m.qi2; break;
              case M_FP: x = coriolis_at(p, al, be, omega, ax); break;
              case M_RJP: case M_RJU: case M_RJV: x = 1.0 / J; break;
              case M_RJPHA: case M_RJQHA: case M_RJUHA: case M_RJVHA: x = 1.0 / jha; break;
              case M_JQI2P: x = J * m.qi2; break;
              case M_QI1U: x = m.qi1; break;
              case M_QI3V: x = m.qi3; break;
              case M_JQ2P: x = J * m.q2; break;
              case M_Q1U: x = m.q1; break;
              case M_Q3V: x = m.q3; break;
              default: x = J; break;
            }
            hm[(size_t)p * g.ps + (size_t)j * g.P + i] = x;
          }
      ok(cudaMemcpy(c->met + (size_t)k * g.fs, hm.data(), fb, cudaMemcpyHostToDevice));
    }
    if (!tables_only) {
      ok(cudaMemsetAsync(c->wk, 0, W_COUNT * fb, st));
      ok(cudaMemsetAsync(c->rk, 0, 9 * fb, st));
    }
    ok(cudaMemcpyAsync(c->halo, tab.data(), sizeof(int) * tab.size(), cudaMemcpyHostToDevice, st));
    ok(cudaMemcpyAsync(c->ecs_w, ew.data(), sizeof(double) * ew.size(), cudaMemcpyHostToDevice, st));
    ok(cudaMemcpyAsync(c->ecs_ind, eind.data(), sizeof(int) * eind.size(), cudaMemcpyHostToDevice, st));
    ok(cudaMemcpyAsync(c->ecs_tm, etm.data(), sizeof(double) * etm.size(), cudaMemcpyHostToDevice, st));
    ok(cudaMemcpyAsync(c->ecs_jr, ejr.data(), sizeof(double) * ejr.size(), cudaMemcpyHostToDevice, st));
    ok(cudaMemcpyAsync(c->xy_w, xyw.data(), sizeof(double) * xyw.size(), cudaMemcpyHostToDevice, st));
    ok(cudaMemcpyAsync(c->xy_ind, xyind.data(), sizeof(int) * xyind.size(), cudaMemcpyHostToDevice, st));
    if (fp32 && !tables_only && ok(cudaMalloc(&c->met32, sizeof(float) * M_COUNT * g.fs)))
      ok(launch_to_f32(c->met, c->met32, (long long)M_COUNT * g.fs, st));  // rounded once
    ok(cudaMemcpyAsync(c->wts, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice, st));
    ok(cudaStreamSynchronize(st));  // the host buffers go out of scope
  }
  if (e != cudaSuccess) {
    why = std::string("C-grid setup: ") + cudaGetErrorString(e);
    cgrid_destroy(c);
    return e == cudaErrorMemoryAllocation ? 3 : 2;
  }
  *out = c;
  return 0;
}

}  // namespace

int cgrid_create(const FieldGeom& g, int N, int order, double radius, double grav, double omega, const double axis[3],
                 bool fp32, cudaStream_t st, CGrid** out, std::string& why) {
  return create_impl(g, N, order, radius, grav, omega, axis, fp32, false, st, out, why);
}

int cgrid_create_tables(const FieldGeom& g, int N, double radius, cudaStream_t st, CGrid** out, std::string& why) {
  const double axis[3] = {0.0, 0.0, 1.0};
  return create_impl(g, N, 42, radius, 0.0, 0.0, axis, false, true, st, out, why);
}

void cgrid_destroy(CGrid* c) {
  if (!c) return;
  for (void* p : {(void*)c->met, (void*)c->met32, (void*)c->wk, (void*)c->rk, (void*)c->dw, (void*)c->halo,
                  (void*)c->ecs_w, (void*)c->ecs_ind, (void*)c->ecs_tm, (void*)c->ecs_jr, (void*)c->ext,
                  (void*)c->xy_w, (void*)c->xy_ind, (void*)c->xy_ext, (void*)c->xy_mt, (void*)c->wts,
                  (void*)c->part})
    if (p) cudaFree(p);
  for (cudaStream_t s : c->bs)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : c->ev)
    if (e) cudaEventDestroy(e);
  delete c;
}

int cgrid_order(const CGrid* c) { return c->order; }

void cgrid_mesh_dims(const CGrid* c, int mesh, int* nx, int* ny) {
  const int N = c->N;
  *nx = (mesh == CMESH_U || mesh == CMESH_Q) ? N + 1 : N;
  *ny = (mesh == CMESH_V || mesh == CMESH_Q) ? N + 1 : N;
}

cudaError_t cgrid_co2contra(CGrid* c, const double* u, const double* v, double* ut, double* vt, cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.u = u; a.v = v; a.ut = ut; a.vt = vt;
  a.flags = F_CO | F_WUT;
  CKE(run_centre_a(c, a, st));
  return run_faces_a(c, a, st);
}

cudaError_t cgrid_massflux(CGrid* c, const double* h, const double* ut, const double* vt, double* hu, double* hv,
                           cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.h = h; a.ut_in = ut; a.vt_in = vt; a.hu = hu; a.hv = hv;
  a.flags = F_MF | F_WFLUX;
  return run_faces_a(c, a, st);
}

cudaError_t cgrid_ke(CGrid* c, const double* u, const double* v, const double* ut, const double* vt, double* ke,
                     cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.u = u; a.v = v; a.ut_in = ut; a.vt_in = vt; a.KE = ke;
  a.flags = F_KE;
  CKE(run_faces_a(c, a, st));
  return run_centre_b(c, a, st);
}

cudaError_t cgrid_grad(CGrid* c, const double* f, double* gx, double* gy, cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.ke_in = f; a.o1 = gx; a.o2 = gy;
  a.flags = F_GRAD | F_SEP;
  return run_faces_b(c, a, st);
}

cudaError_t cgrid_div(CGrid* c, const double* hu, const double* hv, double* div, cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.hu_in = hu; a.hv_in = hv; a.o1 = div;
  if (c->order == 42) {
    a.flags = F_G;
    CKE(run_faces_a(c, a, st));
  }
  a.flags = F_DIV | F_SEP;
  return run_centre_b(c, a, st);
}

cudaError_t cgrid_curl(CGrid* c, const Topology& tp, double* edge, const double* u, const double* v, double* curl,
                       cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.u = u; a.v = v; a.curl = curl;
  CKE(run_curl(c, a, st));
  return launch_sync_scalar(c->g, tp, curl, edge, st);
}

cudaError_t cgrid_coriolis(CGrid* c, const double* hu, const double* hv, const double* h, const double* curl,
                           double* cor_u, double* cor_v, cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.hu_in = hu; a.hv_in = hv; a.h = h; a.curl_in = curl;
  a.flags = F_G;
  CKE(run_faces_a(c, a, st));
  CKE(run_w2uv(c, a, st));
  a.flags = F_COR;
  CKE(run_centre_b(c, a, st));
  a.o1 = cor_u; a.o2 = cor_v;
  a.flags = F_COR | F_SEP;
  return run_faces_b(c, a, st);
}

cudaError_t cgrid_apply(CGrid* c, const Topology& tp, double* edge, const double* hs, const double* in, double* out,
                        cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.hs = hs;
  a.mode = 0;
  a.tend = out;
  return rhs(c, a, in, st);
}

cudaError_t cgrid_apply32(CGrid* c, const Topology& tp, float* edge, const float* hs, const float* in, float* out,
                          cudaStream_t st) {
  if (!c->met32) return cudaErrorInvalidValue;
  CArgsT<float> a = base_args<float>(c);
  a.hs = hs;
  a.mode = 0;
  a.tend = out;
  return rhs(c, a, in, st);
}

// The FP32 form: stage inputs are the state's high part (stage 1) or Y in
// FP32; the increments add up in acc and the last stage adds them to the
// (hi, lo) pair with an exact two-sum.  In-place safety as for FP64.
cudaError_t cgrid_rk4_32(CGrid* c, const Topology& tp, float* edge, const float* hs, float* hi, float* lo, double dt,
                         cudaStream_t st) {
  if (!c->met32) return cudaErrorInvalidValue;
  CArgsT<float> a = base_args<float>(c);
  a.hs = hs;
  a.dt = float(dt); a.hdt = float(0.5 * dt); a.c6 = float(dt / 6.0); a.c3 = float(dt / 3.0);
  a.y0 = hi;
  a.lo = lo;
  a.Y = reinterpret_cast<float*>(c->rk);
  a.acc = a.Y + 3 * c->g.fs;
  for (int s = 1; s <= 4; ++s) {
    a.mode = s;
    CKE(rhs(c, a, s == 1 ? static_cast<const float*>(hi) : a.Y, st));
  }
  return cudaSuccess;
}

// Stage 1 reads y0 and writes Y; stages 2 and 3 read Y and write Y in place;
// stage 4 reads Y and writes y0.  In place is safe: the passes that read the
// stage input at neighbouring points (centre_a, faces_a, curl) run before the
// two that write it (centre_b, faces_b), and those read only their own point
// of it, before writing it.
cudaError_t cgrid_rk4(CGrid* c, const Topology& tp, double* edge, const double* hs, double* y0, double dt,
                      cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.hs = hs;
  a.dt = dt; a.hdt = 0.5 * dt; a.c6 = dt / 6.0; a.c3 = dt / 3.0;
  a.y0 = y0;
  a.Y = c->rk;
  a.Kb = c->rk + 3 * c->g.fs;
  a.acc = c->rk + 6 * c->g.fs;
  for (int s = 1; s <= 4; ++s) {
    a.mode = s;
    CKE(rhs(c, a, s == 1 ? y0 : a.Y, st));
  }
  return cudaSuccess;
}

cudaError_t cgrid_unpack(CGrid* c, int mesh, const double* dense, void* field, float* lo, cudaStream_t st) {
  int nx, ny;
  cgrid_mesh_dims(c, mesh, &nx, &ny);
  const long long n = 6LL * nx * ny;
  cunpack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(c->g, nx, ny, dense, lo ? nullptr : (double*)field,
                                                              lo ? (float*)field : nullptr, lo);
  return cudaGetLastError();
}

cudaError_t cgrid_pack(CGrid* c, int mesh, const void* field, const float* lo, double* dense, cudaStream_t st) {
  int nx, ny;
  cgrid_mesh_dims(c, mesh, &nx, &ny);
  const long long n = 6LL * nx * ny;
  cpack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(c->g, nx, ny, lo ? nullptr : (const double*)field,
                                                            lo ? (const float*)field : nullptr, lo, dense);
  return cudaGetLastError();
}

cudaError_t cgrid_grad_perp(CGrid* c, const double* w, double* gu, double* gv, cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.curl_in = w; a.o1 = gu; a.o2 = gv;
  return run_gperp(c, a, st);
}

cudaError_t cgrid_contra2co(CGrid* c, const double* ut, const double* vt, double* u, double* v, cudaStream_t st) {
  return transform(c, base_args<double>(c), ut, vt, u, v, true, st);
}

cudaError_t cgrid_diffusion_prepare(CGrid* c) {
  if (c->dw) return cudaSuccess;
  cudaError_t e = cudaMalloc(&c->dw, sizeof(double) * kDiffFields * c->g.fs);
  if (e == cudaSuccess) e = cudaMemset(c->dw, 0, sizeof(double) * kDiffFields * c->g.fs);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();  // the context stream does not wait on the legacy one
  for (cudaStream_t& s : c->bs)
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  for (cudaEvent_t& ev : c->ev)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    // leave nothing half made: the next call retries from scratch
    if (c->dw) cudaFree(c->dw);
    c->dw = nullptr;
    for (cudaStream_t& s : c->bs) { if (s) cudaStreamDestroy(s); s = nullptr; }
    for (cudaEvent_t& ev : c->ev) { if (ev) cudaEventDestroy(ev); ev = nullptr; }
  }
  return e;
}

cudaError_t cgrid_diffusion(CGrid* c, const Topology& tp, double* edge, int parts, double c4uv, double c4h,
                            const double* in, double* out, cudaStream_t st) {
  if (in == out || parts < 1 || parts > 3) return cudaErrorInvalidValue;
  return diffusion<double>(c, tp, edge, parts, c4uv, c4h, in, out, nullptr, 0.0, 0, st);
}

cudaError_t cgrid_diffusion_step(CGrid* c, const Topology& tp, double* edge, int parts, double c4uv, double c4h,
                                 double* y0, double dt, cudaStream_t st) {
  if (parts < 1 || parts > 3) return cudaErrorInvalidValue;
  return diffusion<double>(c, tp, edge, parts, c4uv, c4h, y0, y0, nullptr, dt, 1, st);
}

cudaError_t cgrid_diffusion32(CGrid* c, const Topology& tp, float* edge, int parts, double c4uv, double c4h,
                              const float* in, float* out, cudaStream_t st) {
  if (!c->met32 || in == out || parts < 1 || parts > 3) return cudaErrorInvalidValue;
  return diffusion<float>(c, tp, edge, parts, c4uv, c4h, in, out, nullptr, 0.0, 0, st);
}

cudaError_t cgrid_diffusion_step32(CGrid* c, const Topology& tp, float* edge, int parts, double c4uv, double c4h,
                                   float* hi, float* lo, double dt, cudaStream_t st) {
  if (!c->met32 || parts < 1 || parts > 3) return cudaErrorInvalidValue;
  return diffusion<float>(c, tp, edge, parts, c4uv, c4h, hi, hi, lo, dt, 2, st);
}

cudaError_t cgrid_grad_a2_ecs(CGrid* c, const double* f, double* gx, double* gy, cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.ke_in = f; a.o1 = gx; a.o2 = gy;
  grad_a2_kernel<<<grid_for(c->N, c->N), kBlock, 0, st>>>(a);
  return cudaGetLastError();
}

// Scratch for the extended tiles of two fields of the widest halo asked for
// (the halo entry points are synchronous).
cudaError_t ext_scratch(CGrid* c, int halo_width, cudaStream_t st) {
  if (c->ext_hw >= halo_width) return cudaSuccess;
  const int W = c->N + 2 * halo_width;
  CKE(cudaStreamSynchronize(st));
  if (c->ext) cudaFree(c->ext);
  c->ext = nullptr;
  c->ext_hw = 0;
  CKE(cudaMalloc(&c->ext, sizeof(double) * 2 * 6 * (size_t)W * W));
  c->ext_hw = halo_width;
  return cudaSuccess;
}

cudaError_t cgrid_ecs_o_halo(CGrid* c, const double* f, int halo_width, double* ext_host, cudaStream_t st) {
  if (halo_width < 1 || halo_width > 2) return cudaErrorInvalidValue;
  const int W = c->N + 2 * halo_width;
  const size_t bytes = sizeof(double) * 6 * (size_t)W * W;
  CKE(ext_scratch(c, halo_width, st));
  CArgsT<double> a = base_args<double>(c);
  a.ke_in = f;
  ecs_ext_kernel<<<grid_for(W, W), kBlock, 0, st>>>(a, halo_width, c->ext);
  CKE(cudaGetLastError());
  CKE(cudaMemcpyAsync(ext_host, c->ext, bytes, cudaMemcpyDeviceToHost, st));
  return cudaStreamSynchronize(st);
}

cudaError_t cgrid_ecs_a_vec_halo(CGrid* c, const double* u, const double* v, int halo_width, double* eu_host,
                                 double* ev_host, cudaStream_t st) {
  if (halo_width < 1 || halo_width > 2) return cudaErrorInvalidValue;
  const int W = c->N + 2 * halo_width;
  const size_t n = 6 * (size_t)W * W;
  CKE(ext_scratch(c, halo_width, st));
  CArgsT<double> a = base_args<double>(c);
  a.u = u; a.v = v;
  ecs_vec_ext_kernel<<<grid_for(W, W), kBlock, 0, st>>>(a, halo_width, c->ext, c->ext + n);
  CKE(cudaGetLastError());
  CKE(cudaMemcpyAsync(eu_host, c->ext, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  CKE(cudaMemcpyAsync(ev_host, c->ext + n, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  return cudaStreamSynchronize(st);
}

// The ECS_xy extended tiles of width up to kXyRows, and the metric tables of
// laplace_ch (both allocated on first use; these entry points are synchronous
// on the host or enqueue after a one-time set-up).
cudaError_t xy_prepare(CGrid* c, bool metric, cudaStream_t st) {
  const int n = c->N + 1, W = n + 2 * kXyRows, M = n + 2 * kXyRows;
  if (!c->xy_ext) {
    CKE(cudaStreamSynchronize(st));
    CKE(cudaMalloc(&c->xy_ext, sizeof(double) * 6 * (size_t)W * W));
  }
  if (metric && !c->xy_mt) {
    // J, Qi11, Qi12, Qi22 at the nodes, at (i+1/2, j) and at (i, j+1/2) of
    // the extended node grid (1-based i, j from 1-kXyRows to n+kXyRows)
    std::vector<double> t((size_t)3 * M * M * 4);
    for (int k = 0; k < 3; ++k)
      for (int y = 1 - kXyRows; y <= n + kXyRows; ++y)
        for (int x = 1 - kXyRows; x <= n + kXyRows; ++x) {
          const double si = k == 1 ? x + 0.5 : x, sj = k == 2 ? y + 0.5 : y;
          const MetricAt m = metric_at(-0.25 * kPiC + (si - 1.0) * c->hx, -0.25 * kPiC + (sj - 1.0) * c->hx);
          double* q = &t[(((size_t)k * M + (y - 1 + kXyRows)) * M + (x - 1 + kXyRows)) * 4];
          q[0] = m.J; q[1] = m.qi1; q[2] = m.qi2; q[3] = m.qi3;
        }
    CKE(cudaStreamSynchronize(st));
    CKE(cudaMalloc(&c->xy_mt, sizeof(double) * t.size()));
    CKE(cudaMemcpy(c->xy_mt, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice));
  }
  return cudaSuccess;
}

cudaError_t cgrid_laplace_ch_prepare(CGrid* c, cudaStream_t st) { return xy_prepare(c, true, st); }

cudaError_t cgrid_ecs_xy_halo(CGrid* c, const double* f, int halo_width, double* ext_host, cudaStream_t st) {
  if (halo_width < 1 || halo_width > kXyRows) return cudaErrorInvalidValue;
  CKE(xy_prepare(c, false, st));
  const int W = c->N + 1 + 2 * halo_width;
  CArgsT<double> a = base_args<double>(c);
  a.ke_in = f;
  xy_ext_kernel<<<grid_for(W, W), kBlock, 0, st>>>(a, halo_width, c->xy_ext);
  CKE(cudaGetLastError());
  CKE(cudaMemcpyAsync(ext_host, c->xy_ext, sizeof(double) * 6 * (size_t)W * W, cudaMemcpyDeviceToHost, st));
  return cudaStreamSynchronize(st);
}

cudaError_t cgrid_laplace_ch(CGrid* c, const Topology& tp, double* edge, int order, const double* f, double* out,
                             cudaStream_t st) {
  if (order != 2 && order != 4) return cudaErrorInvalidValue;
  CKE(xy_prepare(c, true, st));
  const int hw = order == 2 ? 1 : 3, n = c->N + 1, W = n + 2 * hw;
  CArgsT<double> a = base_args<double>(c);
  a.ke_in = f;
  xy_ext_kernel<<<grid_for(W, W), kBlock, 0, st>>>(a, hw, c->xy_ext);
  CKE(cudaGetLastError());
  if (order == 2) laplace_ch_kernel<2><<<grid_for(n, n), kBlock, 0, st>>>(a, c->xy_ext, c->xy_mt, out);
  else laplace_ch_kernel<4><<<grid_for(n, n), kBlock, 0, st>>>(a, c->xy_ext, c->xy_mt, out);
  CKE(cudaGetLastError());
  return launch_sync_scalar(c->g, tp, out, edge, st);  // the Ah scalar sync (laplace_factory_mod.f90:124)
}

cudaError_t cgrid_grad_c2_ecs(CGrid* c, const double* f, double* gx, double* gy, cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.ke_in = f; a.o1 = gx; a.o2 = gy;
  grad_c2_kernel<<<grid_for(c->N + 1, c->N + 1), kBlock, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t cgrid_div_a2_ecs(CGrid* c, const double* u, const double* v, double* div, cudaStream_t st) {
  CArgsT<double> a = base_args<double>(c);
  a.u = u; a.v = v; a.o1 = div;
  div_a2_kernel<<<grid_for(c->N, c->N), kBlock, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t cgrid_mass(CGrid* c, int mesh, const double* f, double* result, cudaStream_t st) {
  int nx, ny;
  cgrid_mesh_dims(c, mesh, &nx, &ny);
  const double* J = c->metric(mesh == CMESH_P ? M_JP : mesh == CMESH_U ? M_JU : mesh == CMESH_V ? M_JV : M_JQ);
  const double* wc = c->wts;
  const double* wi = c->wts + c->N;
  const double* ax = (mesh == CMESH_U || mesh == CMESH_Q) ? wi : wc;
  const double* ay = (mesh == CMESH_V || mesh == CMESH_Q) ? wi : wc;
  mass_partial_kernel<<<kMassBlocks, kMassThreads, 0, st>>>(c->g, nx, ny, f, J, ax, ay, c->hx * c->hx, c->part);
  mass_final_kernel<<<1, 32, 0, st>>>(c->part, kMassBlocks, result);
  return cudaGetLastError();
}

}  // namespace swm
