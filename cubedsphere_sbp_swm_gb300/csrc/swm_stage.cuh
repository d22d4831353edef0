// swm_stage.cuh -- fused vector-invariant RHS + RK4 stage epilogue, and the
// cube-edge pass that finishes the panel-boundary nodes.
//
// One RK stage is two launches:
//   stage_kernel  every node: co2contra, mass flux, KE, SBP grad(KE),
//                 curl = div(v/J, -u/J) and div(h u) with their one-sided
//                 boundary closures; interior nodes then get Coriolis, the
//                 tendency and the RK stage combination; panel-boundary nodes
//                 write their pre-sync (gx, gy, zeta, div) to the edge buffer.
//   edge_kernel   every panel-boundary node: the reference's cube-edge syncs
//                 (2-way average on edges, 3-way at cube corners, metric-
//                 weighted for the covariant gradient), then the same
//                 Coriolis / tendency / RK epilogue.
// Reference: operator_swm_mod.f90:61-113, rk4_mod.f90:20-42,
// sbp_operator_mod.f90:152-228, div_ah_sbp_mod.f90:46-96,
// grad_ah_sbp_mod.f90:51-88, curl_div_based_mod.f90:26-66,
// coriolis_colocated_mod.f90:79-103, halo_Ah_scalar_sync_mod.f90:38-93,
// ecs_Ah_vec_sync_mod.f90:62-125.
#pragma once

#include "swm_device.cuh"

namespace swm {

template <int ORD> struct Ord;
template <> struct Ord<21> { static constexpr int idx = 0, NE = 1, NW = 2, H = 1, RMAX = 1; };
template <> struct Ord<42> { static constexpr int idx = 1, NE = 4, NW = 6, H = 2, RMAX = 3; };
template <> struct Ord<43> { static constexpr int idx = 2, NE = 4, NW = 6, H = 2, RMAX = 5; };
template <> struct Ord<63> { static constexpr int idx = 3, NE = 6, NW = 9, H = 3, RMAX = 5; };

// Threads per CTA of the FP64 kernel = the most columns a unit reads.  Two
// warps: the column strips (own columns + 2*RMAX halo) then fill both warps,
// and every FP64 instruction runs on nearly full warps (GB300's FP64 pipe is
// the bound; at 128 threads a strip of N=384 left a warp with 6 live lanes).
constexpr int STAGE_BW = 64;
// Derived fields of the FP64 kernel's row rings: the y ring holds what the
// y stencils read along a column (2*RMAX+1 rows), the x ring what is read
// only on the row being finished (RMAX+1 rows: written RMAX rows ahead).
enum { RY_KE = 0, RY_U, RY_GV, RY_N };
enum { RX_V = 0, RX_GU, RX_JUT, RX_JVT, RX_N };

// Interior central difference with the antisymmetric coefficients of the
// order's interior stencil; fm(o) returns the value at offset o.
template <int ORD, class T, class F>
__device__ __forceinline__ T d_interior(F fm) {
  if constexpr (Ord<ORD>::H == 1) {
    return T(0.5) * (fm(1) - fm(-1));
  } else if constexpr (Ord<ORD>::H == 2) {
    return T(2.0 / 3.0) * (fm(1) - fm(-1)) + T(-1.0 / 12.0) * (fm(2) - fm(-2));
  } else {
    return T(3.0 / 4.0) * (fm(1) - fm(-1)) + T(-3.0 / 20.0) * (fm(2) - fm(-2)) +
           T(1.0 / 60.0) * (fm(3) - fm(-3));
  }
}

// SBP derivative at line index k of a line of n nodes; fa(m) returns the value
// at absolute line index m.
template <int ORD, class T, class FA>
__device__ __forceinline__ T d_line(int k, int n, FA fa) {
  constexpr int NE = Ord<ORD>::NE, NW = Ord<ORD>::NW, ID = Ord<ORD>::idx;
  if (k < NE) {
    T acc = T(0);
    const int last = c_sbp[ID].last[k];
#pragma unroll
    for (int m = 0; m < NW; ++m)
      if (m < last) acc += sbp_ql<T>(ID, k, m) * fa(m);
    return acc;
  } else if (k >= n - NE) {
    const int r = n - 1 - k;
    const int last = c_sbp[ID].last[r];
    T acc = T(0);
#pragma unroll
    for (int m = NW - 1; m >= 0; --m)
      if (m < last) acc += sbp_qr<T>(ID, r, m) * fa(n - 1 - m);
    return acc;
  }
  return d_interior<ORD, T>([&](int o) { return fa(k + o); });
}

// Tendency at one node from its (synced) derivative terms and the RK stage
// epilogue.  kk = (k_h, k_u, k_v).
template <class T>
__device__ __forceinline__ void stage_epilogue(const InstDev<T>& I, int mode, long long idx,
                                               T kh, T ku, T kv) {
  const long long fs = I.fs;
  const T kk[3] = {kh, ku, kv};
  if (mode == MODE_APPLY) {
#pragma unroll
    for (int c = 0; c < 3; ++c) I.out[c * fs + idx] = kk[c];
    return;
  }
  if constexpr (sizeof(T) == 8) {
    // FP64: the reference's order.  y = 1*v0 + c*k; w = v0 + dt/6 k1,
    // w += dt/3 k2, w += dt/3 k3, v0 = w + dt/6 k4 (rk4_mod.f90:28-40).
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long o = c * fs + idx;
      if (mode == MODE_RK1) {
        const T b = I.base[o];
        I.out[o] = T(1.0) * b + I.c_in * kk[c];
        I.acc[o] = b + I.c_acc * kk[c];
      } else if (mode == MODE_RK4) {
        I.base_out[o] = I.acc[o] + I.c_acc * kk[c];
      } else {
        I.out[o] = T(1.0) * I.base[o] + I.c_in * kk[c];
        I.acc[o] = I.acc[o] + I.c_acc * kk[c];
      }
    }
  } else {
    // FP32 compensated form: the stage increments accumulate separately from
    // the state (dacc = dt/6 k1 + dt/3 k2 + dt/3 k3), and the final stage adds
    // dacc + dt/6 k4 to the (hi, lo) state pair with an exact two-sum, so the
    // FP32 state keeps the low-order bits across steps.
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const long long o = c * fs + idx;
      if (mode == MODE_RK1) {
        I.out[o] = I.base[o] + I.c_in * kk[c];
        I.acc[o] = I.c_acc * kk[c];
      } else if (mode == MODE_RK4) {
        const T d = I.acc[o] + I.c_acc * kk[c];
        const T hi = I.base_out[o], lo = I.base_lo[o];
        const T t = lo + d;
        const T s = hi + t;
        const T bb = s - hi;
        const T err = (hi - (s - bb)) + (t - bb);
        I.base_out[o] = s;
        I.base_lo[o] = err;
      } else {
        I.out[o] = I.base[o] + I.c_in * kk[c];
        I.acc[o] = I.acc[o] + I.c_acc * kk[c];
      }
    }
  }
}

// The same epilogue with the RK inputs already loaded: rb = base (FP32 RK4:
// the state's high part), ra = running sum, rl = state's low part.
template <class T>
__device__ __forceinline__ void stage_epilogue_pre(const InstDev<T>& I, int mode, long long idx,
                                                   T kh, T ku, T kv, const T* rb, const T* ra,
                                                   const T* rl) {
  const long long fs = I.fs;
  const T kk[3] = {kh, ku, kv};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const long long o = c * fs + idx;
    if (mode == MODE_APPLY) {
      I.out[o] = kk[c];
    } else if (sizeof(T) == 8) {
      if (mode == MODE_RK1) {
        I.out[o] = T(1.0) * rb[c] + I.c_in * kk[c];
        I.acc[o] = rb[c] + I.c_acc * kk[c];
      } else if (mode == MODE_RK4) {
        I.base_out[o] = ra[c] + I.c_acc * kk[c];
      } else {
        I.out[o] = T(1.0) * rb[c] + I.c_in * kk[c];
        I.acc[o] = ra[c] + I.c_acc * kk[c];
      }
    } else {
      if (mode == MODE_RK1) {
        I.out[o] = rb[c] + I.c_in * kk[c];
        I.acc[o] = I.c_acc * kk[c];
      } else if (mode == MODE_RK4) {
        const T d = ra[c] + I.c_acc * kk[c];
        const T t = rl[c] + d;
        const T s = rb[c] + t;
        const T bb = s - rb[c];
        I.base_out[o] = s;
        I.base_lo[o] = (rb[c] - (s - bb)) + (t - bb);
      } else {
        I.out[o] = rb[c] + I.c_in * kk[c];
        I.acc[o] = ra[c] + I.c_acc * kk[c];
      }
    }
  }
}

// Coriolis + tendency at a node, given the synced gx, gy, zeta, div.
// cor_u = (f+zeta)*hv/h*J with hv/h = vt (coriolis_colocated_mod.f90:93-100).
template <class T>
__device__ __forceinline__ void node_tendency(T gx, T gy, T zeta, T dv, T f, T J, T ut, T vt,
                                              T& kh, T& ku, T& kv) {
  const T fz = f + zeta;
  ku = -gx + fz * (J * vt);
  kv = -gy - fz * (J * ut);
  kh = -dv;
}
// The same with J*ut and J*vt formed beforehand.
template <class T>
__device__ __forceinline__ void node_tendency_j(T gx, T gy, T zeta, T dv, T f, T jut, T jvt,
                                                T& kh, T& ku, T& kv) {
  const T fz = f + zeta;
  ku = -gx + fz * jvt;
  kv = -gy - fz * jut;
  kh = -dv;
}

// SBP derivative times s: interior rows with the interior coefficients
// pre-multiplied by s (sc[o-1] for offset o), closure rows as d_line * s.
template <int ORD, class T>
struct ScaledInterior {
  T c[Ord<ORD>::H];
};
template <int ORD, class T>
__device__ __forceinline__ ScaledInterior<ORD, T> scaled_interior(T s) {
  ScaledInterior<ORD, T> r;
  if constexpr (Ord<ORD>::H == 1) {
    r.c[0] = T(0.5) * s;
  } else if constexpr (Ord<ORD>::H == 2) {
    r.c[0] = T(2.0 / 3.0) * s;
    r.c[1] = T(-1.0 / 12.0) * s;
  } else {
    r.c[0] = T(3.0 / 4.0) * s;
    r.c[1] = T(-3.0 / 20.0) * s;
    r.c[2] = T(1.0 / 60.0) * s;
  }
  return r;
}
template <int ORD, class T, class FA>
__device__ __forceinline__ T d_line_scaled(int k, int n, FA fa, const ScaledInterior<ORD, T>& sc,
                                           T s) {
  constexpr int NE = Ord<ORD>::NE, H = Ord<ORD>::H;
  if (k >= NE && k < n - NE) {
    T acc = sc.c[0] * (fa(k + 1) - fa(k - 1));
#pragma unroll
    for (int o = 2; o <= H; ++o) acc += sc.c[o - 1] * (fa(k + o) - fa(k - o));
    return acc;
  }
  return d_line<ORD, T>(k, n, fa) * s;
}

// ---------------------------------------------------------------------------
// Fused stage kernel.  One CTA = one work unit (panel strip x row segment);
// thread t owns column cl0+t.  Rows stream through shared-memory rings of
// the derived fields (KE, u and J h vt for 2*RMAX+1 rows; v, J h ut, ut, vt
// and J for RMAX+1 rows), so every input node is read from global memory
// once per unit.
// ---------------------------------------------------------------------------
template <class T, int ORD>
__global__ void __launch_bounds__(STAGE_BW)
    stage_kernel(InstDev<T> one, const InstDev<T>* many, const WorkUnit* units, int mode) {
  constexpr int RMAX = Ord<ORD>::RMAX, RB = 2 * RMAX + 1, RX1 = RMAX + 1, NE = Ord<ORD>::NE;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T(*yring)[RY_N][STAGE_BW] = reinterpret_cast<T(*)[RY_N][STAGE_BW]>(smem_raw);
  T(*xring)[RX_N][STAGE_BW] =
      reinterpret_cast<T(*)[RX_N][STAGE_BW]>(smem_raw + sizeof(T) * RB * RY_N * STAGE_BW);

  const WorkUnit wu = units[blockIdx.x];
  const InstDev<T>& I = many ? many[wu.inst] : one;
  const int n = I.n, P = I.P;
  const long long pbase = (long long)wu.panel * I.ps;
  const long long fs = I.fs;
  const int t = threadIdx.x;
  const int col = wu.cl0 + t;
  const bool load_col = col < wu.cl1;
  const T grav = I.grav;
  static_assert(sizeof(T) == 8, "the FP32 form runs the TMA kernel");
  const T ghs = I.ghs;
  const ScaledInterior<ORD, T> ghs_c = scaled_interior<ORD, T>(ghs);

  auto load_row = [&](int r) {
    if (!load_col) return;
    const long long idx = pbase + (long long)r * P + col;
    const T h = I.in[idx], u = I.in[fs + idx], v = I.in[2 * fs + idx];
    const T J = I.metric[MJ * fs + idx];
    const T q1 = I.metric[MQI1 * fs + idx], q2 = I.metric[MQI2 * fs + idx],
            q3 = I.metric[MQI3 * fs + idx];
    const T ut = q1 * u + q2 * v;
    const T vt = q2 * u + q3 * v;
    T ke = (u * ut + v * vt) / T(2.0);
    ke = ke + grav * h;
    if (I.hs) ke = ke + grav * I.hs[idx];
    // J ut and J vt serve the mass flux (times h) and the Coriolis term
    const T jut = J * ut, jvt = J * vt;
    const int s = r % RB, sx = r % RX1;
    yring[s][RY_KE][t] = ke;
    yring[s][RY_U][t] = u;
    yring[s][RY_GV][t] = h * jvt;
    xring[sx][RX_V][t] = v;
    xring[sx][RX_GU][t] = h * jut;
    xring[sx][RX_JUT][t] = jut;
    xring[sx][RX_JVT][t] = jvt;
  };

  int loaded = wu.rl0;
  {
    const int target = min((int)wu.rl1, wu.j0 + RMAX + 1);
    for (; loaded < target; ++loaded) load_row(loaded);
  }
  for (int j = wu.j0; j < wu.j1; ++j) {
    if (j > wu.j0) {
      __syncthreads();
      const int target = min((int)wu.rl1, j + RMAX + 1);
      for (; loaded < target; ++loaded) load_row(loaded);
    }
    __syncthreads();
    if (col < wu.i0 || col >= wu.i1) continue;
    const int sj = j % RB, sxj = j % RX1;
    // x derivatives (along the row, neighbours are other threads' columns).
    // For the 4/2 and 4/3 stencils the KE gradient's 1/(hx a) rides in the
    // interior coefficients (measured on GB300: 2.8% faster FP64 steps at
    // N=384 d42); for 6/3 that form measured 5% slower at N=1024, so it
    // scales the derivative.
    constexpr bool kScaledGrad = Ord<ORD>::H <= 2;
    auto grad_ke = [&](int k, auto fa) {
      if constexpr (kScaledGrad) return d_line_scaled<ORD, T>(k, n, fa, ghs_c, ghs);
      else return d_line<ORD, T>(k, n, fa) * ghs;
    };
    const T gx = grad_ke(col, [&](int m) { return yring[sj][RY_KE][m - wu.cl0]; });
    const T dxv = d_line<ORD, T>(col, n, [&](int m) { return xring[sxj][RX_V][m - wu.cl0]; });
    const T dxgu = d_line<ORD, T>(col, n, [&](int m) { return xring[sxj][RX_GU][m - wu.cl0]; });
    // y derivatives (along this thread's column)
    auto ya = [&](int f) {
      return d_line<ORD, T>(j, n, [&](int m) { return yring[m % RB][f][t]; });
    };
    const T gy = grad_ke(j, [&](int m) { return yring[m % RB][RY_KE][t]; });
    const T dyu = ya(RY_U), dygv = ya(RY_GV);
    const T rJ = I.metric[MRJ * fs + pbase + (long long)j * P + col];
    const T zeta = (dxv - dyu) * rJ;
    const T dv = (dxgu + dygv) * rJ;
    const long long idx = pbase + (long long)j * P + col;
    const bool bnd = (col == 0) | (col == n - 1) | (j == 0) | (j == n - 1);
    if (bnd) {
      T* E = I.edge + (long long)wu.panel * 16 * n;
      // the four values one by one (an array of them was kept in local memory
      // for every node, boundary or not)
      auto put = [&](int side, int k) {
        T* e = E + (side * 4) * n + k;
        e[0] = gx; e[n] = gy; e[2 * n] = zeta; e[3 * n] = dv;
      };
      if (col == 0) put(SIDE_L, j);
      if (col == n - 1) put(SIDE_R, j);
      if (j == 0) put(SIDE_B, col);
      if (j == n - 1) put(SIDE_T, col);
      continue;
    }
    const T f = I.metric[MF * fs + idx];
    T kh, ku, kv;
    node_tendency_j<T>(gx, gy, zeta, dv, f, xring[sxj][RX_JUT][t], xring[sxj][RX_JVT][t], kh, ku, kv);
    stage_epilogue<T>(I, mode, idx, kh, ku, kv);
  }
  (void)NE;
}

template <class T, int ORD>
constexpr size_t stage_smem_bytes() {
  return sizeof(T) * ((2 * Ord<ORD>::RMAX + 1) * RY_N + (Ord<ORD>::RMAX + 1) * RX_N) * STAGE_BW;
}

template <class T, int ORD>
cudaError_t launch_stage_ord(const InstDev<T>& one, const InstDev<T>* many, const WorkUnit* units,
                             int nunits, int mode, cudaStream_t st) {
  constexpr size_t smem = stage_smem_bytes<T, ORD>();
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(stage_kernel<T, ORD>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  if (nunits <= 0) return cudaSuccess;
  stage_kernel<T, ORD><<<nunits, STAGE_BW, smem, st>>>(one, many, units, mode);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Cube-edge syncs at one panel-boundary node (p, i, j): returns the synced
// gx, gy (covariant gradient), zeta and div.  E points at the edge buffer of
// the instance; ring values come from the neighbour panels' entries.
// ---------------------------------------------------------------------------
template <class T>
struct EdgeView {
  const T* E;
  int n;
  __device__ __forceinline__ T get(int p, int side, int v, int k) const {
    return E[((long long)(p * 4 + side) * 4 + v) * n + k];
  }
};

template <class T>
__device__ __forceinline__ void ring_scalar(const EdgeView<T>& ev, const Topology& tp, int p,
                                            int side, int v, int k, T& out) {
  const EdgeLink L = tp.link[p][side];
  const int kk = L.rev ? ev.n - 1 - k : k;
  out = ev.get(L.q, L.side_q, v, kk);
}

template <class T>
__device__ __forceinline__ void ring_vector(const EdgeView<T>& ev, const Topology& tp, int p,
                                            int side, int k, T& rx, T& ry) {
  const EdgeLink L = tp.link[p][side];
  const int kk = L.rev ? ev.n - 1 - k : k;
  const T gxq = ev.get(L.q, L.side_q, EV_GX, kk), gyq = ev.get(L.q, L.side_q, EV_GY, kk);
  if (L.dim_i) { rx = T(L.istep) * gxq; ry = T(L.jstep) * gyq; }
  else { rx = T(L.jstep) * gyq; ry = T(L.istep) * gxq; }
}

// Scalar sync of value slot v at node (p,i,j) (halo_Ah_scalar_sync_mod.f90:38-93).
template <class T>
__device__ T sync_scalar_node(const EdgeView<T>& ev, const Topology& tp, int p, int i, int j,
                              int v, T own) {
  const int e = ev.n - 1;
  T a, b;
  if (i == 0 && j == 0) { ring_scalar(ev, tp, p, SIDE_L, v, 0, a); ring_scalar(ev, tp, p, SIDE_B, v, 0, b); return (own + a + b) / T(3.0); }
  if (i == e && j == 0) { ring_scalar(ev, tp, p, SIDE_R, v, 0, a); ring_scalar(ev, tp, p, SIDE_B, v, e, b); return (own + a + b) / T(3.0); }
  if (i == 0 && j == e) { ring_scalar(ev, tp, p, SIDE_L, v, e, a); ring_scalar(ev, tp, p, SIDE_T, v, 0, b); return (own + a + b) / T(3.0); }
  if (i == e && j == e) { ring_scalar(ev, tp, p, SIDE_R, v, e, a); ring_scalar(ev, tp, p, SIDE_T, v, e, b); return (own + a + b) / T(3.0); }
  if (i == 0) { ring_scalar(ev, tp, p, SIDE_L, v, j, a); return T(0.5) * (a + own); }
  if (i == e) { ring_scalar(ev, tp, p, SIDE_R, v, j, a); return T(0.5) * (own + a); }
  if (j == 0) { ring_scalar(ev, tp, p, SIDE_B, v, i, a); return T(0.5) * (own + a); }
  ring_scalar(ev, tp, p, SIDE_T, v, i, a);
  return T(0.5) * (own + a);
}

// Covariant vector sync at node (p,i,j): syncronize_grad_on_edges with U = gy,
// V = gx (ecs_Ah_vec_sync_mod.f90:52, 62-125).  qw = qb|qt|ql|qr (n each).
template <class T>
__device__ void sync_vector_node(const EdgeView<T>& ev, const Topology& tp, const double* qw,
                                 int p, int i, int j, T& gx, T& gy) {
  const int n = ev.n, e = n - 1;
  const double* qb = qw;
  const double* qt = qw + n;
  const double* ql = qw + 2 * n;
  const double* qr = qw + 3 * n;
  T V = gx, U = gy;
  T rx, ry, sx, sy;
  if (i == 0 && j == 0) {
    ring_vector(ev, tp, p, SIDE_L, 0, rx, ry); ring_vector(ev, tp, p, SIDE_B, 0, sx, sy);
    gy = (U + ry + sy + T(qb[0]) * sx) / T(3.0);
    gx = (V + rx + sx + T(ql[0]) * ry) / T(3.0);
  } else if (i == e && j == 0) {
    ring_vector(ev, tp, p, SIDE_R, 0, rx, ry); ring_vector(ev, tp, p, SIDE_B, e, sx, sy);
    gy = (U + ry + sy + T(qb[e]) * sx) / T(3.0);
    gx = (V + rx + sx + T(qr[0]) * ry) / T(3.0);
  } else if (i == 0 && j == e) {
    ring_vector(ev, tp, p, SIDE_L, e, rx, ry); ring_vector(ev, tp, p, SIDE_T, 0, sx, sy);
    gy = (U + ry + sy + T(qt[0]) * sx) / T(3.0);
    gx = (V + rx + sx + T(ql[e]) * ry) / T(3.0);
  } else if (i == e && j == e) {
    ring_vector(ev, tp, p, SIDE_R, e, rx, ry); ring_vector(ev, tp, p, SIDE_T, e, sx, sy);
    gy = (U + ry + sy + T(qt[e]) * sx) / T(3.0);
    gx = (V + rx + sx + T(qr[e]) * ry) / T(3.0);
  } else if (i == 0) {
    ring_vector(ev, tp, p, SIDE_L, j, rx, ry);
    gy = T(0.5) * (ry + U);
    gx = T(0.5) * (V + rx + T(ql[j]) * ry);
  } else if (i == e) {
    ring_vector(ev, tp, p, SIDE_R, j, rx, ry);
    gy = T(0.5) * (U + ry);
    gx = T(0.5) * (V + rx + T(qr[j]) * ry);
  } else if (j == 0) {
    ring_vector(ev, tp, p, SIDE_B, i, sx, sy);
    gx = T(0.5) * (sx + V);
    gy = T(0.5) * (sy + U + T(qb[i]) * sx);
  } else {
    ring_vector(ev, tp, p, SIDE_T, i, sx, sy);
    gx = T(0.5) * (V + sx);
    gy = T(0.5) * (U + sy + T(qt[i]) * sx);
  }
}

// boundary node b of a panel (0 <= b < 4n-4) -> (i, j); bottom and top rows
// own the corners.
__device__ __forceinline__ void boundary_node(int b, int n, int& i, int& j) {
  if (b < n) { i = b; j = 0; }
  else if (b < 2 * n) { i = b - n; j = n - 1; }
  else if (b < 3 * n - 2) { i = 0; j = b - 2 * n + 1; }
  else { i = n - 1; j = b - (3 * n - 2) + 1; }
}

// ---------------------------------------------------------------------------
// Edge kernel: finishes every panel-boundary node of every instance.
// blockIdx.y = instance, x covers 6*(4n-4) nodes.
// ---------------------------------------------------------------------------
template <class T>
__global__ void edge_kernel(InstDev<T> one, const InstDev<T>* many, Topology tp, int mode) {
  const InstDev<T>& I = many ? many[blockIdx.y] : one;
  const int n = I.n, nb = 4 * n - 4, e = n - 1;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= 6 * nb) return;
  const int p = g / nb;
  int i, j;
  boundary_node(g - p * nb, n, i, j);
  // The node lies on a left/right side (lr), a bottom/top side (bt), or both
  // (cube corner).  Every address below is known before any load, so all
  // loads of the node issue together.
  const bool lr = (i == 0) | (i == e), bt = (j == 0) | (j == e);
  const int sLR = i == 0 ? SIDE_L : SIDE_R, sBT = j == 0 ? SIDE_B : SIDE_T;
  const EdgeLink LL = tp.link[p][sLR], LB = tp.link[p][sBT];
  const T* E = I.edge;
  auto at = [&](int q, int s, int v, int k) { return E[((q * 4 + s) * 4 + v) * n + k]; };
  const int so = lr ? sLR : sBT, ko = lr ? j : i;          // own values
  const int kl = LL.rev ? e - j : j, kb = LB.rev ? e - i : i;  // neighbour positions
  T own[4], nl[4], nbt[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    own[v] = at(p, so, v, ko);
    nl[v] = lr ? at(LL.q, LL.side_q, v, kl) : T(0);
    nbt[v] = bt ? at(LB.q, LB.side_q, v, kb) : T(0);
  }
  const double* qw = I.qw;
  const T qlr = lr ? T(qw[(i == 0 ? 2 : 3) * n + j]) : T(0);   // ql / qr at j
  const T qbt = bt ? T(qw[(j == 0 ? 0 : 1) * n + i]) : T(0);   // qb / qt at i
  const long long fs = I.fs;
  const long long idx = (long long)p * I.ps + (long long)j * I.P + i;
  const T u = I.in[fs + idx], v = I.in[2 * fs + idx];
  const T q1 = I.metric[MQI1 * fs + idx], q2 = I.metric[MQI2 * fs + idx],
          q3 = I.metric[MQI3 * fs + idx];
  const T J = I.metric[MJ * fs + idx], f = I.metric[MF * fs + idx];
  // RK inputs of the node, loaded with everything else
  const bool fp32 = sizeof(T) == 4;
  const bool needB = mode == MODE_RK1 || mode == MODE_RK2 || mode == MODE_RK3 ||
                     (fp32 && mode == MODE_RK4);
  const bool needA = mode == MODE_RK2 || mode == MODE_RK3 || mode == MODE_RK4;
  const bool needL = fp32 && mode == MODE_RK4;
  const T* bsrc = mode == MODE_RK4 ? I.base_out : I.base;
  T rb[3], ra[3], rlo[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    rb[c] = needB ? bsrc[c * fs + idx] : T(0);
    ra[c] = needA ? I.acc[c * fs + idx] : T(0);
    rlo[c] = needL ? I.base_lo[c * fs + idx] : T(0);
  }

  // neighbour vectors in this panel's frame (pack_to_buf_vec component map)
  auto rot = [](const EdgeLink& L, T gxq, T gyq, T& rx, T& ry) {
    if (L.dim_i) { rx = T(L.istep) * gxq; ry = T(L.jstep) * gyq; }
    else { rx = T(L.jstep) * gyq; ry = T(L.istep) * gxq; }
  };
  T rx, ry, sx, sy;
  rot(LL, nl[EV_GX], nl[EV_GY], rx, ry);
  rot(LB, nbt[EV_GX], nbt[EV_GY], sx, sy);
  const T U = own[EV_GY], V = own[EV_GX];
  T gx, gy, zeta, dv;
  if (lr && bt) {
    // cube corner: 3-way averages (halo_Ah_scalar_sync_mod.f90:56-85,
    // ecs_Ah_vec_sync_mod.f90:77-100)
    gy = (U + ry + sy + qbt * sx) / T(3.0);
    gx = (V + rx + sx + qlr * ry) / T(3.0);
    zeta = (own[EV_ZETA] + nl[EV_ZETA] + nbt[EV_ZETA]) / T(3.0);
    dv = (own[EV_DIV] + nl[EV_DIV] + nbt[EV_DIV]) / T(3.0);
  } else if (lr) {
    gy = T(0.5) * (U + ry);
    gx = T(0.5) * (V + rx + qlr * ry);
    zeta = T(0.5) * (own[EV_ZETA] + nl[EV_ZETA]);
    dv = T(0.5) * (own[EV_DIV] + nl[EV_DIV]);
  } else {
    gx = T(0.5) * (V + sx);
    gy = T(0.5) * (U + sy + qbt * sx);
    zeta = T(0.5) * (own[EV_ZETA] + nbt[EV_ZETA]);
    dv = T(0.5) * (own[EV_DIV] + nbt[EV_DIV]);
  }
  const T ut = q1 * u + q2 * v, vt = q2 * u + q3 * v;
  T kh, ku, kv;
  node_tendency<T>(gx, gy, zeta, dv, f, J, ut, vt, kh, ku, kv);
  stage_epilogue_pre<T>(I, mode, idx, kh, ku, kv, rb, ra, rlo);
}

}  // namespace swm
