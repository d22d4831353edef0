// swm_adjoint.cu -- tangent-linear (TL) and adjoint (AD) kernels of the FP64
// vector-invariant model operator F (operator_swm_mod.f90:61-113), for the
// discrete adjoint of the RK4 step.  No counterpart in the reference.
//
// With base state y = (h, u, v), ut = Qi11 u + Qi12 v, vt = Qi12 u + Qi22 v,
// K = (u ut + v vt)/2 + g (h + hs), the operator is
//   (GX, GY) = Sv(ghs Dx K, ghs Dy K)              covariant vector sync Sv
//   Z        = Ss(rJ (Dx v - Dy u))                scalar sync Ss (curl)
//   DIV      = Ss(rJ (Dx (J h ut) + Dy (J h vt)))  (divergence of the mass flux)
//   k_u = -GX + (f + Z) J vt,  k_v = -GY - (f + Z) J ut,  k_h = -DIV
// with rJ = 1/(J hx a).  The TL kernels below linearise the pointwise parts;
// the linear parts (D, Sv, Ss) reuse the forward operator kernels.  The AD
// kernels apply the exact transposes: D^T through a transposed closure table
// (SbpT), Ss^T = Ss (the sync averages each class of duplicated edge nodes
// with equal weights, a symmetric projection) and Sv^T in two deterministic
// passes (pull back onto the neighbour values each node read, then gather).
#include "swm_ops.cuh"
#include "swm_stage.cuh"

namespace swm {

namespace {

constexpr int TPB = 256;
inline int nblk(long long count) { return (int)((count + TPB - 1) / TPB); }

struct Node {
  int p, i, j;
  long long x;
};

__device__ __forceinline__ bool node_of(const FieldGeom& g, Node& o) {
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nn = (long long)g.n * g.n;
  if (gid >= 6 * nn) return false;
  o.p = (int)(gid / nn);
  const long long r = gid - (long long)o.p * nn;
  o.j = (int)(r / g.n);
  o.i = (int)(r - (long long)o.j * g.n);
  o.x = (long long)o.p * g.ps + (long long)o.j * g.P + o.i;
  return true;
}

// (D^T f)_c of the 1-D SBP operator along one grid line; F(k) is f at line
// index k.  Columns near the ends use the transposed closure block, the
// interior the negated interior stencil (the interior stencil is
// antisymmetric).
template <class Get>
__device__ __forceinline__ double dT_line(const SbpT& t, int n, int c, Get F) {
  double s = 0.0;
  if (c < t.ct) {
    for (int r = 0; r < t.kr; ++r) s += t.t[c * t.kr + r] * F(r);
    return s;
  }
  if (c >= n - t.ct) {
    const int cc = n - 1 - c;
    for (int r = 0; r < t.kr; ++r) s += t.t[cc * t.kr + r] * F(n - 1 - r);
    return -s;
  }
  for (int m = 0; m < t.nin; ++m) s += t.qin[m] * F(c + t.inshift + m);
  return -s;
}

__global__ void tl_pre_kernel(FieldGeom g, const double* m, double grav, const double* y,
                              const double* dx, double* w) {
  Node o;
  if (!node_of(g, o)) return;
  const long long fs = g.fs, x = o.x;
  const double h = y[x], u = y[fs + x], v = y[2 * fs + x];
  const double dh = dx[x], du = dx[fs + x], dv = dx[2 * fs + x];
  const double q1 = m[MQI1 * fs + x], q2 = m[MQI2 * fs + x], q3 = m[MQI3 * fs + x];
  const double ut = q1 * u + q2 * v, vt = q2 * u + q3 * v;
  const double dut = q1 * du + q2 * dv, dvt = q2 * du + q3 * dv;
  w[x] = 0.5 * (du * ut + u * dut + dv * vt + v * dvt) + grav * dh;   // dK
  w[fs + x] = dh * ut + h * dut;                                       // d(h ut)
  w[2 * fs + x] = dh * vt + h * dvt;                                   // d(h vt)
  w[3 * fs + x] = dut;
  w[4 * fs + x] = dvt;
}

// dk from the synced linear parts: dG = (dGX, dGY), dZ, dDIV
__global__ void tl_post_kernel(FieldGeom g, const double* m, const double* y, const double* zeta,
                               const double* w, const double* dgx, const double* dgy,
                               const double* dz, const double* ddiv, double* dk) {
  Node o;
  if (!node_of(g, o)) return;
  const long long fs = g.fs, x = o.x;
  const double u = y[fs + x], v = y[2 * fs + x];
  const double q1 = m[MQI1 * fs + x], q2 = m[MQI2 * fs + x], q3 = m[MQI3 * fs + x];
  const double J = m[MJ * fs + x], fz = m[MF * fs + x] + zeta[x];
  const double ut = q1 * u + q2 * v, vt = q2 * u + q3 * v;
  const double dut = w[3 * fs + x], dvt = w[4 * fs + x];
  dk[x] = -ddiv[x];
  dk[fs + x] = -dgx[x] + dz[x] * J * vt + fz * J * dvt;
  dk[2 * fs + x] = -dgy[x] - dz[x] * J * ut - fz * J * dut;
}

// Cotangents of the synced quantities from the cotangent lk of (k_h, k_u, k_v):
// A = (lGX, lGY, lDIV, lZ, l_ut part, l_vt part)
__global__ void ad_pre_kernel(FieldGeom g, const double* m, const double* y, const double* zeta,
                              const double* lk, double* A) {
  Node o;
  if (!node_of(g, o)) return;
  const long long fs = g.fs, x = o.x;
  const double u = y[fs + x], v = y[2 * fs + x];
  const double q1 = m[MQI1 * fs + x], q2 = m[MQI2 * fs + x], q3 = m[MQI3 * fs + x];
  const double J = m[MJ * fs + x], fz = m[MF * fs + x] + zeta[x];
  const double ut = q1 * u + q2 * v, vt = q2 * u + q3 * v;
  const double lh = lk[x], lu = lk[fs + x], lv = lk[2 * fs + x];
  A[x] = -lu;
  A[fs + x] = -lv;
  A[2 * fs + x] = -lh;
  A[3 * fs + x] = J * (vt * lu - ut * lv);
  A[4 * fs + x] = -fz * J * lv;
  A[5 * fs + x] = fz * J * lu;
}

// out = F'(y)^T lk from the synced-transposed cotangents A (see ad_pre_kernel)
__global__ void ad_main_kernel(FieldGeom g, SbpT t, const double* m, double ghs, double grav,
                               const double* y, const double* A, double* out) {
  Node o;
  if (!node_of(g, o)) return;
  const long long fs = g.fs, x = o.x;
  const int n = g.n;
  const long long row = (long long)o.p * g.ps + (long long)o.j * g.P;   // node (0, j)
  const long long col = (long long)o.p * g.ps + o.i;                     // node (i, 0)
  const double* A1 = A;
  const double* A2 = A + fs;
  const double* A3 = A + 2 * fs;
  const double* A4 = A + 3 * fs;
  const double* rJ = m + MRJ * fs;
  const double dx1 = dT_line(t, n, o.i, [&](int k) { return A1[row + k]; });
  const double dy2 = dT_line(t, n, o.j, [&](int k) { return A2[col + (long long)k * g.P]; });
  const double dx3 = dT_line(t, n, o.i, [&](int k) { return rJ[row + k] * A3[row + k]; });
  const double dy3 = dT_line(t, n, o.j, [&](int k) {
    const long long q = col + (long long)k * g.P;
    return rJ[q] * A3[q];
  });
  const double dx4 = dT_line(t, n, o.i, [&](int k) { return rJ[row + k] * A4[row + k]; });
  const double dy4 = dT_line(t, n, o.j, [&](int k) {
    const long long q = col + (long long)k * g.P;
    return rJ[q] * A4[q];
  });
  const double h = y[x], u = y[fs + x], v = y[2 * fs + x];
  const double q1 = m[MQI1 * fs + x], q2 = m[MQI2 * fs + x], q3 = m[MQI3 * fs + x];
  const double J = m[MJ * fs + x];
  const double ut = q1 * u + q2 * v, vt = q2 * u + q3 * v;
  const double lK = ghs * (dx1 + dy2);
  const double lGu = dx3, lGv = dy3;          // cotangents of J h ut, J h vt
  const double lut = A[4 * fs + x] + J * h * lGu + 0.5 * u * lK;
  const double lvt = A[5 * fs + x] + J * h * lGv + 0.5 * v * lK;
  out[x] = J * (ut * lGu + vt * lGv) + grav * lK;
  out[fs + x] = -dy4 + 0.5 * ut * lK + q1 * lut + q2 * lvt;
  out[2 * fs + x] = dx4 + 0.5 * vt * lK + q2 * lut + q3 * lvt;
}

// Sv^T, pass 1: at every panel-boundary node, pull the cotangent (lgx, lgy)
// of the node's synced output back onto the raw neighbour values the sync
// read (ring_vector, component map included) and store it at the reading
// node's slot C[p][side][EV_GX|EV_GY][k].
__device__ __forceinline__ void put_ring(double* C, const Topology& tp, int n, int p, int side,
                                         int k, double lrx, double lry) {
  const EdgeLink L = tp.link[p][side];
  double lgx, lgy;
  if (L.dim_i) { lgx = L.istep * lrx; lgy = L.jstep * lry; }
  else { lgy = L.jstep * lrx; lgx = L.istep * lry; }
  C[((long long)(p * 4 + side) * 4 + EV_GX) * n + k] = lgx;
  C[((long long)(p * 4 + side) * 4 + EV_GY) * n + k] = lgy;
}

__global__ void adsync_vec_pull_kernel(FieldGeom g, Topology tp, const double* qw,
                                       const double* lgx, const double* lgy, double* C) {
  const int n = g.n, nb = 4 * n - 4, e = n - 1;
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6 * nb) return;
  const int p = gi / nb;
  int i, j;
  boundary_node(gi - p * nb, n, i, j);
  const long long x = (long long)p * g.ps + (long long)j * g.P + i;
  const double a = lgx[x], b = lgy[x];     // cotangents of the synced gx (V) and gy (U)
  const double* qb = qw;
  const double* qt = qw + n;
  const double* ql = qw + 2 * n;
  const double* qr = qw + 3 * n;
  const double t3 = 1.0 / 3.0;
  if (i == 0 && j == 0) {
    put_ring(C, tp, n, p, SIDE_L, 0, a * t3, b * t3 + ql[0] * a * t3);
    put_ring(C, tp, n, p, SIDE_B, 0, a * t3 + qb[0] * b * t3, b * t3);
  } else if (i == e && j == 0) {
    put_ring(C, tp, n, p, SIDE_R, 0, a * t3, b * t3 + qr[0] * a * t3);
    put_ring(C, tp, n, p, SIDE_B, e, a * t3 + qb[e] * b * t3, b * t3);
  } else if (i == 0 && j == e) {
    put_ring(C, tp, n, p, SIDE_L, e, a * t3, b * t3 + ql[e] * a * t3);
    put_ring(C, tp, n, p, SIDE_T, 0, a * t3 + qt[0] * b * t3, b * t3);
  } else if (i == e && j == e) {
    put_ring(C, tp, n, p, SIDE_R, e, a * t3, b * t3 + qr[e] * a * t3);
    put_ring(C, tp, n, p, SIDE_T, e, a * t3 + qt[e] * b * t3, b * t3);
  } else if (i == 0) {
    put_ring(C, tp, n, p, SIDE_L, j, 0.5 * a, 0.5 * b + 0.5 * ql[j] * a);
  } else if (i == e) {
    put_ring(C, tp, n, p, SIDE_R, j, 0.5 * a, 0.5 * b + 0.5 * qr[j] * a);
  } else if (j == 0) {
    put_ring(C, tp, n, p, SIDE_B, i, 0.5 * a + 0.5 * qb[i] * b, 0.5 * b);
  } else {
    put_ring(C, tp, n, p, SIDE_T, i, 0.5 * a + 0.5 * qt[i] * b, 0.5 * b);
  }
}

// Sv^T, pass 2: a node's input cotangent is its own share of its synced
// output plus what every copy that read it pulled back (in fixed order).
__global__ void adsync_vec_gather_kernel(FieldGeom g, Topology tp, const double* C, double* lgx,
                                         double* lgy) {
  const int n = g.n, nb = 4 * n - 4, e = n - 1;
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6 * nb) return;
  const int p = gi / nb;
  int i, j;
  boundary_node(gi - p * nb, n, i, j);
  const long long x = (long long)p * g.ps + (long long)j * g.P + i;
  const bool corner = (i == 0 || i == e) && (j == 0 || j == e);
  const double own = corner ? 1.0 / 3.0 : 0.5;
  double ax = own * lgx[x], ay = own * lgy[x];
  auto add = [&](int side, int k) {
    const EdgeLink L = tp.link[p][side];
    const int kk = L.rev ? n - 1 - k : k;
    ax += C[((long long)(L.q * 4 + L.side_q) * 4 + EV_GX) * n + kk];
    ay += C[((long long)(L.q * 4 + L.side_q) * 4 + EV_GY) * n + kk];
  };
  if (i == 0) add(SIDE_L, j);
  if (i == e) add(SIDE_R, j);
  if (j == 0) add(SIDE_B, i);
  if (j == e) add(SIDE_T, i);
  lgx[x] = ax;
  lgy[x] = ay;
}

}  // namespace

cudaError_t launch_tl_pre(const FieldGeom& g, const double* m64, double grav, const double* y,
                          const double* dx, double* w, cudaStream_t st) {
  tl_pre_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, m64, grav, y, dx, w);
  return cudaGetLastError();
}

cudaError_t launch_tl_post(const FieldGeom& g, const double* m64, const double* y,
                           const double* zeta, const double* w, const double* dgx,
                           const double* dgy, const double* dz, const double* ddiv, double* dk,
                           cudaStream_t st) {
  tl_post_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, m64, y, zeta, w, dgx, dgy, dz, ddiv, dk);
  return cudaGetLastError();
}

cudaError_t launch_ad_pre(const FieldGeom& g, const double* m64, const double* y,
                          const double* zeta, const double* lk, double* A, cudaStream_t st) {
  ad_pre_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, m64, y, zeta, lk, A);
  return cudaGetLastError();
}

cudaError_t launch_ad_main(const FieldGeom& g, const SbpT& t, const double* m64, double ghs,
                           double grav, const double* y, const double* A, double* out,
                           cudaStream_t st) {
  ad_main_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, t, m64, ghs, grav, y, A, out);
  return cudaGetLastError();
}

cudaError_t launch_adsync_vector(const FieldGeom& g, const Topology& tp, const double* qw,
                                 double* lgx, double* lgy, double* C, cudaStream_t st) {
  const int nb = 6 * (4 * g.n - 4);
  adsync_vec_pull_kernel<<<nblk(nb), TPB, 0, st>>>(g, tp, qw, lgx, lgy, C);
  adsync_vec_gather_kernel<<<nblk(nb), TPB, 0, st>>>(g, tp, C, lgx, lgy);
  return cudaGetLastError();
}

}  // namespace swm
