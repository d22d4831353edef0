// swm_adjoint.cu -- tangent-linear (TL, FP64) and adjoint (AD, FP64 or FP32)
// kernels of the vector-invariant model operator F (operator_swm_mod.f90:
// 61-113), for the discrete adjoint of the RK4 step.  No counterpart in the
// reference.
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

// Columns next to each line end that need the transposed closure block (ct)
// and the rows those columns read (kr), per SBP order:
// ct = max(max_r last[r], ne + H), kr = ct + H.
template <int ORD> struct AdOrd;
template <> struct AdOrd<21> { static constexpr int CT = 2, KR = 3; };
template <> struct AdOrd<42> { static constexpr int CT = 6, KR = 8; };
template <> struct AdOrd<43> { static constexpr int CT = 6, KR = 8; };
template <> struct AdOrd<63> { static constexpr int CT = 9, KR = 12; };

// (D^T f)_c of the 1-D SBP operator along one grid line; F(k) is f at line
// index k.  Columns near the ends use the transposed closure block, the
// interior the negated interior stencil (the interior stencil is
// antisymmetric).
template <int ORD, class T, class Get>
__device__ __forceinline__ T dT_line(const SbpT& t, int n, int c, Get F) {
  constexpr int CT = AdOrd<ORD>::CT, KR = AdOrd<ORD>::KR;
  T s = T(0);
  if (c < CT) {
#pragma unroll
    for (int r = 0; r < KR; ++r) s += T(t.t[c * KR + r]) * F(r);
    return s;
  }
  if (c >= n - CT) {
    const int cc = n - 1 - c;
#pragma unroll
    for (int r = 0; r < KR; ++r) s += T(t.t[cc * KR + r]) * F(n - 1 - r);
    return -s;
  }
  return -d_interior<ORD, T>([&](int o) { return F(c + o); });
}

// Pre-sync curl of the base state, rJ (Dx v - Dy u), with the values of the
// panel-boundary nodes also stored in the EV_ZETA slots of the edge buffer
// Z (the layout of the forward edge buffer).
template <class T, int ORD>
__global__ void zeta_pre_kernel(FieldGeom g, const T* m, const T* y, T* zeta, T* Z) {
  Node o;
  if (!node_of(g, o)) return;
  const long long fs = g.fs, x = o.x;
  const int n = g.n, e = n - 1;
  const long long row = (long long)o.p * g.ps + (long long)o.j * g.P;
  const long long col = (long long)o.p * g.ps + o.i;
  const T* u = y + fs;
  const T* v = y + 2 * fs;
  const T dxv = d_line<ORD, T>(o.i, n, [&](int k) { return v[row + k]; });
  const T dyu = d_line<ORD, T>(o.j, n, [&](int k) { return u[col + (long long)k * g.P]; });
  const T z = (dxv - dyu) * m[MRJ * fs + x];
  zeta[x] = z;
  auto put = [&](int side, int k) { Z[((long long)(o.p * 4 + side) * 4 + EV_ZETA) * n + k] = z; };
  if (o.i == 0) put(SIDE_L, o.j);
  if (o.i == e) put(SIDE_R, o.j);
  if (o.j == 0) put(SIDE_B, o.i);
  if (o.j == e) put(SIDE_T, o.i);
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

// Sv^T pull of one boundary node: the cotangent of a raw neighbour value
// read through ring_vector (component map included) goes to the reading
// node's slot C[p][side][EV_GX|EV_GY][k].
template <class T>
__device__ __forceinline__ void put_ring(T* C, const Topology& tp, int n, int p, int side,
                                         int k, T lrx, T lry) {
  const EdgeLink L = tp.link[p][side];
  T lgx, lgy;
  if (L.dim_i) { lgx = T(L.istep) * lrx; lgy = T(L.jstep) * lry; }
  else { lgy = T(L.jstep) * lrx; lgx = T(L.istep) * lry; }
  C[((long long)(p * 4 + side) * 4 + EV_GX) * n + k] = lgx;
  C[((long long)(p * 4 + side) * 4 + EV_GY) * n + k] = lgy;
}

// the pulls of one boundary node (i, j) of panel p: (a, b) are the
// cotangents of its synced (gx, gy) = (V, U) (syncronize_grad_on_edges,
// transposed case by case), s1/s2 the two scalar fields
template <class T>
__device__ __forceinline__ void pull_node(T* C, const Topology& tp, const double* qw, int n,
                                          int p, int i, int j, T a, T b, T s1, T s2) {
  const int e = n - 1;
  const double* qb = qw;
  const double* qt = qw + n;
  const double* ql = qw + 2 * n;
  const double* qr = qw + 3 * n;
  const T t3 = T(1.0 / 3.0), hf = T(0.5);
  if (i == 0 && j == 0) {
    put_ring(C, tp, n, p, SIDE_L, 0, a * t3, b * t3 + T(ql[0]) * a * t3);
    put_ring(C, tp, n, p, SIDE_B, 0, a * t3 + T(qb[0]) * b * t3, b * t3);
  } else if (i == e && j == 0) {
    put_ring(C, tp, n, p, SIDE_R, 0, a * t3, b * t3 + T(qr[0]) * a * t3);
    put_ring(C, tp, n, p, SIDE_B, e, a * t3 + T(qb[e]) * b * t3, b * t3);
  } else if (i == 0 && j == e) {
    put_ring(C, tp, n, p, SIDE_L, e, a * t3, b * t3 + T(ql[e]) * a * t3);
    put_ring(C, tp, n, p, SIDE_T, 0, a * t3 + T(qt[0]) * b * t3, b * t3);
  } else if (i == e && j == e) {
    put_ring(C, tp, n, p, SIDE_R, e, a * t3, b * t3 + T(qr[e]) * a * t3);
    put_ring(C, tp, n, p, SIDE_T, e, a * t3 + T(qt[e]) * b * t3, b * t3);
  } else if (i == 0) {
    put_ring(C, tp, n, p, SIDE_L, j, hf * a, hf * b + hf * T(ql[j]) * a);
  } else if (i == e) {
    put_ring(C, tp, n, p, SIDE_R, j, hf * a, hf * b + hf * T(qr[j]) * a);
  } else if (j == 0) {
    put_ring(C, tp, n, p, SIDE_B, i, hf * a + hf * T(qb[i]) * b, hf * b);
  } else {
    put_ring(C, tp, n, p, SIDE_T, i, hf * a + hf * T(qt[i]) * b, hf * b);
  }
  auto putS = [&](int side, int k) {
    C[((long long)(p * 4 + side) * 4 + EV_ZETA) * n + k] = s1;
    C[((long long)(p * 4 + side) * 4 + EV_DIV) * n + k] = s2;
  };
  if (i == 0) putS(SIDE_L, j);
  if (i == e) putS(SIDE_R, j);
  if (j == 0) putS(SIDE_B, i);
  if (j == e) putS(SIDE_T, i);
}

// Cotangents of the synced quantities from lk = alpha*lam + beta*mu (mu
// nullable) of (k_h, k_u, k_v), with the base curl synced here (zeta holds
// the pre-sync curl, Z its edge values):
// A = (lGX, lGY, rJ*lDIV, rJ*lZ, l_ut part, l_vt part); at panel-boundary
// nodes the raw (unsynced) cotangents are pulled into C for adsync_gather.
template <class T>
__global__ void ad_pre_kernel(FieldGeom g, Topology tp, const double* qw, const T* m, const T* y,
                              const T* zeta, const T* Z, const T* lam, const T* mu, T alpha,
                              T beta, T* A, T* C) {
  Node o;
  if (!node_of(g, o)) return;
  const long long fs = g.fs, x = o.x;
  const int n = g.n, e = n - 1;
  const bool edge = o.i == 0 || o.i == e || o.j == 0 || o.j == e;
  T z = zeta[x];
  if (edge) z = sync_scalar_node<T>(EdgeView<T>{Z, n}, tp, o.p, o.i, o.j, EV_ZETA, z);
  const T u = y[fs + x], v = y[2 * fs + x];
  const T q1 = m[MQI1 * fs + x], q2 = m[MQI2 * fs + x], q3 = m[MQI3 * fs + x];
  const T J = m[MJ * fs + x], fz = m[MF * fs + x] + z, rJ = m[MRJ * fs + x];
  const T ut = q1 * u + q2 * v, vt = q2 * u + q3 * v;
  T lh = alpha * lam[x], lu = alpha * lam[fs + x], lv = alpha * lam[2 * fs + x];
  if (mu) {
    lh += beta * mu[x];
    lu += beta * mu[fs + x];
    lv += beta * mu[2 * fs + x];
  }
  const T lz = J * (vt * lu - ut * lv);
  A[x] = -lu;
  A[fs + x] = -lv;
  A[2 * fs + x] = -lh * rJ;
  A[3 * fs + x] = lz * rJ;
  A[4 * fs + x] = -fz * J * lv;
  A[5 * fs + x] = fz * J * lu;
  if (edge) pull_node(C, tp, qw, n, o.p, o.i, o.j, -lu, -lv, -lh, lz);
}

// mu = F'(y)^T lk from the synced-transposed cotangents A (ad_pre_kernel +
// adsync_gather_kernel); also acc_out = acc_in + mu (acc_in/acc_out
// nullable; acc_out may be acc_in)
template <class T, int ORD>
__global__ void ad_main_kernel(FieldGeom g, SbpT t, const T* m, T ghs, T grav, const T* y,
                               const T* A, T* out, const T* acc_in, T* acc_out) {
  Node o;
  if (!node_of(g, o)) return;
  const long long fs = g.fs, x = o.x;
  const int n = g.n;
  const long long row = (long long)o.p * g.ps + (long long)o.j * g.P;   // node (0, j)
  const long long col = (long long)o.p * g.ps + o.i;                     // node (i, 0)
  const T* A1 = A;
  const T* A2 = A + fs;
  const T* W3 = A + 2 * fs;
  const T* W4 = A + 3 * fs;
  const T dx1 = dT_line<ORD, T>(t, n, o.i, [&](int k) { return A1[row + k]; });
  const T dy2 = dT_line<ORD, T>(t, n, o.j, [&](int k) { return A2[col + (long long)k * g.P]; });
  const T dx3 = dT_line<ORD, T>(t, n, o.i, [&](int k) { return W3[row + k]; });
  const T dy3 = dT_line<ORD, T>(t, n, o.j, [&](int k) { return W3[col + (long long)k * g.P]; });
  const T dx4 = dT_line<ORD, T>(t, n, o.i, [&](int k) { return W4[row + k]; });
  const T dy4 = dT_line<ORD, T>(t, n, o.j, [&](int k) { return W4[col + (long long)k * g.P]; });
  const T h = y[x], u = y[fs + x], v = y[2 * fs + x];
  const T q1 = m[MQI1 * fs + x], q2 = m[MQI2 * fs + x], q3 = m[MQI3 * fs + x];
  const T J = m[MJ * fs + x];
  const T ut = q1 * u + q2 * v, vt = q2 * u + q3 * v;
  const T lK = ghs * (dx1 + dy2);
  const T lGu = dx3, lGv = dy3;          // cotangents of J h ut, J h vt
  const T lut = A[4 * fs + x] + J * h * lGu + T(0.5) * u * lK;
  const T lvt = A[5 * fs + x] + J * h * lGv + T(0.5) * v * lK;
  const T mh = J * (ut * lGu + vt * lGv) + grav * lK;
  const T mu_ = -dy4 + T(0.5) * ut * lK + q1 * lut + q2 * lvt;
  const T mv = dx4 + T(0.5) * vt * lK + q2 * lut + q3 * lvt;
  if (out) {
    out[x] = mh;
    out[fs + x] = mu_;
    out[2 * fs + x] = mv;
  }
  if (acc_out) {
    acc_out[x] = acc_in[x] + mh;
    acc_out[fs + x] = acc_in[fs + x] + mu_;
    acc_out[2 * fs + x] = acc_in[2 * fs + x] + mv;
  }
}

// Pass 2: a node's vector input cotangent is its own share of its synced
// output plus what every copy that read it pulled back (fixed order); the
// two scalar fields get the forward scalar sync (its own transpose).
// s1, s2 are scaled by rJ in the field (A's W3/W4) and raw in C
template <class T>
__global__ void adsync_gather_kernel(FieldGeom g, Topology tp, const T* m, const T* C, T* lgx,
                                     T* lgy, T* s1, T* s2) {
  const int n = g.n, nb = 4 * n - 4, e = n - 1;
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6 * nb) return;
  const int p = gi / nb;
  int i, j;
  boundary_node(gi - p * nb, n, i, j);
  const long long x = (long long)p * g.ps + (long long)j * g.P + i;
  const bool corner = (i == 0 || i == e) && (j == 0 || j == e);
  const T own = corner ? T(1.0 / 3.0) : T(0.5);
  T ax = own * lgx[x], ay = own * lgy[x];
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
  const EdgeView<T> ev{C, n};
  const T own1 = ev.get(p, i == 0 ? SIDE_L : i == e ? SIDE_R : j == 0 ? SIDE_B : SIDE_T, EV_ZETA,
                             (i == 0 || i == e) ? j : i);
  const T own2 = ev.get(p, i == 0 ? SIDE_L : i == e ? SIDE_R : j == 0 ? SIDE_B : SIDE_T, EV_DIV,
                             (i == 0 || i == e) ? j : i);
  const T rJ = m[MRJ * g.fs + x];
  const T z = sync_scalar_node<T>(ev, tp, p, i, j, EV_ZETA, own1);
  const T d = sync_scalar_node<T>(ev, tp, p, i, j, EV_DIV, own2);
  lgx[x] = ax;
  lgy[x] = ay;
  s1[x] = z * rJ;
  s2[x] = d * rJ;
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

template <class T>
cudaError_t launch_zeta_pre(const FieldGeom& g, int order, const T* m, const T* y, T* zeta, T* Z,
                            cudaStream_t st) {
  const int nb = nblk(6LL * g.n * g.n);
  switch (order) {
    case 21: zeta_pre_kernel<T, 21><<<nb, TPB, 0, st>>>(g, m, y, zeta, Z); break;
    case 42: zeta_pre_kernel<T, 42><<<nb, TPB, 0, st>>>(g, m, y, zeta, Z); break;
    case 43: zeta_pre_kernel<T, 43><<<nb, TPB, 0, st>>>(g, m, y, zeta, Z); break;
    case 63: zeta_pre_kernel<T, 63><<<nb, TPB, 0, st>>>(g, m, y, zeta, Z); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_ad_pre(const FieldGeom& g, const Topology& tp, const double* qw, const T* m,
                          const T* y, const T* zeta, const T* Z, const T* lam, const T* mu, T alpha,
                          T beta, T* A, T* C, cudaStream_t st) {
  ad_pre_kernel<T><<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, tp, qw, m, y, zeta, Z, lam, mu, alpha,
                                                           beta, A, C);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_adsync_gather(const FieldGeom& g, const Topology& tp, const T* m, const T* C,
                                 T* A, cudaStream_t st) {
  const int nb = 6 * (4 * g.n - 4);
  adsync_gather_kernel<T><<<nblk(nb), TPB, 0, st>>>(g, tp, m, C, A, A + g.fs, A + 2 * g.fs,
                                                     A + 3 * g.fs);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_ad_main(const FieldGeom& g, int order, const SbpT& t, const T* m, T ghs, T grav,
                           const T* y, const T* A, T* out, const T* acc_in, T* acc_out,
                           cudaStream_t st) {
  const int nb = nblk(6LL * g.n * g.n);
  switch (order) {
    case 21: ad_main_kernel<T, 21><<<nb, TPB, 0, st>>>(g, t, m, ghs, grav, y, A, out, acc_in, acc_out); break;
    case 42: ad_main_kernel<T, 42><<<nb, TPB, 0, st>>>(g, t, m, ghs, grav, y, A, out, acc_in, acc_out); break;
    case 43: ad_main_kernel<T, 43><<<nb, TPB, 0, st>>>(g, t, m, ghs, grav, y, A, out, acc_in, acc_out); break;
    case 63: ad_main_kernel<T, 63><<<nb, TPB, 0, st>>>(g, t, m, ghs, grav, y, A, out, acc_in, acc_out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

#define SWM_AD_INSTANTIATE(T)                                                                    \
  template cudaError_t launch_zeta_pre<T>(const FieldGeom&, int, const T*, const T*, T*, T*,      \
                                          cudaStream_t);                                          \
  template cudaError_t launch_ad_pre<T>(const FieldGeom&, const Topology&, const double*,        \
                                        const T*, const T*, const T*, const T*, const T*,        \
                                        const T*, T, T, T*, T*, cudaStream_t);                   \
  template cudaError_t launch_adsync_gather<T>(const FieldGeom&, const Topology&, const T*,      \
                                               const T*, T*, cudaStream_t);                      \
  template cudaError_t launch_ad_main<T>(const FieldGeom&, int, const SbpT&, const T*, T, T,     \
                                         const T*, const T*, T*, const T*, T*, cudaStream_t);
SWM_AD_INSTANTIATE(float)
SWM_AD_INSTANTIATE(double)
#undef SWM_AD_INSTANTIATE

int adjoint_table_ct(int order) {
  switch (order) {
    case 21: return AdOrd<21>::CT;
    case 42: return AdOrd<42>::CT;
    case 43: return AdOrd<43>::CT;
    case 63: return AdOrd<63>::CT;
    default: return -1;
  }
}

}  // namespace swm
