// swm_ops.cu -- FP64 geometry precompute, per-operator (unfused) FP64
// kernels, cube-edge syncs on fields, state combinations and deterministic
// FP64 reductions.
#include "swm_ops.cuh"
#include "swm_stage.cuh"

namespace swm {

namespace {

constexpr double kPi = 3.141592653589793238462643383279502884;

// Panel frames (ex, ey, inward normal n) of the six cube faces
// (topology/cubed_sphere_topology_mod.f90:29-55 of the reference).
__constant__ int c_ex[6][3] = {{-1, 0, 0}, {0, 0, -1}, {1, 0, 0}, {0, 0, 1}, {1, 0, 0}, {1, 0, 0}};
__constant__ int c_ey[6][3] = {{0, 1, 0}, {0, 1, 0}, {0, 1, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, -1}};
__constant__ int c_n[6][3] = {{0, 0, 1}, {-1, 0, 0}, {0, 0, -1}, {1, 0, 0}, {0, 1, 0}, {0, -1, 0}};

constexpr int TPB = 256;

inline int nblk(long long count, int tpb = TPB) { return (int)((count + tpb - 1) / tpb); }

// valid node g in [0, 6n^2) -> (p, i, j, pitched index)
struct NodeIx {
  int p, i, j;
  long long idx;
};
__device__ __forceinline__ NodeIx node_of(const FieldGeom& g, long long gi) {
  NodeIx r;
  const long long nn = (long long)g.n * g.n;
  r.p = (int)(gi / nn);
  const long long rem = gi - (long long)r.p * nn;
  r.j = (int)(rem / g.n);
  r.i = (int)(rem - (long long)r.j * g.n);
  r.idx = (long long)r.p * g.ps + (long long)r.j * g.P + r.i;
  return r;
}

// ---------------------------------------------------------------------------
// Geometry: equiangular cubed sphere metric on the unit sphere
// (equiang_cs/ecs_metric_mod.f90:326-478, mesh_factory_mod.f90:85-133,
// coriolis_factory_mod.f90:151-172).  alpha_i = -pi/4 + i*hx, hx = (pi/2)/N.
// ---------------------------------------------------------------------------
__global__ void geometry_kernel(FieldGeom g, double hx, double radius, double omega, double ax,
                                double ay, double az, double* m) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const NodeIx k = node_of(g, gi);
  const double al = -0.25 * kPi + k.i * hx, be = -0.25 * kPi + k.j * hx;
  const double ta = tan(al), tb = tan(be);
  const double sg = sqrt(1.0 + ta * ta + tb * tb);
  const double A = 1.0 + ta * ta, B = 1.0 + tb * tb;
  const double J = A * B / (sg * sg * sg);
  m[MJ * g.fs + k.idx] = J;
  m[MQI1 * g.fs + k.idx] = sg * sg / A;
  m[MQI2 * g.fs + k.idx] = sg * sg * ta * tb / (A * B);
  m[MQI3 * g.fs + k.idx] = sg * sg / B;
  // point on the sphere: proto-face (ta, tb, 1)/sg mapped to panel p
  const double rp[3] = {ta / sg, tb / sg, 1.0 / sg};
  double r[3];
  for (int c = 0; c < 3; ++c)
    r[c] = c_ex[k.p][c] * rp[0] + c_ey[k.p][c] * rp[1] - c_n[k.p][c] * rp[2];
  const double nn = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  m[MF * g.fs + k.idx] = 2.0 * omega * ((ax * r[0] + ay * r[1] + az * r[2]) / nn);
  m[MRJ * g.fs + k.idx] = 1.0 / (J * hx * radius);
}

__device__ void a1p(double a, double b, double v[3]) {
  const double ta = tan(a), tb = tan(b);
  const double p = pow(1.0 + ta * ta + tb * tb, 1.5);
  v[0] = (1.0 + ta * ta) * (1.0 + tb * tb) / p;
  v[1] = -ta * tb * (1.0 + ta * ta) / p;
  v[2] = -ta * (1.0 + ta * ta) / p;
}
__device__ void a2p(double a, double b, double v[3]) {
  const double ta = tan(a), tb = tan(b);
  const double p = pow(1.0 + ta * ta + tb * tb, 1.5);
  v[0] = -ta * tb * (1.0 + tb * tb) / p;
  v[1] = (1.0 + ta * ta) * (1.0 + tb * tb) / p;
  v[2] = -tb * (1.0 + tb * tb) / p;
}
__device__ void b1p(double a, double b, double v[3]) {
  const double ta = tan(a), tb = tan(b);
  const double s = sqrt(1.0 + ta * ta + tb * tb);
  v[0] = (1.0 + tb * tb - (ta * tb) * (ta * tb) / (1.0 + ta * ta)) / s;
  v[1] = 0.0;
  v[2] = -ta * (1.0 + tb * tb / (1.0 + ta * ta)) / s;
}
__device__ void b2p(double a, double b, double v[3]) {
  const double ta = tan(a), tb = tan(b);
  const double s = sqrt(1.0 + ta * ta + tb * tb);
  v[0] = 0.0;
  v[1] = ((1.0 + ta * ta) - (ta * tb) * (ta * tb) / (1.0 + tb * tb)) / s;
  v[2] = -tb * (ta * ta / (1.0 + tb * tb) + 1.0) / s;
}

// Cartesian contravariant basis vectors b1, b2 of every node, mapped from
// the prototype face to panel p (mesh_factory_mod.f90:131-132 with
// ecs_metric_mod.f90 calculate_b1/b2): 6 fields b1x b1y b1z b2x b2y b2z.
__global__ void basis_kernel(FieldGeom g, double hx, double* b) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const NodeIx k = node_of(g, gi);
  const double al = -0.25 * kPi + k.i * hx, be = -0.25 * kPi + k.j * hx;
  double v1[3], v2[3];
  b1p(al, be, v1);
  b2p(al, be, v2);
  for (int c = 0; c < 3; ++c) {
    b[c * g.fs + k.idx] = c_ex[k.p][c] * v1[0] + c_ey[k.p][c] * v1[1] - c_n[k.p][c] * v1[2];
    b[(3 + c) * g.fs + k.idx] = c_ex[k.p][c] * v2[0] + c_ey[k.p][c] * v2[1] - c_n[k.p][c] * v2[2];
  }
}

// Covariant-vector sync weights: dot products of the basis vectors of the
// two panels across each edge (ecs_Ah_vec_sync_factory_mod.f90:97-144).
__global__ void sync_weights_kernel(int n, double hx, double* qw) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double c = -0.25 * kPi + k * hx, q = 0.25 * kPi;
  double a[3], b[3];
  a2p(c, -q, a); b1p(c, q, b);
  qw[k] = a[0] * b[0] + a[1] * (-b[2]) + a[2] * b[1];
  a2p(c, q, a); b1p(c, -q, b);
  qw[n + k] = a[0] * b[0] + a[1] * b[2] + a[2] * (-b[1]);
  a1p(-q, c, a); b2p(q, c, b);
  qw[2 * n + k] = a[0] * (-b[2]) + a[1] * b[1] + a[2] * b[0];
  a1p(q, c, a); b2p(-q, c, b);
  qw[3 * n + k] = a[0] * b[2] + a[1] * b[1] + a[2] * (-b[0]);
}

__global__ void to_f32_kernel(const double* s, float* d, long long count) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < count) d[k] = (float)s[k];
}

// ---------------------------------------------------------------------------
// Per-operator FP64 kernels (reference formulas and operation order).
// ---------------------------------------------------------------------------
__global__ void co2contra_kernel(FieldGeom g, const double* m, const double* u, const double* v,
                                 double* ut, double* vt) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const long long x = node_of(g, gi).idx;
  const double q1 = m[MQI1 * g.fs + x], q2 = m[MQI2 * g.fs + x], q3 = m[MQI3 * g.fs + x];
  const double a = q1 * u[x] + q2 * v[x];
  const double b = q2 * u[x] + q3 * v[x];
  ut[x] = a;
  vt[x] = b;
}

__global__ void massflux_kernel(FieldGeom g, const double* h, const double* ut, const double* vt,
                                double* hu, double* hv) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const long long x = node_of(g, gi).idx;
  hu[x] = 1.0 * h[x] * ut[x];
  hv[x] = 1.0 * h[x] * vt[x];
}

__global__ void ke_kernel(FieldGeom g, const double* u, const double* v, const double* ut,
                          const double* vt, double* ke) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const long long x = node_of(g, gi).idx;
  ke[x] = (u[x] * ut[x] + v[x] * vt[x]) / 2.0;
}

__global__ void ke_update_kernel(FieldGeom g, double grav, const double* h, const double* hs,
                                 double* ke) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const long long x = node_of(g, gi).idx;
  ke[x] = ke[x] + grav * h[x] + grav * (hs ? hs[x] : 0.0);
}

// SBP derivative with a runtime operator index (table in constant memory).
template <class FA>
__device__ __forceinline__ double d_line_rt(int id, int k, int n, FA fa) {
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

__global__ void grad_kernel(FieldGeom g, int id, double ghs, const double* f, double* gx,
                            double* gy) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const NodeIx k = node_of(g, gi);
  const double* F = f + (long long)k.p * g.ps;
  const double dx = d_line_rt(id, k.i, g.n, [&](int m) { return F[(long long)k.j * g.P + m]; });
  const double dy = d_line_rt(id, k.j, g.n, [&](int m) { return F[(long long)m * g.P + k.i]; });
  gx[k.idx] = dx * ghs;
  gy[k.idx] = dy * ghs;
}

__global__ void div_kernel(FieldGeom g, int id, double hx_a, const double* mt, const double* u,
                           const double* v, int curl_form, double* out) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const NodeIx k = node_of(g, gi);
  const long long pb = (long long)k.p * g.ps;
  const double* J = mt + MJ * g.fs + pb;
  const double* U = u + pb;
  const double* V = v + pb;
  // Gu = J*u, Gv = J*v; for the curl, (u', v') = (v/J, -u/J) first
  auto gu = [&](long long o) { return curl_form ? J[o] * (V[o] / J[o]) : J[o] * U[o]; };
  auto gv = [&](long long o) { return curl_form ? J[o] * (-U[o] / J[o]) : J[o] * V[o]; };
  const double dx = d_line_rt(id, k.i, g.n, [&](int m) { return gu((long long)k.j * g.P + m); });
  const double dy = d_line_rt(id, k.j, g.n, [&](int m) { return gv((long long)m * g.P + k.i); });
  out[k.idx] = (dx + dy) / (mt[MJ * g.fs + k.idx] * hx_a);
}

__global__ void coriolis_kernel(FieldGeom g, const double* m, const double* hu, const double* hv,
                                const double* h, const double* cu, double* cor_u, double* cor_v) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const long long x = node_of(g, gi).idx;
  const double fz = m[MF * g.fs + x] + cu[x];
  const double J = m[MJ * g.fs + x];
  cor_u[x] = fz * hv[x] / h[x] * J;
  cor_v[x] = -(fz * hu[x] / h[x] * J);
}

__global__ void fill_kernel(long long count, double value, double* out) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < count) out[k] = value;
}

__global__ void axpby_kernel(long long count, double s1, const double* a, double s2,
                             const double* b, double* out) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  out[k] = b ? s1 * a[k] + s2 * b[k] : s1 * a[k];
}

// gather boundary values of up to two fields into edge slots v0 (and v1)
template <class T>
__global__ void gather_edge_kernel(FieldGeom g, const T* f0, int v0, const T* f1, int v1, T* E) {
  const int n = g.n, nb = 4 * n - 4;
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6 * nb) return;
  const int p = gi / nb;
  int i, j;
  boundary_node(gi - p * nb, n, i, j);
  const long long x = (long long)p * g.ps + (long long)j * g.P + i;
  const T a = f0[x], b = f1 ? f1[x] : T(0);
  auto put = [&](int side, int k) {
    E[((long long)(p * 4 + side) * 4 + v0) * n + k] = a;
    if (f1) E[((long long)(p * 4 + side) * 4 + v1) * n + k] = b;
  };
  if (i == 0) put(SIDE_L, j);
  if (i == n - 1) put(SIDE_R, j);
  if (j == 0) put(SIDE_B, i);
  if (j == n - 1) put(SIDE_T, i);
}

template <class T>
__global__ void sync_scalar_kernel(FieldGeom g, Topology tp, const T* E, T* f) {
  const int n = g.n, nb = 4 * n - 4;
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6 * nb) return;
  const int p = gi / nb;
  int i, j;
  boundary_node(gi - p * nb, n, i, j);
  const long long x = (long long)p * g.ps + (long long)j * g.P + i;
  const EdgeView<T> ev{E, n};
  f[x] = sync_scalar_node<T>(ev, tp, p, i, j, EV_ZETA, f[x]);
}

template <class T>
__global__ void sync_vector_kernel(FieldGeom g, Topology tp, const double* qw, const T* E, T* gx,
                                   T* gy) {
  const int n = g.n, nb = 4 * n - 4;
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6 * nb) return;
  const int p = gi / nb;
  int i, j;
  boundary_node(gi - p * nb, n, i, j);
  const long long x = (long long)p * g.ps + (long long)j * g.P + i;
  const EdgeView<T> ev{E, n};
  T a = gx[x], b = gy[x];
  sync_vector_node<T>(ev, tp, qw, p, i, j, a, b);
  gx[x] = a;
  gy[x] = b;
}

// ---------------------------------------------------------------------------
// Deterministic reductions: fixed grid, per-block tree, then one block sums
// the partials in a fixed order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double red_op(int kind, double x, double y) {
  return kind == 2 ? fmin(x, y) : kind == 3 ? fmax(x, y) : x + y;
}

__global__ void reduce_partial_kernel(FieldGeom g, int kind, const double* a, const double* b,
                                      const double* J, const double* Aw, double hx2,
                                      double* partial) {
  __shared__ double sh[TPB];
  const long long total = 6LL * g.n * g.n;
  const double init = kind == 2 ? INFINITY : kind == 3 ? -INFINITY : 0.0;
  double acc = init;
  for (long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x; gi < total;
       gi += (long long)gridDim.x * blockDim.x) {
    const NodeIx k = node_of(g, gi);
    double val = a[k.idx];
    if (kind == 0 && b) val = val * b[k.idx];
    if (kind == 1 || kind == 4) {
      if (kind == 4) val = val * b[k.idx];
      val = val * J[k.idx] * hx2 * Aw[k.i] * Aw[k.j];
    }
    acc = red_op(kind, acc, val);
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = TPB / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = red_op(kind, sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void reduce_final_kernel(int kind, const double* partial, int np, double* result) {
  __shared__ double sh[TPB];
  const double init = kind == 2 ? INFINITY : kind == 3 ? -INFINITY : 0.0;
  double acc = init;
  for (int k = threadIdx.x; k < np; k += blockDim.x) acc = red_op(kind, acc, partial[k]);
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = TPB / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = red_op(kind, sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *result = sh[0];
}

__global__ void diag_kernel(FieldGeom g, const double* m, double grav, const double* h,
                            const double* u, const double* v, const double* hs, const double* z,
                            double* ke_u, double* ke_v, double* pe, double* ens) {
  const long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= 6LL * g.n * g.n) return;
  const long long x = node_of(g, gi).idx;
  const double q1 = m[MQI1 * g.fs + x], q2 = m[MQI2 * g.fs + x], q3 = m[MQI3 * g.fs + x];
  const double ut = q1 * u[x] + q2 * v[x];
  const double vt = q2 * u[x] + q3 * v[x];
  const double hu = 1.0 * h[x] * ut, hv = 1.0 * h[x] * vt;
  ke_u[x] = 0.5 * hu * u[x];
  ke_v[x] = 0.5 * hv * v[x];
  const double ph = 1.0 * h[x] + 1.0 * (hs ? hs[x] : 0.0);
  pe[x] = 0.5 * grav * ph * ph;
  double c = z[x] + 1.0 * m[MF * g.fs + x];
  c = 0.5 * c * c;
  ens[x] = 1.0 * c / h[x];
}

// ---------------------------------------------------------------------------
// FP32 (hi, lo) pair helpers
// ---------------------------------------------------------------------------
// FP32 (hi, lo) pairs combined in double-float arithmetic: error-free
// two-sum and two-product (fmaf), then renormalisation; the coefficients
// come split into float pairs.  FP32 instructions only (GB300's FP64 rate
// would bound an FP64 evaluation); about 2^-44 relative accuracy.
__device__ __forceinline__ void quick_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void df_mul(float xh, float xl, float yh, float yl, float& h, float& l) {
  const float p = xh * yh;
  float e = fmaf(xh, yh, -p);
  e = fmaf(xh, yl, e);
  e = fmaf(xl, yh, e);
  quick_two_sum(p, e, h, l);
}
__device__ __forceinline__ void df_add(float ah, float al, float bh, float bl, float& h, float& l) {
  float sm, e;
  two_sum(ah, bh, sm, e);
  e += al + bl;
  quick_two_sum(sm, e, h, l);
}

__global__ void axpby_pair_kernel(long long count, float s1h, float s1l, const float* ahi,
                                  const float* alo, float s2h, float s2l, const float* bhi,
                                  const float* blo, float* ohi, float* olo) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  float h, l;
  df_mul(s1h, s1l, ahi[k], alo[k], h, l);
  if (bhi) {
    float h2, l2;
    df_mul(s2h, s2l, bhi[k], blo[k], h2, l2);
    df_add(h, l, h2, l2, h, l);
  }
  ohi[k] = h;
  olo[k] = l;
}

__global__ void fill_pair_kernel(long long count, float vh, float vl, float* ohi, float* olo) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  ohi[k] = vh;
  olo[k] = vl;
}

__global__ void split_kernel(long long count, const double* s, float* hi, float* lo) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const float h = (float)s[k];
  hi[k] = h;
  lo[k] = (float)(s[k] - (double)h);
}

__global__ void join_kernel(long long count, const float* hi, const float* lo, double* d) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  d[k] = (double)hi[k] + (double)lo[k];
}

// Packed <-> pitched state fields.  Thread k handles packed value k of the
// nf fields (k = c*6*n*n + (p*n + j)*n + i), so a warp touches 32
// consecutive packed doubles: whole 128-byte lines of the packed side, which
// may sit in host memory behind the host-device link.  The state fields hold
// n*P pitched rows per panel (ps = n*P).  Indices fit 32 bits for n <= 8191.
__device__ __forceinline__ void packed_index(const FieldGeom& g, unsigned k, unsigned& c,
                                             unsigned& r, long long& o) {
  const unsigned n = (unsigned)g.n, nn6 = 6u * n * n;
  c = k / nn6;
  r = k - c * nn6;
  const unsigned row = r / n;
  o = (long long)c * g.fs + (long long)row * g.P + (r - row * n);
}

__device__ __forceinline__ double* field_of(const PackedFields& pf, unsigned c) {
  return c == 0 ? pf.f[0] : (c == 1 ? pf.f[1] : pf.f[2]);
}

template <class T>
__global__ void unpack_kernel(FieldGeom g, unsigned total, PackedFields src, T* hi, float* lo) {
  const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= total) return;
  unsigned c, r;
  long long o;
  packed_index(g, k, c, r, o);
  const double x = field_of(src, c)[r];
  if constexpr (sizeof(T) == 8) {
    hi[o] = x;
  } else {
    const float h = (float)x;
    hi[o] = h;
    lo[o] = (float)(x - (double)h);
  }
}

template <class T>
__global__ void pack_kernel(FieldGeom g, unsigned total, const T* hi, const float* lo,
                            PackedFields dst) {
  const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= total) return;
  unsigned c, r;
  long long o;
  packed_index(g, k, c, r, o);
  double x;
  if constexpr (sizeof(T) == 8) x = hi[o];
  else x = (double)hi[o] + (double)lo[o];
  field_of(dst, c)[r] = x;
}

}  // namespace

// ===========================================================================
// launchers
// ===========================================================================
cudaError_t launch_geometry(const FieldGeom& g, int N, double radius, double omega,
                            const double axis[3], double* m64, double* qw, cudaStream_t st) {
  const double hx = (0.25 * kPi - (-0.25 * kPi)) / (double)N;
  const double an = sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
  geometry_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, hx, radius, omega, axis[0] / an,
                                                          axis[1] / an, axis[2] / an, m64);
  sync_weights_kernel<<<nblk(g.n), TPB, 0, st>>>(g.n, hx, qw);
  return cudaGetLastError();
}

cudaError_t launch_basis(const FieldGeom& g, double hx, double* b, cudaStream_t st) {
  basis_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, hx, b);
  return cudaGetLastError();
}

cudaError_t launch_to_f32(const double* src, float* dst, long long count, cudaStream_t st) {
  to_f32_kernel<<<nblk(count), TPB, 0, st>>>(src, dst, count);
  return cudaGetLastError();
}

cudaError_t launch_co2contra(const FieldGeom& g, const double* m64, const double* u,
                             const double* v, double* ut, double* vt, cudaStream_t st) {
  co2contra_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, m64, u, v, ut, vt);
  return cudaGetLastError();
}

cudaError_t launch_massflux(const FieldGeom& g, const double* h, const double* ut,
                            const double* vt, double* hu, double* hv, cudaStream_t st) {
  massflux_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, h, ut, vt, hu, hv);
  return cudaGetLastError();
}

cudaError_t launch_ke(const FieldGeom& g, const double* u, const double* v, const double* ut,
                      const double* vt, double* ke, cudaStream_t st) {
  ke_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, u, v, ut, vt, ke);
  return cudaGetLastError();
}

cudaError_t launch_ke_update(const FieldGeom& g, double grav, const double* h, const double* hs,
                             double* ke, cudaStream_t st) {
  ke_update_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, grav, h, hs, ke);
  return cudaGetLastError();
}

cudaError_t launch_grad_presync(const FieldGeom& g, int order, double ghs, const double* f,
                                double* gx, double* gy, cudaStream_t st) {
  grad_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, sbp_index(order), ghs, f, gx, gy);
  return cudaGetLastError();
}

cudaError_t launch_div_presync(const FieldGeom& g, int order, double hx_a, const double* m64,
                               const double* u, const double* v, int curl_form, double* out,
                               cudaStream_t st) {
  div_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, sbp_index(order), hx_a, m64, u, v,
                                                     curl_form, out);
  return cudaGetLastError();
}

cudaError_t launch_coriolis(const FieldGeom& g, const double* m64, const double* hu,
                            const double* hv, const double* h, const double* curl, double* cor_u,
                            double* cor_v, cudaStream_t st) {
  coriolis_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, m64, hu, hv, h, curl, cor_u, cor_v);
  return cudaGetLastError();
}

cudaError_t launch_fill(long long count, double value, double* out, cudaStream_t st) {
  fill_kernel<<<nblk(count), TPB, 0, st>>>(count, value, out);
  return cudaGetLastError();
}

cudaError_t launch_axpby(long long count, double s1, const double* a, double s2, const double* b,
                         double* out, cudaStream_t st) {
  axpby_kernel<<<nblk(count), TPB, 0, st>>>(count, s1, a, s2, b, out);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_sync_scalar_t(const FieldGeom& g, const Topology& tp, T* f, T* edge,
                                 cudaStream_t st) {
  const int nb = 6 * (4 * g.n - 4);
  gather_edge_kernel<T><<<nblk(nb), TPB, 0, st>>>(g, f, EV_ZETA, nullptr, 0, edge);
  sync_scalar_kernel<T><<<nblk(nb), TPB, 0, st>>>(g, tp, edge, f);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_sync_vector_t(const FieldGeom& g, const Topology& tp, const double* qw, T* gx,
                                 T* gy, T* edge, cudaStream_t st) {
  const int nb = 6 * (4 * g.n - 4);
  gather_edge_kernel<T><<<nblk(nb), TPB, 0, st>>>(g, gx, EV_GX, gy, EV_GY, edge);
  sync_vector_kernel<T><<<nblk(nb), TPB, 0, st>>>(g, tp, qw, edge, gx, gy);
  return cudaGetLastError();
}
template cudaError_t launch_sync_scalar_t<float>(const FieldGeom&, const Topology&, float*, float*,
                                                 cudaStream_t);
template cudaError_t launch_sync_scalar_t<double>(const FieldGeom&, const Topology&, double*,
                                                  double*, cudaStream_t);
template cudaError_t launch_sync_vector_t<float>(const FieldGeom&, const Topology&, const double*,
                                                 float*, float*, float*, cudaStream_t);
template cudaError_t launch_sync_vector_t<double>(const FieldGeom&, const Topology&, const double*,
                                                  double*, double*, double*, cudaStream_t);

cudaError_t launch_sync_scalar(const FieldGeom& g, const Topology& tp, double* f, double* edge,
                               cudaStream_t st) {
  return launch_sync_scalar_t<double>(g, tp, f, edge, st);
}

cudaError_t launch_sync_vector(const FieldGeom& g, const Topology& tp, const double* qw,
                               double* gx, double* gy, double* edge, cudaStream_t st) {
  return launch_sync_vector_t<double>(g, tp, qw, gx, gy, edge, st);
}

cudaError_t launch_reduce(const FieldGeom& g, int kind, const double* a, const double* b,
                          const double* J, const double* Aw, double hx2, double* partial,
                          int nblocks, double* result, cudaStream_t st) {
  reduce_partial_kernel<<<nblocks, TPB, 0, st>>>(g, kind, a, b, J, Aw, hx2, partial);
  reduce_final_kernel<<<1, TPB, 0, st>>>(kind, partial, nblocks, result);
  return cudaGetLastError();
}

cudaError_t launch_diag_integrands(const FieldGeom& g, const double* m64, double grav,
                                   const double* h, const double* u, const double* v,
                                   const double* hs, const double* zeta, double* ke_u,
                                   double* ke_v, double* pe, double* ens, cudaStream_t st) {
  diag_kernel<<<nblk(6LL * g.n * g.n), TPB, 0, st>>>(g, m64, grav, h, u, v, hs, zeta, ke_u, ke_v,
                                                      pe, ens);
  return cudaGetLastError();
}

cudaError_t launch_axpby_f32pair(long long count, double s1, const float* ahi, const float* alo,
                                 double s2, const float* bhi, const float* blo, float* ohi,
                                 float* olo, cudaStream_t st) {
  const float s1h = (float)s1, s1l = (float)(s1 - (double)s1h);
  const float s2h = (float)s2, s2l = (float)(s2 - (double)s2h);
  axpby_pair_kernel<<<nblk(count), TPB, 0, st>>>(count, s1h, s1l, ahi, alo, s2h, s2l, bhi, blo, ohi,
                                                 olo);
  return cudaGetLastError();
}

cudaError_t launch_fill_f32pair(long long count, double value, float* ohi, float* olo,
                                cudaStream_t st) {
  const float vh = (float)value, vl = (float)(value - (double)vh);
  fill_pair_kernel<<<nblk(count), TPB, 0, st>>>(count, vh, vl, ohi, olo);
  return cudaGetLastError();
}

cudaError_t launch_split_f64(long long count, const double* src, float* hi, float* lo,
                             cudaStream_t st) {
  split_kernel<<<nblk(count), TPB, 0, st>>>(count, src, hi, lo);
  return cudaGetLastError();
}

cudaError_t launch_join_f32pair(long long count, const float* hi, const float* lo, double* dst,
                                cudaStream_t st) {
  join_kernel<<<nblk(count), TPB, 0, st>>>(count, hi, lo, dst);
  return cudaGetLastError();
}

cudaError_t launch_unpack_state(const FieldGeom& g, int nf, const PackedFields& src, void* hi,
                                float* lo, cudaStream_t st) {
  if (nf < 1 || nf > 3 || g.n > 8191) return cudaErrorInvalidValue;
  const unsigned total = (unsigned)(nf * 6LL * g.n * g.n);
  if (lo) unpack_kernel<float><<<nblk(total), TPB, 0, st>>>(g, total, src, (float*)hi, lo);
  else unpack_kernel<double><<<nblk(total), TPB, 0, st>>>(g, total, src, (double*)hi, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_pack_state(const FieldGeom& g, int nf, const void* hi, const float* lo,
                              const PackedFields& dst, cudaStream_t st) {
  if (nf < 1 || nf > 3 || g.n > 8191) return cudaErrorInvalidValue;
  const unsigned total = (unsigned)(nf * 6LL * g.n * g.n);
  if (lo) pack_kernel<float><<<nblk(total), TPB, 0, st>>>(g, total, (const float*)hi, lo, dst);
  else pack_kernel<double><<<nblk(total), TPB, 0, st>>>(g, total, (const double*)hi, nullptr, dst);
  return cudaGetLastError();
}

}  // namespace swm
