// swm_oracle.cpp -- FP64 CPU oracle for the shallow-water hot path.
//
// TEST INFRASTRUCTURE ONLY (see swm_oracle.h).  This file restates, in plain
// C++, the algorithms of the reference Fortran code (vvshashkin/
// cubedsphere_sbp_swm); every routine names the reference file:line it
// follows.  It keeps the reference's evaluation order where that is cheap
// (SBP row sums left to right, the corner "/3" averages, the two-part RK4
// update) so that the oracle reproduces the reference's printed golden
// numbers.  OpenMP parallelises the field loops over panel rows for the timed
// CPU baseline; every result is independent of the thread count (no parallel
// floating-point reductions).

#include "swm_oracle.h"
#include "swm_oracle_common.h"
#include "../cubedsphere_sbp_swm_gb300/csrc/swm_narrow_tables.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using namespace orc_common;

// ---------------------------------------------------------------------------
// SBP first-derivative operators (sbp_operators_collection_mod.f90:15-85,
// sbp_factory_mod.f90:38-179).  Ql[r][m] multiplies f[m] for left closure row
// r (0-based); the right block is the sign-flipped mirror.
// ---------------------------------------------------------------------------
struct Sbp {
  int ne = 0, nw = 0;
  std::vector<double> Ql;   // ne*nw
  std::vector<int> last;    // nonzero count per closure row
  std::vector<double> Qin;  // interior stencil
  int inshift = 0;
  std::vector<double> A;    // diagonal norm (quadrature) edge weights
};

Sbp make_sbp(int order) {
  Sbp s;
  if (order == 21) {
    s.ne = 1; s.nw = 2;
    s.Ql = {-1.0, 1.0};
    s.last = {2};
    s.Qin = {-0.5, 0.0, 0.5}; s.inshift = -1;
    s.A = {0.5, 1.0};
  } else if (order == 42) {
    s.ne = 4; s.nw = 6;
    s.Ql = {-1.4117647058823528, 1.7352941176470589, -0.2352941176470588, -0.08823529411764705, 0.0, 0.0,
            -0.5, 0.0, 0.5, 0.0, 0.0, 0.0,
            0.09302325581395347, -0.686046511627907, 0.0, 0.686046511627907, -0.09302325581395347, 0.0,
            0.030612244897959186, -0.0, -0.6020408163265307, 0.0, 0.653061224489796, -0.0816326530612245};
    s.last = {4, 3, 5, 6};
    s.Qin = {1.0 / 12.0, -2.0 / 3.0, 0.0, 2.0 / 3.0, -1.0 / 12.0}; s.inshift = -2;
    s.A = {17.0 / 48.0, 59.0 / 48.0, 43.0 / 48.0, 49.0 / 48.0};
  } else if (order == 43) {
    s.ne = 4; s.nw = 6;
    s.Ql = {-1.8280236842718398, 2.978054584697369, -1.4653148294044123, 0.3078538227474199, 0.008136925288119662, -0.0007068190566565205,
            -0.37814159126691327, -0.31480210500706657, 0.707290999364066, 0.04835554461933453, -0.06866771096803422, 0.005964863258613564,
            0.1162478575921292, -0.8028500807354999, 0.21558841368737428, 0.5078566674295846, -0.03231754093993847, -0.004525317033649745,
            -0.010287398573128293, 0.12592344801071614, -0.7341531396449149, 0.04979271660173103, 0.6506171865540596, -0.08189281294846368};
    s.last = {6, 6, 6, 6};
    s.Qin = {1.0 / 12.0, -2.0 / 3.0, 0.0, 2.0 / 3.0, -1.0 / 12.0}; s.inshift = -2;
    s.A = {17.0 / 48.0, 59.0 / 48.0, 43.0 / 48.0, 49.0 / 48.0};
  } else if (order == 63) {
    // Sixth-order interior / third-order boundary closure with one free
    // parameter q56, assembled from its rational entries exactly as the
    // reference parameter block does.
    const double A1 = 13649.0 / 43200.0, A2 = 12013.0 / 8640.0, A3 = 2711.0 / 4320.0,
                 A4 = 5359.0 / 4320.0, A5 = 7877.0 / 8640.0, A6 = 43801.0 / 43200.0;
    const double q56 = 5591070156686698065364559.0 / 7931626489314500743872000.0;
    const double q11 = -1.0 / 2.0;
    const double q12 = -953.0 / 16200.0 + q56;
    const double q13 = 715489.0 / 259200.0 - (4.0 * q56);
    const double q14 = -62639.0 / 14400.0 + (6.0 * q56);
    const double q15 = 147127.0 / 51840.0 - (4.0 * q56);
    const double q16 = -89387.0 / 129600.0 + q56;
    const double q23 = -57139.0 / 8640.0 + (10.0 * q56);
    const double q24 = 745733.0 / 51840.0 - (20.0 * q56);
    const double q25 = -18343.0 / 1728.0 + (15.0 * q56);
    const double q26 = 240569.0 / 86400.0 - (4.0 * q56);
    const double q34 = -176839.0 / 12960.0 + (20.0 * q56);
    const double q35 = 242111.0 / 17280.0 - (20.0 * q56);
    const double q36 = -182261.0 / 43200.0 + (6.0 * q56);
    const double q45 = -165041.0 / 25920.0 + (10.0 * q56);
    const double q46 = 710473.0 / 259200.0 - (4.0 * q56);
    const double q47 = 1.0 / 60.0, q57 = -3.0 / 20.0, q58 = 1.0 / 60.0;
    const double q67 = 3.0 / 4.0, q68 = -3.0 / 20.0, q69 = 1.0 / 60.0;
    s.ne = 6; s.nw = 9;
    s.Ql = {q11 / A1, q12 / A1, q13 / A1, q14 / A1, q15 / A1, q16 / A1, 0.0, 0.0, 0.0,
            -q12 / A2, 0.0, q23 / A2, q24 / A2, q25 / A2, q26 / A2, 0.0, 0.0, 0.0,
            -q13 / A3, -q23 / A3, 0.0, q34 / A3, q35 / A3, q36 / A3, 0.0, 0.0, 0.0,
            -q14 / A4, -q24 / A4, -q34 / A4, 0.0, q45 / A4, q46 / A4, q47 / A4, 0.0, 0.0,
            -q15 / A5, -q25 / A5, -q35 / A5, -q45 / A5, 0.0, q56 / A5, q57 / A5, q58 / A5, 0.0,
            -q16 / A6, -q26 / A6, -q36 / A6, -q46 / A6, -q56 / A6, 0.0, q67 / A6, q68 / A6, q69 / A6};
    s.last = {6, 6, 6, 7, 8, 9};
    s.Qin = {-1.0 / 60.0, 3.0 / 20.0, -3.0 / 4.0, 0.0, 3.0 / 4.0, -3.0 / 20.0, 1.0 / 60.0};
    s.inshift = -3;
    s.A = {A1, A2, A3, A4, A5, A6};
  }
  return s;
}

// sbp_apply (sbp_operator_mod.f90:152-228) along one line of n values with
// stride st: out[k] for k in [0,n).
inline double sbp_point(const Sbp& s, const double* f, int n, int st, int k) {
  double acc = 0.0;
  if (k < s.ne) {
    const double* q = &s.Ql[k * s.nw];
    for (int m = 0; m < s.last[k]; ++m) acc += q[m] * f[m * st];
  } else if (k < n - s.ne) {
    const int w = (int)s.Qin.size();
    for (int t = 0; t < w; ++t) acc += s.Qin[t] * f[(k + s.inshift + t) * st];
  } else {
    // mirrored right block, summed from the outermost tap inwards like the
    // reference's Qr(nwst:nw) * f(mx:n)
    const int r = n - 1 - k;
    const double* q = &s.Ql[r * s.nw];
    for (int m = s.last[r] - 1; m >= 0; --m) acc += (-q[m]) * f[(n - 1 - m) * st];
  }
  return acc;
}


// Halo ring slot: side 0 = i=0 (left), 1 = i=n+1 (right), 2 = j=0 (bottom),
// 3 = j=n+1 (top); position k = 0..n-1 along the side.
struct RingSrc {
  int q;            // sender panel
  int node;         // sender node index within its panel (j*n+i)
  int istep, jstep;
  bool dim_i;
};

}  // namespace

struct orc_domain {
  int N = 0, n = 0, order = 42;
  double hx = 0.0, scale = 1.0, grav = 9.80616, omega = 1.0, axis[3] = {0, 0, 1};
  Sbp sbp;
  std::vector<double> A;                // quadrature weights per line index (n)
  std::vector<double> J, Qi1, Qi2, Qi3, Q1, Q2, Q3, f, rx, ry, rz;
  std::vector<double> a1, a2, b1, b2;   // 3 per node
  std::vector<double> qb, qt, ql, qr;   // covariant sync weights
  std::vector<RingSrc> ring;            // [p][side][k]
  int npts() const { return 6 * n * n; }
  // Work arrays of the operators and of RK4, allocated on first use and kept
  // (the reference's operator owns its work fields the same way), so a timed
  // step does not pay for fresh pages.
  // The slot table has a fixed size, so references to slots stay valid.
  static constexpr int kWorkSlots = 24;
  mutable std::vector<double> ws[kWorkSlots];
  std::vector<double>& work(int slot, size_t len) const {
    if (ws[slot].size() != len) ws[slot].assign(len, 0.0);
    return ws[slot];
  }
};
enum { W_UT = 0, W_VT, W_HU, W_HV, W_KE, W_GX, W_GY, W_CU, W_CORU, W_CORV, W_DV,
       W_CURL_U, W_CURL_V, W_GU, W_GV, W_K1, W_K2, W_K3, W_K4, W_Y, W_RING, W_RING_U, W_RING_V,
       W_COUNT };
static_assert(W_COUNT <= orc_domain::kWorkSlots, "oracle work slots");

namespace {

int g_threads = 1;

double alpha_of(const orc_domain& d, int i0) { return -0.25 * PI + i0 * d.hx; }

void build_ring(orc_domain& d) {
  const int n = d.n;
  d.ring.assign(6 * 4 * n, RingSrc{-1, -1, 0, 0, true});
  for (int p = 0; p < 6; ++p) {
    for (int q = 0; q < 6; ++q) {
      if (q == p) continue;
      int istep, jstep; bool dim_i;
      basis_orientation(p, q, istep, jstep, dim_i);
      for (int js = 1; js <= n; ++js)
        for (int is = 1; is <= n; ++is) {
          if (is != 1 && is != n && js != 1 && js != n) continue;
          int it, jt;
          transform_index(q, is, js, p, n, n, it, jt);
          int side = -1, k = -1;
          if (it == 0 && jt >= 1 && jt <= n) { side = 0; k = jt - 1; }
          else if (it == n + 1 && jt >= 1 && jt <= n) { side = 1; k = jt - 1; }
          else if (jt == 0 && it >= 1 && it <= n) { side = 2; k = it - 1; }
          else if (jt == n + 1 && it >= 1 && it <= n) { side = 3; k = it - 1; }
          if (side < 0) continue;
          d.ring[(p * 4 + side) * n + k] = RingSrc{q, (js - 1) * n + (is - 1), istep, jstep, dim_i};
        }
    }
  }
  for (const RingSrc& r : d.ring)
    if (r.q < 0) std::abort();  // every ring slot has exactly one sender
}

void build(orc_domain& d, int N, int order, double radius, double grav, double omega,
           const double axis[3]) {
  d.N = N; d.n = N + 1; d.order = order;
  d.scale = radius; d.grav = grav; d.omega = omega;
  const double an = std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
  for (int c = 0; c < 3; ++c) d.axis[c] = axis[c] / an;
  d.hx = (0.25 * PI - (-0.25 * PI)) / (double)N;
  d.sbp = make_sbp(order);
  // quadrature edge weights: Ah21 / Ah42 / Ah63 (d43 has no norm of its own
  // in the reference and is paired with SBP_Ah42_quadrature)
  Sbp qs = make_sbp(order == 43 ? 42 : order);
  const int n = d.n, ne = (int)qs.A.size();
  d.A.assign(n, 1.0);
  for (int i = 0; i < std::min(ne, n); ++i) d.A[i] = qs.A[i];
  for (int i = std::max(n - ne, 0); i < n; ++i) d.A[i] = qs.A[n - 1 - i];

  const int np = d.npts();
  for (auto* v : {&d.J, &d.Qi1, &d.Qi2, &d.Qi3, &d.Q1, &d.Q2, &d.Q3, &d.f, &d.rx, &d.ry, &d.rz}) v->assign(np, 0.0);
  for (auto* v : {&d.a1, &d.a2, &d.b1, &d.b2}) v->assign(3 * np, 0.0);
  for (int p = 0; p < 6; ++p)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const int id = p * n * n + j * n + i;
        const double al = alpha_of(d, i), be = alpha_of(d, j);
        const double ta = std::tan(al), tb = std::tan(be);
        const double sg = std::sqrt(1.0 + ta * ta + tb * tb);
        d.J[id] = (1.0 + ta * ta) * (1.0 + tb * tb) / (sg * sg * sg);
        d.Qi1[id] = sg * sg / (1.0 + ta * ta);
        d.Qi2[id] = sg * sg * ta * tb / ((1.0 + ta * ta) * (1.0 + tb * tb));
        d.Qi3[id] = sg * sg / (1.0 + tb * tb);
        const double s4 = (sg * sg) * (sg * sg);
        d.Q1[id] = (1.0 + ta * ta) * (1.0 + ta * ta) * (1.0 + tb * tb) / s4;
        d.Q2[id] = -(1.0 + ta * ta) * (1.0 + tb * tb) * ta * tb / s4;
        d.Q3[id] = (1.0 + ta * ta) * (1.0 + tb * tb) * (1.0 + tb * tb) / s4;
        double v[3], w[3];
        r_proto(al, be, v); to_face(p, v, w);
        d.rx[id] = w[0]; d.ry[id] = w[1]; d.rz[id] = w[2];
        const double nn = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        const double pr = (d.axis[0] * w[0] + d.axis[1] * w[1] + d.axis[2] * w[2]) / nn;
        d.f[id] = 2.0 * d.omega * pr;
        a1_proto(al, be, v); to_face(p, v, &d.a1[3 * id]);
        a2_proto(al, be, v); to_face(p, v, &d.a2[3 * id]);
        b1_proto(al, be, v); to_face(p, v, &d.b1[3 * id]);
        b2_proto(al, be, v); to_face(p, v, &d.b2[3 * id]);
      }

  // covariant sync weights (ecs_Ah_vec_sync_factory_mod.f90:97-144)
  d.qb.assign(n, 0.0); d.qt.assign(n, 0.0); d.ql.assign(n, 0.0); d.qr.assign(n, 0.0);
  for (int k = 0; k < n; ++k) {
    const double c = -0.25 * PI + k * d.hx;
    double a[3], b[3];
    a2_proto(c, -0.25 * PI, a); b1_proto(c, 0.25 * PI, b);
    d.qb[k] = a[0] * b[0] + a[1] * (-b[2]) + a[2] * b[1];
    a2_proto(c, 0.25 * PI, a); b1_proto(c, -0.25 * PI, b);
    d.qt[k] = a[0] * b[0] + a[1] * b[2] + a[2] * (-b[1]);
    a1_proto(-0.25 * PI, c, a); b2_proto(0.25 * PI, c, b);
    d.ql[k] = a[0] * (-b[2]) + a[1] * b[1] + a[2] * b[0];
    a1_proto(0.25 * PI, c, a); b2_proto(-0.25 * PI, c, b);
    d.qr[k] = a[0] * b[2] + a[1] * b[1] + a[2] * (-b[0]);
  }
  build_ring(d);
}

// ---------------------------------------------------------------------------
// Halo exchange of the 1-wide ring (parallel/exchange_halo_mod.f90:42-167,
// parallel/buffer_mod.f90:48-277): scalar copy, or the vector copy with the
// component swap/negation of pack_to_buf_vec.
// ---------------------------------------------------------------------------
void exchange_scalar(const orc_domain& d, const double* f, std::vector<double>& ring) {
  const int n = d.n;
  ring.assign(6 * 4 * n, 0.0);
  for (int s = 0; s < 6 * 4 * n; ++s) {
    const RingSrc& r = d.ring[s];
    ring[s] = f[r.q * n * n + r.node];
  }
}

void exchange_vector(const orc_domain& d, const double* u, const double* v,
                     std::vector<double>& ru, std::vector<double>& rv) {
  const int n = d.n;
  ru.assign(6 * 4 * n, 0.0); rv.assign(6 * 4 * n, 0.0);
  for (int s = 0; s < 6 * 4 * n; ++s) {
    const RingSrc& r = d.ring[s];
    const double uq = u[r.q * n * n + r.node], vq = v[r.q * n * n + r.node];
    if (r.dim_i) { ru[s] = r.istep * uq; rv[s] = r.jstep * vq; }
    else { ru[s] = r.jstep * vq; rv[s] = r.istep * uq; }
  }
}

// Scalar edge/corner averaging (halo/halo_Ah_scalar_sync_mod.f90:38-93).
void sync_scalar(const orc_domain& d, double* f) {
  const int n = d.n;
  std::vector<double>& ring = d.work(W_RING, 6 * 4 * n);
  exchange_scalar(d, f, ring);
  for (int p = 0; p < 6; ++p) {
    double* F = f + p * n * n;
    const double* L = &ring[(p * 4 + 0) * n];
    const double* R = &ring[(p * 4 + 1) * n];
    const double* B = &ring[(p * 4 + 2) * n];
    const double* T = &ring[(p * 4 + 3) * n];
    auto at = [&](int i, int j) -> double& { return F[j * n + i]; };
    const int e = n - 1;
    at(0, 0) = (at(0, 0) + L[0] + B[0]) / 3.0;
    for (int j = 1; j < e; ++j) at(0, j) = 0.5 * (L[j] + at(0, j));
    at(0, e) = (at(0, e) + L[e] + T[0]) / 3.0;
    at(e, 0) = (at(e, 0) + R[0] + B[e]) / 3.0;
    for (int j = 1; j < e; ++j) at(e, j) = 0.5 * (at(e, j) + R[j]);
    at(e, e) = (at(e, e) + R[e] + T[e]) / 3.0;
    for (int i = 1; i < e; ++i) at(i, 0) = 0.5 * (at(i, 0) + B[i]);
    for (int i = 1; i < e; ++i) at(i, e) = 0.5 * (at(i, e) + T[i]);
  }
}

// Covariant vector edge sync: syncronize_grad_on_edges called with the
// components swapped (ecs_Ah_vec_sync_mod.f90:34-125): U = gy, V = gx.
void sync_vector_cov(const orc_domain& d, double* gx, double* gy) {
  const int n = d.n;
  std::vector<double>& rgx = d.work(W_RING_U, 6 * 4 * n);
  std::vector<double>& rgy = d.work(W_RING_V, 6 * 4 * n);
  exchange_vector(d, gx, gy, rgx, rgy);
  const double* qb = d.qb.data(); const double* qt = d.qt.data();
  const double* ql = d.ql.data(); const double* qr = d.qr.data();
  for (int p = 0; p < 6; ++p) {
    double* U = gy + p * n * n;
    double* V = gx + p * n * n;
    const double* UL = &rgy[(p * 4 + 0) * n]; const double* VL = &rgx[(p * 4 + 0) * n];
    const double* UR = &rgy[(p * 4 + 1) * n]; const double* VR = &rgx[(p * 4 + 1) * n];
    const double* UB = &rgy[(p * 4 + 2) * n]; const double* VB = &rgx[(p * 4 + 2) * n];
    const double* UT = &rgy[(p * 4 + 3) * n]; const double* VT = &rgx[(p * 4 + 3) * n];
    auto u = [&](int i, int j) -> double& { return U[j * n + i]; };
    auto v = [&](int i, int j) -> double& { return V[j * n + i]; };
    const int e = n - 1;
    u(0, 0) = (u(0, 0) + UL[0] + UB[0] + qb[0] * VB[0]) / 3.0;
    v(0, 0) = (v(0, 0) + VL[0] + VB[0] + ql[0] * UL[0]) / 3.0;
    u(e, 0) = (u(e, 0) + UR[0] + UB[e] + qb[e] * VB[e]) / 3.0;
    v(e, 0) = (v(e, 0) + VR[0] + VB[e] + qr[0] * UR[0]) / 3.0;
    u(0, e) = (u(0, e) + UL[e] + UT[0] + qt[0] * VT[0]) / 3.0;
    v(0, e) = (v(0, e) + VL[e] + VT[0] + ql[e] * UL[e]) / 3.0;
    u(e, e) = (u(e, e) + UR[e] + UT[e] + qt[e] * VT[e]) / 3.0;
    v(e, e) = (v(e, e) + VR[e] + VT[e] + qr[e] * UR[e]) / 3.0;
    for (int j = 1; j < e; ++j) {
      u(0, j) = 0.5 * (UL[j] + u(0, j));
      v(0, j) = 0.5 * (v(0, j) + VL[j] + ql[j] * UL[j]);
      u(e, j) = 0.5 * (u(e, j) + UR[j]);
      v(e, j) = 0.5 * (v(e, j) + VR[j] + qr[j] * UR[j]);
    }
    for (int i = 1; i < e; ++i) {
      v(i, 0) = 0.5 * (VB[i] + v(i, 0));
      u(i, 0) = 0.5 * (UB[i] + u(i, 0) + qb[i] * VB[i]);
      v(i, e) = 0.5 * (v(i, e) + VT[i]);
      u(i, e) = 0.5 * (u(i, e) + UT[i] + qt[i] * VT[i]);
    }
  }
}

// ---------------------------------------------------------------------------
// Horizontal operators on the Ah grid.
// ---------------------------------------------------------------------------
// grad_ah_sbp: calc_grad_on_tile (gradient/grad_ah_sbp_mod.f90:51-88), then
// the covariant sync.
void grad(const orc_domain& d, const double* f, double* gx, double* gy) {
  const int n = d.n;
  const double hs = d.hx * d.scale;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int pj = 0; pj < 6 * n; ++pj) {
    const int p = pj / n, j = pj % n;
    const double* F = f + p * n * n;
    for (int i = 0; i < n; ++i) {
      const double dx = sbp_point(d.sbp, F + j * n, n, 1, i);
      const double dy = sbp_point(d.sbp, F + i, n, n, j);
      gx[p * n * n + j * n + i] = dx / hs;
      gy[p * n * n + j * n + i] = dy / hs;
    }
  }
  sync_vector_cov(d, gx, gy);
}

// div_ah_sbp: calc_div_on_tile (divergence/div_ah_sbp_mod.f90:46-96), then
// the scalar sync.  u, v are contravariant components.
void div(const orc_domain& d, const double* u, const double* v, double* out) {
  const int n = d.n, np = d.npts();
  std::vector<double>& Gu = d.work(W_GU, np);
  std::vector<double>& Gv = d.work(W_GV, np);
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int k = 0; k < np; ++k) { Gu[k] = d.J[k] * u[k]; Gv[k] = d.J[k] * v[k]; }
  const double hx = d.hx, sc = d.scale;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int pj = 0; pj < 6 * n; ++pj) {
    const int p = pj / n, j = pj % n;
    const double* GU = &Gu[p * n * n];
    const double* GV = &Gv[p * n * n];
    for (int i = 0; i < n; ++i) {
      const int id = p * n * n + j * n + i;
      const double dx = sbp_point(d.sbp, GU + j * n, n, 1, i);
      const double dy = sbp_point(d.sbp, GV + i, n, n, j);
      out[id] = (dx + dy) / (d.J[id] * hx * sc);
    }
  }
  sync_scalar(d, out);
}

// curl_div_based (curl/curl_div_based_mod.f90:26-66): div(v/J, -u/J).
void curl(const orc_domain& d, const double* u, const double* v, double* out) {
  const int np = d.npts();
  std::vector<double>& ut = d.work(W_CURL_U, np);
  std::vector<double>& vt = d.work(W_CURL_V, np);
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int k = 0; k < np; ++k) { ut[k] = v[k] / d.J[k]; vt[k] = -u[k] / d.J[k]; }
  div(d, ut.data(), vt.data(), out);
}

// co2contra_colocated (co2contra/co2contra_colocated_mod.f90:36-60, 78-102)
void co2contra(const orc_domain& d, const double* u, const double* v, double* ut, double* vt) {
  const int np = d.npts();
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int k = 0; k < np; ++k) {
    const double a = d.Qi1[k] * u[k] + d.Qi2[k] * v[k];
    const double b = d.Qi2[k] * u[k] + d.Qi3[k] * v[k];
    ut[k] = a; vt[k] = b;
  }
}
void contra2co(const orc_domain& d, const double* ut, const double* vt, double* u, double* v) {
  const int np = d.npts();
  for (int k = 0; k < np; ++k) {
    const double a = d.Q1[k] * ut[k] + d.Q2[k] * vt[k];
    const double b = d.Q2[k] * ut[k] + d.Q3[k] * vt[k];
    u[k] = a; v[k] = b;
  }
}

// calc_coriolis_vec_inv_tile (coriolis/coriolis_colocated_mod.f90:79-103)
void coriolis(const orc_domain& d, const double* hu, const double* hv, const double* h,
              const double* cu, double* cor_u, double* cor_v) {
  const int np = d.npts();
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int k = 0; k < np; ++k) {
    const double fz = d.f[k] + cu[k];
    cor_u[k] = fz * hv[k] / h[k] * d.J[k];
    cor_v[k] = -(fz * hu[k] / h[k] * d.J[k]);
  }
}

// operator_swm_t%apply (models/shallow_water/operator/operator_swm_mod.f90:61-113)
void apply(const orc_domain& d, const double* hs, const double* h, const double* u,
           const double* v, double* th, double* tu, double* tv) {
  const int np = d.npts();
  std::vector<double>& ut = d.work(W_UT, np);
  std::vector<double>& vt = d.work(W_VT, np);
  std::vector<double>& hu = d.work(W_HU, np);
  std::vector<double>& hv = d.work(W_HV, np);
  std::vector<double>& KE = d.work(W_KE, np);
  std::vector<double>& gx = d.work(W_GX, np);
  std::vector<double>& gy = d.work(W_GY, np);
  std::vector<double>& cu = d.work(W_CU, np);
  std::vector<double>& cor_u = d.work(W_CORU, np);
  std::vector<double>& cor_v = d.work(W_CORV, np);
  std::vector<double>& dv = d.work(W_DV, np);
  co2contra(d, u, v, ut.data(), vt.data());
  const double g = d.grav;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int k = 0; k < np; ++k) {
    hu[k] = 1.0 * h[k] * ut[k];                       // massflux_colocated_mod.f90:19-29
    hv[k] = 1.0 * h[k] * vt[k];
    KE[k] = (u[k] * ut[k] + v[k] * vt[k]) / 2.0;      // KE_colocated_mod.f90:41-47
    KE[k] = KE[k] + g * h[k] + g * (hs ? hs[k] : 0.0);  // operator_swm_mod.f90:85
  }
  grad(d, KE.data(), gx.data(), gy.data());
  curl(d, u, v, cu.data());
  coriolis(d, hu.data(), hv.data(), h, cu.data(), cor_u.data(), cor_v.data());
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int k = 0; k < np; ++k) {
    tu[k] = -1.0 * gx[k] + 1.0 * cor_u[k];
    tv[k] = -1.0 * gy[k] + 1.0 * cor_v[k];
  }
  div(d, hu.data(), hv.data(), dv.data());
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int k = 0; k < np; ++k) th[k] = -1.0 * dv[k];
}

// rk4_t%step (time_schemes/rk4_mod.f90:20-42)
void rk4(const orc_domain& d, const double* hs, double* h, double* u, double* v, double dt,
         int nsteps) {
  const int np = d.npts();
  std::vector<double>& k1 = d.work(W_K1, 3 * (size_t)np);
  std::vector<double>& k2 = d.work(W_K2, 3 * (size_t)np);
  std::vector<double>& k3 = d.work(W_K3, 3 * (size_t)np);
  std::vector<double>& k4 = d.work(W_K4, 3 * (size_t)np);
  std::vector<double>& y = d.work(W_Y, 3 * (size_t)np);
  double* F0[3] = {h, u, v};
  auto A = [&](std::vector<double>& out, const double* yh, const double* yu, const double* yv) {
    apply(d, hs, yh, yu, yv, &out[0], &out[np], &out[2 * np]);
  };
  auto assign = [&](double s2, const std::vector<double>& kk) {
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int k = 0; k < np; ++k)
      for (int c = 0; c < 3; ++c) y[c * np + k] = 1.0 * F0[c][k] + s2 * kk[c * np + k];
  };
  for (int s = 0; s < nsteps; ++s) {
    A(k1, h, u, v);
    assign(0.5 * dt, k1);
    A(k2, &y[0], &y[np], &y[2 * np]);
    assign(0.5 * dt, k2);
    A(k3, &y[0], &y[np], &y[2 * np]);
    assign(dt, k3);
    A(k4, &y[0], &y[np], &y[2 * np]);
    const double c6 = dt / 6.0, c3 = dt / 3.0;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int k = 0; k < np; ++k)
      for (int c = 0; c < 3; ++c) {
        double x = F0[c][k];
        x = x + c6 * k1[c * np + k] + c3 * k2[c * np + k];
        x = x + c3 * k3[c * np + k] + c6 * k4[c * np + k];
        F0[c][k] = x;
      }
  }
}

// SBP quadrature mass (quadrature/sbp_quadrature_mod.f90:21-40 summed over
// tiles as abstract_quadrature_mod.f90:27-44).
double mass(const orc_domain& d, const double* f) {
  const int n = d.n;
  double tot = 0.0;
  for (int p = 0; p < 6; ++p) {
    double acc = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const int id = p * n * n + j * n + i;
        acc = acc + f[id] * d.J[id] * d.hx * d.hx * d.A[i] * d.A[j];
      }
    tot = tot + acc;
  }
  return tot;
}

// l2norm (vec_math_mod.f90:50-90), one level.
double l2sq(const orc_domain& d, const double* f) {
  const int n = d.n;
  double tot = 0.0;
  for (int p = 0; p < 6; ++p) {
    double acc = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const int id = p * n * n + j * n + i;
        acc = acc + f[id] * f[id] * d.J[id] * d.hx * d.hx;
      }
    tot = tot + acc;
  }
  return tot;
}

double maxabs(const std::vector<double>& f) {
  double m = 0.0;
  for (double x : f) m = std::max(m, std::fabs(x));
  return m;
}


template <class Gen>
void set_vector(const orc_domain& d, Gen gen, bool contravariant, std::vector<double>& u,
                std::vector<double>& v) {
  const int np = d.npts();
  u.assign(np, 0.0); v.assign(np, 0.0);
  const std::vector<double>& e1 = contravariant ? d.b1 : d.a1;
  const std::vector<double>& e2 = contravariant ? d.b2 : d.a2;
  for (int k = 0; k < np; ++k) {
    double w[3];
    gen(d.rx[k], d.ry[k], d.rz[k], w);
    u[k] = w[0] * e1[3 * k] + w[1] * e1[3 * k + 1] + w[2] * e1[3 * k + 2];
    v[k] = w[0] * e2[3 * k] + w[1] * e2[3 * k + 1] + w[2] * e2[3 * k + 2];
  }
}

// ---------------------------------------------------------------------------
// Hyperdiffusion: the diffusion operator of the split step
// (models/shallow_water/operator/operator_swm_diff_mod.f90:25-46).
// ---------------------------------------------------------------------------
using swm::NarrowD2;

const NarrowD2& narrow_table(int order) {
  return order == 63 ? swm::kNarrow63 : order == 21 ? swm::kNarrow21 : swm::kNarrow42;
}

// Narrow variable-coefficient second derivative D2^(b) at node k of a line of
// n values f with coefficients b (stride st): closure rows near either end
// (laplace_Ah_sbp42_narrow_mod.f90:128-274, the right end 275-421 counts the
// nodes from that end), interior stencil (lines 229-246; 6/3: the di_*
// formulas, laplace_Ah_sbp63_narrow_mod.f90:861-881).
double d2_point(const NarrowD2& T, const double* f, const double* b, int n, int st, int k) {
  if (k < T.rows || k >= n - T.rows) {
    const bool left = k < T.rows;
    const int r = left ? k : n - 1 - k;
    auto at = [&](const double* a, int m) { return a[(left ? m : n - 1 - m) * st]; };
    double acc = 0.0;
    for (int c = 0; c < T.cols; ++c) {
      double m = 0.0;
      for (int q = 0; q < T.nb; ++q) m += T.c[r][c][q] * at(b, q);
      acc += m * at(f, c);
    }
    return T.rowscale[r] * acc;
  }
  const int w = 2 * T.hw + 1;
  double acc = 0.0;
  for (int o = 0; o < w; ++o) {
    double cf = 0.0;
    for (int q = 0; q < w; ++q) cf += T.in[o][q] * b[(k + q - T.hw) * st];
    acc += cf * f[(k + o - T.hw) * st];
  }
  return acc;
}

// laplace_Ah_sbp{42,63,21}_narrow calc_laplace (laplace_Ah_sbp42_narrow_mod.f90:
// 23-58, laplace_Ah_sbp21_narrow_mod.f90:23-243): first derivatives times J*Qi12 (calc_tile_d1x_d1y, 60-93), the
// narrow D2 along x with b = J*Qi11 and along y with b = J*Qi22, the
// cross-derivative boundary fluxes on the x rows (717-743), the mixed terms
// D_y(d1f_x) + D_x(d1f_y) (745-752), division by (hx*scale)^2 and by J, then
// the Ah scalar sync.  The first derivatives use the SBP operator of the
// same order (laplace_factory_mod.f90:179-214).
void laplace_narrow(const orc_domain& d, int narrow, const double* f, double* out) {
  const NarrowD2& T = narrow_table(narrow);
  const Sbp s1 = make_sbp(narrow);
  const int n = d.n, np = d.npts();
  std::vector<double> bx(np), by(np), d1x(np), d1y(np);
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int k = 0; k < np; ++k) {
    bx[k] = d.Qi1[k] * d.J[k];
    by[k] = d.Qi3[k] * d.J[k];
  }
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int pj = 0; pj < 6 * n; ++pj) {
    const int p = pj / n, j = pj % n;
    const double* F = f + p * n * n;
    for (int i = 0; i < n; ++i) {
      const int id = p * n * n + j * n + i;
      d1x[id] = sbp_point(s1, F + j * n, n, 1, i) * d.J[id] * d.Qi2[id];
      d1y[id] = sbp_point(s1, F + i, n, n, j) * d.J[id] * d.Qi2[id];
    }
  }
  const double hs = d.hx * d.scale;
#pragma omp parallel for schedule(static) num_threads(g_threads)
  for (int pj = 0; pj < 6 * n; ++pj) {
    const int p = pj / n, j = pj % n;
    const int o = p * n * n;
    for (int i = 0; i < n; ++i) {
      const int id = o + j * n + i;
      double d2x = d2_point(T, f + o + j * n, &bx[o + j * n], n, 1, i);
      const double d2y = d2_point(T, f + o + i, &by[o + i], n, n, j);
      if (i == 0) d2x = d2x - 0.5 * (T.penalty * (-2.0 * d1y[id]));
      if (i == n - 1) d2x = d2x - 0.5 * (T.penalty * (2.0 * d1y[id]));
      if (j == 0) d2x = d2x - 0.5 * (T.penalty * (-2.0 * d1x[id]));
      if (j == n - 1) d2x = d2x - 0.5 * (T.penalty * (2.0 * d1x[id]));
      const double d2yx = sbp_point(s1, &d1x[o + i], n, n, j);
      const double d2xy = sbp_point(s1, &d1y[o + j * n], n, 1, i);
      double v = 1.0 * d2x + 1.0 * d2y;
      v = v + 1.0 * d2xy + 1.0 * d2yx;
      v = v / (hs * hs);
      out[id] = v / d.J[id];
    }
  }
  sync_scalar(d, out);
}

// hordiff_scalar_t%calc_diff with diff_order 2 (hordiff_scalar_mod.f90:33-53;
// coefficient hordiff_coeff*scale*hx, hordiff_factory_mod.f90:157-188):
// out = -(c^4) * lap(lap(f)).
void hordiff_scalar(const orc_domain& d, int narrow, double coeff, const double* f, double* out) {
  const int np = d.npts();
  std::vector<double> t(np), t2(np);
  laplace_narrow(d, narrow, f, t.data());
  laplace_narrow(d, narrow, t.data(), t2.data());
  const double dc = coeff * d.scale * d.hx;
  const double dc2 = dc * dc;
  const double c = -1.0 * (dc2 * dc2);
  for (int k = 0; k < np; ++k) out[k] = c * t2[k];
}

// hordiff_colocated_xyz_t%calc_diff_vec (hordiff_colocated_mod.f90:41-58):
// the Cartesian vector b1*u + b2*v (vec_math_mod.f90:107-126), the scalar
// operator on each Cartesian component, the projections onto b1 and b2
// (vec_math_mod.f90:128-160) and the covariant vector sync.
void hordiff_vec_xyz(const orc_domain& d, int narrow, double coeff, const double* u,
                     const double* v, double* ut, double* vt) {
  const int np = d.npts();
  std::vector<double> c[3], t[3];
  for (int a = 0; a < 3; ++a) { c[a].assign(np, 0.0); t[a].assign(np, 0.0); }
  for (int k = 0; k < np; ++k)
    for (int a = 0; a < 3; ++a) c[a][k] = d.b1[3 * k + a] * u[k] + d.b2[3 * k + a] * v[k];
  for (int a = 0; a < 3; ++a) hordiff_scalar(d, narrow, coeff, c[a].data(), t[a].data());
  for (int k = 0; k < np; ++k) {
    ut[k] = t[0][k] * d.b1[3 * k] + t[1][k] * d.b1[3 * k + 1] + t[2][k] * d.b1[3 * k + 2];
    vt[k] = t[0][k] * d.b2[3 * k] + t[1][k] * d.b2[3 * k + 1] + t[2][k] * d.b2[3 * k + 2];
  }
  sync_vector_cov(d, ut, vt);
}

// ---------------------------------------------------------------------------
// Lat-lon output of Ah fields: the interpolator of create_latlon_interp
// (regridders/regrid_factory_mod.f90:195-299), the scalar and vector regrids
// (regrid_to_latlon_mod.f90:54-124, 126-165) and the ECS map from a point on
// the sphere to (panel, alpha, beta) (equiang_cs/ecs_metric_mod.f90:480-506).
// ---------------------------------------------------------------------------
void cart_to_native(const double r[3], int& panel, double& alpha, double& beta) {
  panel = 0;
  double best = 0.0;
  for (int p = 0; p < 6; ++p) {
    const double rn = -(r[0] * TN[p][0] + r[1] * TN[p][1] + r[2] * TN[p][2]);
    if (rn > best) { panel = p; best = rn; }
  }
  alpha = std::atan((TEX[panel][0] * r[0] + TEX[panel][1] * r[1] + TEX[panel][2] * r[2]) / best);
  beta = std::atan((TEY[panel][0] * r[0] + TEY[panel][1] * r[1] + TEY[panel][2] * r[2]) / best);
}

struct LatLonInterp {
  int nlon = 0, nlat = 0, w = 0;
  std::vector<int> panel, xi, yi;      // stencil start (0-based) per point
  std::vector<double> wx, wy;          // w weights per point
  std::vector<double> alpha, beta;
};

// Point (i, j) of the Nlon x Nlat grid: lon = i*2pi/Nlon, lat = -pi/2 + j*pi/(Nlat-1).
void latlon_point(int nlon, int nlat, int i, int j, double& lat, double& lon) {
  const double hlon = 2.0 * PI / (double)nlon, hlat = PI / (nlat - 1.0);
  lat = -0.5 * PI + hlat * j;
  lon = hlon * i;
}

LatLonInterp make_latlon_interp(const orc_domain& d, int nlon, int nlat, int w) {
  LatLonInterp L;
  L.nlon = nlon; L.nlat = nlat; L.w = w;
  const int np = nlon * nlat, n = d.n;
  L.panel.resize(np); L.xi.resize(np); L.yi.resize(np);
  L.wx.resize((size_t)w * np); L.wy.resize((size_t)w * np);
  L.alpha.resize(np); L.beta.resize(np);
  const double alpha0 = -0.25 * PI;
  for (int j = 0; j < nlat; ++j)
    for (int i = 0; i < nlon; ++i) {
      const int q = j * nlon + i;
      double lat, lon;
      latlon_point(nlon, nlat, i, j, lat, lon);
      const double r[3] = {std::cos(lat) * std::cos(lon), std::cos(lat) * std::sin(lon), std::sin(lat)};
      int p; double a, b;
      cart_to_native(r, p, a, b);
      L.panel[q] = p; L.alpha[q] = a; L.beta[q] = b;
      // 1-based node coordinates, stencil clipped to the panel's nodes 1..n
      const double zdx = (a - alpha0) / d.hx + 1.0, zdy = (b - alpha0) / d.hx + 1.0;
      int ir = std::min((int)std::floor(zdx) + w / 2, n);
      const int x1 = std::max(ir - w + 1, 1);
      ir = std::min((int)std::floor(zdy) + w / 2, n);
      const int y1 = std::max(ir - w + 1, 1);
      L.xi[q] = x1 - 1; L.yi[q] = y1 - 1;
      const double dx = zdx - x1, dy = zdy - y1;
      double* WX = &L.wx[(size_t)w * q];
      double* WY = &L.wy[(size_t)w * q];
      if (w == 2) {
        WX[0] = 1.0 - dx; WX[1] = dx;
        WY[0] = 1.0 - dy; WY[1] = dy;
      } else {
        WX[0] = -(dx - 1.0) * (dx - 2.0) * (dx - 3.0) / 6.0;
        WX[1] = dx * (dx - 2.0) * (dx - 3.0) / 2.0;
        WX[2] = -dx * (dx - 1.0) * (dx - 3.0) / 2.0;
        WX[3] = dx * (dx - 1.0) * (dx - 2.0) / 6.0;
        WY[0] = -(dy - 1.0) * (dy - 2.0) * (dy - 3.0) / 6.0;
        WY[1] = dy * (dy - 2.0) * (dy - 3.0) / 2.0;
        WY[2] = -dy * (dy - 1.0) * (dy - 3.0) / 2.0;
        WY[3] = dy * (dy - 1.0) * (dy - 2.0) / 6.0;
      }
    }
  return L;
}

// latlon_interpolate (regrid_to_latlon_mod.f90:146-165)
void latlon_interpolate(const orc_domain& d, const LatLonInterp& L, const double* f, double* out) {
  const int n = d.n, w = L.w;
  for (int q = 0; q < L.nlon * L.nlat; ++q) {
    const double* F = f + (size_t)L.panel[q] * n * n;
    double acc = 0.0;
    for (int j1 = 0; j1 < w; ++j1)
      for (int i1 = 0; i1 < w; ++i1) {
        const double p = F[(L.yi[q] + j1) * n + (L.xi[q] + i1)];
        acc = acc + L.wx[(size_t)w * q + i1] * L.wy[(size_t)w * q + j1] * p;
      }
    out[q] = acc;
  }
}

// Ah vector regrid: both components interpolated, then rotated to the
// lat-lon (east, north) components with the dot products of the lat-lon
// unit vectors and b1, b2 (covariant components) or a1, a2 (contravariant)
// at the point (regrid_factory_mod.f90:121-160, regrid_to_latlon_mod.f90:
// 126-144).
void latlon_vector(const orc_domain& d, const LatLonInterp& L, bool contravariant, const double* u,
                   const double* v, double* uo, double* vo) {
  latlon_interpolate(d, L, u, uo);
  latlon_interpolate(d, L, v, vo);
  for (int j = 0; j < L.nlat; ++j)
    for (int i = 0; i < L.nlon; ++i) {
      const int q = j * L.nlon + i;
      double lat, lon;
      latlon_point(L.nlon, L.nlat, i, j, lat, lon);
      const double iv[3] = {-std::sin(lon), std::cos(lon), 0.0};
      const double jv[3] = {-std::sin(lat) * std::cos(lon), -std::sin(lat) * std::sin(lon), std::cos(lat)};
      double e1p[3], e2p[3], e1[3], e2[3];
      if (contravariant) { a1_proto(L.alpha[q], L.beta[q], e1p); a2_proto(L.alpha[q], L.beta[q], e2p); }
      else { b1_proto(L.alpha[q], L.beta[q], e1p); b2_proto(L.alpha[q], L.beta[q], e2p); }
      to_face(L.panel[q], e1p, e1);
      to_face(L.panel[q], e2p, e2);
      const double u2u = iv[0] * e1[0] + iv[1] * e1[1] + iv[2] * e1[2];
      const double u2v = jv[0] * e1[0] + jv[1] * e1[1] + jv[2] * e1[2];
      const double v2u = iv[0] * e2[0] + iv[1] * e2[1] + iv[2] * e2[2];
      const double v2v = jv[0] * e2[0] + jv[1] * e2[1] + jv[2] * e2[2];
      const double zu = uo[q], zv = vo[q];
      uo[q] = u2u * zu + v2u * zv;
      vo[q] = u2v * zu + v2v * zv;
    }
}

bool narrow_ok(const orc_domain& d, int narrow) {
  return (narrow == 21 || narrow == 42 || narrow == 63) && d.n >= 2 * narrow_table(narrow).rows;
}

}  // namespace

// ===========================================================================
// C interface
// ===========================================================================
extern "C" {

orc_domain* orc_create(int N, int sbp_order, double radius, double grav, double omega,
                       const double axis[3]) {
  if (N < 8 || (sbp_order != 21 && sbp_order != 42 && sbp_order != 43 && sbp_order != 63))
    return nullptr;
  orc_domain* d = new orc_domain();
  const double def_axis[3] = {0.0, 0.0, 1.0};
  build(*d, N, sbp_order, radius, grav, omega, axis ? axis : def_axis);
  return d;
}

void orc_destroy(orc_domain* d) { delete d; }
int orc_npts(const orc_domain* d) { return d->npts(); }
void orc_set_threads(int t) { g_threads = t < 1 ? 1 : t; }
int orc_get_threads(void) { return g_threads; }

void orc_geometry(const orc_domain* d, double* J, double* Qi1, double* Qi2, double* Qi3,
                  double* f, double* rx, double* ry, double* rz) {
  const size_t b = sizeof(double) * d->npts();
  if (J) std::memcpy(J, d->J.data(), b);
  if (Qi1) std::memcpy(Qi1, d->Qi1.data(), b);
  if (Qi2) std::memcpy(Qi2, d->Qi2.data(), b);
  if (Qi3) std::memcpy(Qi3, d->Qi3.data(), b);
  if (f) std::memcpy(f, d->f.data(), b);
  if (rx) std::memcpy(rx, d->rx.data(), b);
  if (ry) std::memcpy(ry, d->ry.data(), b);
  if (rz) std::memcpy(rz, d->rz.data(), b);
}

void orc_bases(const orc_domain* d, double* a1, double* a2, double* b1, double* b2) {
  const size_t b = sizeof(double) * 3 * d->npts();
  if (a1) std::memcpy(a1, d->a1.data(), b);
  if (a2) std::memcpy(a2, d->a2.data(), b);
  if (b1) std::memcpy(b1, d->b1.data(), b);
  if (b2) std::memcpy(b2, d->b2.data(), b);
}

void orc_sync_weights(const orc_domain* d, double* qb, double* qt, double* ql, double* qr) {
  const size_t b = sizeof(double) * d->n;
  std::memcpy(qb, d->qb.data(), b); std::memcpy(qt, d->qt.data(), b);
  std::memcpy(ql, d->ql.data(), b); std::memcpy(qr, d->qr.data(), b);
}

void orc_co2contra(const orc_domain* d, const double* u, const double* v, double* ut, double* vt) { co2contra(*d, u, v, ut, vt); }
void orc_contra2co(const orc_domain* d, const double* ut, const double* vt, double* u, double* v) { contra2co(*d, ut, vt, u, v); }
void orc_grad(const orc_domain* d, const double* f, double* gx, double* gy) { grad(*d, f, gx, gy); }
void orc_div(const orc_domain* d, const double* u, const double* v, double* o) { div(*d, u, v, o); }
void orc_curl(const orc_domain* d, const double* u, const double* v, double* o) { curl(*d, u, v, o); }
void orc_sync_scalar(const orc_domain* d, double* f) { sync_scalar(*d, f); }
void orc_sync_vector_cov(const orc_domain* d, double* gx, double* gy) { sync_vector_cov(*d, gx, gy); }
void orc_coriolis(const orc_domain* d, const double* hu, const double* hv, const double* h,
                  const double* cu, double* cor_u, double* cor_v) { coriolis(*d, hu, hv, h, cu, cor_u, cor_v); }

void orc_apply(const orc_domain* d, const double* hs, const double* h, const double* u,
               const double* v, double* th, double* tu, double* tv) { apply(*d, hs, h, u, v, th, tu, tv); }
void orc_rk4(const orc_domain* d, const double* hs, double* h, double* u, double* v, double dt,
             int nsteps) { rk4(*d, hs, h, u, v, dt, nsteps); }

// get_diagnostics (operator_swm_mod.f90:115-155) with calc_energy 211-236 and
// calc_enstrophy 238-260.
void orc_diagnostics(const orc_domain* d, const double* hs, const double* h, const double* u,
                     const double* v, double out[7]) {
  const int np = d->npts();
  double hmin = h[0], hmax = h[0];
  for (int k = 0; k < np; ++k) { hmin = std::min(hmin, h[k]); hmax = std::max(hmax, h[k]); }
  std::vector<double> ut(np), vt(np), hu(np), hv(np), ku(np), kv(np), pe(np), cu(np);
  co2contra(*d, u, v, ut.data(), vt.data());
  for (int k = 0; k < np; ++k) {
    hu[k] = 1.0 * h[k] * ut[k]; hv[k] = 1.0 * h[k] * vt[k];
    ku[k] = 0.5 * hu[k] * u[k]; kv[k] = 0.5 * hv[k] * v[k];
    pe[k] = 1.0 * h[k] + 1.0 * (hs ? hs[k] : 0.0);
    pe[k] = 0.5 * d->grav * pe[k] * pe[k];
  }
  const double ke = mass(*d, ku.data()) + mass(*d, kv.data());
  const double pen = mass(*d, pe.data());
  curl(*d, u, v, cu.data());
  for (int k = 0; k < np; ++k) {
    double c = cu[k] + 1.0 * d->f[k];
    c = 0.5 * c * c;
    cu[k] = 1.0 * c / h[k];
  }
  out[0] = hmin; out[1] = hmax; out[2] = mass(*d, h);
  out[3] = ke + pen; out[4] = ke; out[5] = pen; out[6] = mass(*d, cu.data());
}

// Lat-lon regrids of Ah fields: width 2 (linear) or 4 (cubic); out has
// Nlon*Nlat values, longitude fastest.  -1 on bad arguments.
int orc_latlon_scalar(const orc_domain* d, int nlon, int nlat, int width, const double* f,
                      double* out) {
  if (nlon < 1 || nlat < 2 || (width != 2 && width != 4)) return -1;
  const LatLonInterp L = make_latlon_interp(*d, nlon, nlat, width);
  latlon_interpolate(*d, L, f, out);
  return 0;
}
int orc_latlon_vector(const orc_domain* d, int nlon, int nlat, int width, int contravariant,
                      const double* u, const double* v, double* uo, double* vo) {
  if (nlon < 1 || nlat < 2 || (width != 2 && width != 4)) return -1;
  const LatLonInterp L = make_latlon_interp(*d, nlon, nlat, width);
  latlon_vector(*d, L, contravariant != 0, u, v, uo, vo);
  return 0;
}

// The reference's regrid known-answer test (test/test_regrid/
// test_regrid_mod.f90:16-119) on the Ah grid at N=32, nz=3: the maximum
// interpolation error of the xyz scalar field (kind 0; out[0]) or of the
// solid rotation field's lat-lon components (kind 1 covariant, 2
// contravariant; out[0] u, out[1] v).
int orc_golden_regrid(int kind, int width, double out[2]) {
  const int N = 32, nlon = 4 * N, nlat = 2 * N + 1;
  orc_domain d;
  const double axis[3] = {0.0, 0.0, 1.0};
  build(d, N, 42, 1.0, 9.80616, 1.0, axis);
  const LatLonInterp L = make_latlon_interp(d, nlon, nlat, width);
  const int npl = nlon * nlat;
  std::vector<double> a(npl), b(npl);
  out[0] = out[1] = 0.0;
  for (int k = 0; k < 3; ++k) {
    if (kind == 0) {
      std::vector<double> f(d.npts());
      for (int q = 0; q < d.npts(); ++q) f[q] = field_xyz(k, d.rx[q], d.ry[q], d.rz[q]);
      latlon_interpolate(d, L, f.data(), a.data());
    } else {
      std::vector<double> u, v;
      set_vector(d, [k](double x, double y, double z, double w[3]) { field_solid_rotation(k, x, y, z, w); },
                 kind == 2, u, v);
      latlon_vector(d, L, kind == 2, u.data(), v.data(), a.data(), b.data());
    }
    for (int j = 0; j < nlat; ++j)
      for (int i = 0; i < nlon; ++i) {
        const int q = j * nlon + i;
        double lat, lon;
        latlon_point(nlon, nlat, i, j, lat, lon);
        const double x = std::cos(lat) * std::cos(lon), y = std::cos(lat) * std::sin(lon), z = std::sin(lat);
        if (kind == 0) {
          out[0] = std::max(out[0], std::fabs(a[q] - field_xyz(k, x, y, z)));
        } else {
          double w[3];
          field_solid_rotation(k, x, y, z, w);
          const double ut = -std::sin(lon) * w[0] + std::cos(lon) * w[1];
          const double vt = -std::sin(lat) * std::cos(lon) * w[0] - std::sin(lat) * std::sin(lon) * w[1] +
                            std::cos(lat) * w[2];
          out[0] = std::max(out[0], std::fabs(a[q] - ut));
          out[1] = std::max(out[1], std::fabs(b[q] - vt));
        }
      }
  }
  return 0;
}

// Hyperdiffusion pieces (operator_swm_diff_mod.f90:25-46,
// explicit_Eul1_mod.f90:20-30); narrow = 42 or 63 selects
// laplace_ah_sbp42_narrow or laplace_ah_sbp63_narrow.  -1 on a bad order or
// a grid too small for the closures.
int orc_laplace(const orc_domain* d, int narrow, const double* f, double* out) {
  if (!narrow_ok(*d, narrow)) return -1;
  laplace_narrow(*d, narrow, f, out);
  return 0;
}
int orc_hordiff_scalar(const orc_domain* d, int narrow, double coeff, const double* f, double* out) {
  if (!narrow_ok(*d, narrow)) return -1;
  hordiff_scalar(*d, narrow, coeff, f, out);
  return 0;
}
int orc_hordiff_vec_xyz(const orc_domain* d, int narrow, double coeff, const double* u,
                        const double* v, double* ut, double* vt) {
  if (!narrow_ok(*d, narrow)) return -1;
  hordiff_vec_xyz(*d, narrow, coeff, u, v, ut, vt);
  return 0;
}
int orc_diffusion_apply(const orc_domain* d, int uv_narrow, double uv_coeff, int h_narrow,
                        double h_coeff, const double* h, const double* u, const double* v,
                        double* th, double* tu, double* tv) {
  if (!narrow_ok(*d, uv_narrow) || !narrow_ok(*d, h_narrow)) return -1;
  hordiff_vec_xyz(*d, uv_narrow, uv_coeff, u, v, tu, tv);
  hordiff_scalar(*d, h_narrow, h_coeff, h, th);
  return 0;
}
int orc_diffusion_step(const orc_domain* d, int uv_narrow, double uv_coeff, int h_narrow,
                       double h_coeff, double* h, double* u, double* v, double dt) {
  const int np = d->npts();
  std::vector<double> th(np), tu(np), tv(np);
  if (int rc = orc_diffusion_apply(d, uv_narrow, uv_coeff, h_narrow, h_coeff, h, u, v, th.data(),
                                   tu.data(), tv.data()))
    return rc;
  for (int k = 0; k < np; ++k) {
    h[k] = h[k] + dt * th[k];
    u[k] = u[k] + dt * tu[k];
    v[k] = v[k] + dt * tv[k];
  }
  return 0;
}

double orc_l2norm(const orc_domain* d, const double* f) { return std::sqrt(l2sq(*d, f)); }
double orc_mass(const orc_domain* d, const double* f) { return mass(*d, f); }

// Analytic test fields of the known-answer tests, one level (0..2):
// kind 0 solid rotation, 1 cross-polar flow, 2 xyz gradient, 3 VSH curl-free
// (vectors; contravariant != 0 selects b1/b2 components) and kind 10 xyz,
// 11 cross-polar divergence, 12 cross-polar vorticity (scalars).
int orc_vector_test_field(const orc_domain* d, int kind, int level, int contravariant,
                          double* u, double* v) {
  std::vector<double> uu, vv;
  switch (kind) {
    case 0: set_vector(*d, [level](double x, double y, double z, double w[3]) { field_solid_rotation(level, x, y, z, w); }, contravariant != 0, uu, vv); break;
    case 1: set_vector(*d, field_cross_polar, contravariant != 0, uu, vv); break;
    case 2: set_vector(*d, [level](double x, double y, double z, double w[3]) { field_xyz_grad(level, x, y, z, w); }, contravariant != 0, uu, vv); break;
    case 3: set_vector(*d, field_vsh_curl_free_10, contravariant != 0, uu, vv); break;
    default: return -1;
  }
  std::memcpy(u, uu.data(), sizeof(double) * uu.size());
  std::memcpy(v, vv.data(), sizeof(double) * vv.size());
  return 0;
}

int orc_scalar_test_field(const orc_domain* d, int kind, int level, double* f) {
  for (int k = 0; k < d->npts(); ++k) {
    const double x = d->rx[k], y = d->ry[k], z = d->rz[k];
    switch (kind) {
      case 10: f[k] = field_xyz(level, x, y, z); break;
      case 11: f[k] = field_cross_polar_div(x, y, z); break;
      case 12: f[k] = field_cross_polar_zeta(x, y, z); break;
      default: return -1;
    }
  }
  return 0;
}

// test_div (test_diff_ops/test_diffops_mod.f90:71-125), nz = 3
int orc_golden_div(int N, int order, double out[4]) {
  const double ax[3] = {0, 0, 1};
  orc_domain* d = orc_create(N, order, 1.0, 9.80616, 1.0, ax);
  if (!d) return -1;
  const int np = d->npts();
  std::vector<double> u, v, dv(np), all;
  double l2 = 0.0;
  for (int lev = 0; lev < 3; ++lev) {
    set_vector(*d, [lev](double x, double y, double z, double w[3]) { field_solid_rotation(lev, x, y, z, w); }, true, u, v);
    div(*d, u.data(), v.data(), dv.data());
    for (int k = 0; k < np; ++k) dv[k] = d->scale * dv[k];
    all.insert(all.end(), dv.begin(), dv.end());
    l2 += l2sq(*d, dv.data());
  }
  out[0] = maxabs(all); out[1] = std::sqrt(l2);
  all.clear(); l2 = 0.0;
  for (int lev = 0; lev < 3; ++lev) {
    set_vector(*d, field_cross_polar, true, u, v);
    div(*d, u.data(), v.data(), dv.data());
    for (int k = 0; k < np; ++k)
      dv[k] = d->scale * dv[k] - 1.0 * field_cross_polar_div(d->rx[k], d->ry[k], d->rz[k]);
    all.insert(all.end(), dv.begin(), dv.end());
    l2 += l2sq(*d, dv.data());
  }
  out[2] = maxabs(all); out[3] = std::sqrt(l2);
  orc_destroy(d);
  return 0;
}

// test_grad (test_diffops_mod.f90:127-178), nz = 3
int orc_golden_grad(int N, int order, double out[2]) {
  const double ax[3] = {0, 0, 1};
  orc_domain* d = orc_create(N, order, 1.0, 9.80616, 1.0, ax);
  if (!d) return -1;
  const int np = d->npts();
  std::vector<double> f(np), gx(np), gy(np), tx, ty, ex_all, ey_all;
  double l2x = 0.0, l2y = 0.0;
  for (int lev = 0; lev < 3; ++lev) {
    for (int k = 0; k < np; ++k) f[k] = field_xyz(lev, d->rx[k], d->ry[k], d->rz[k]);
    set_vector(*d, [lev](double x, double y, double z, double w[3]) { field_xyz_grad(lev, x, y, z, w); }, false, tx, ty);
    grad(*d, f.data(), gx.data(), gy.data());
    for (int k = 0; k < np; ++k) {
      gx[k] = d->scale * gx[k] - 1.0 * tx[k];
      gy[k] = d->scale * gy[k] - 1.0 * ty[k];
    }
    ex_all.insert(ex_all.end(), gx.begin(), gx.end());
    ey_all.insert(ey_all.end(), gy.begin(), gy.end());
    l2x += l2sq(*d, gx.data()); l2y += l2sq(*d, gy.data());
  }
  out[0] = maxabs(ex_all) + maxabs(ey_all);
  out[1] = std::sqrt(l2x) + std::sqrt(l2y);
  orc_destroy(d);
  return 0;
}

// test_curl (test_diffops_mod.f90:466-522), nz = 3
int orc_golden_curl(int N, int order, double out[4]) {
  const double ax[3] = {0, 0, 1};
  orc_domain* d = orc_create(N, order, 1.0, 9.80616, 1.0, ax);
  if (!d) return -1;
  const int np = d->npts();
  std::vector<double> u, v, c(np), all;
  double l2 = 0.0;
  for (int lev = 0; lev < 3; ++lev) {
    set_vector(*d, field_vsh_curl_free_10, false, u, v);
    curl(*d, u.data(), v.data(), c.data());
    for (int k = 0; k < np; ++k) c[k] = d->scale * c[k];
    all.insert(all.end(), c.begin(), c.end());
    l2 += l2sq(*d, c.data());
  }
  out[0] = maxabs(all); out[1] = std::sqrt(l2);
  all.clear(); l2 = 0.0;
  for (int lev = 0; lev < 3; ++lev) {
    set_vector(*d, field_cross_polar, false, u, v);
    curl(*d, u.data(), v.data(), c.data());
    for (int k = 0; k < np; ++k)
      c[k] = d->scale * c[k] - 1.0 * field_cross_polar_zeta(d->rx[k], d->ry[k], d->rz[k]);
    all.insert(all.end(), c.begin(), c.end());
    l2 += l2sq(*d, c.data());
  }
  out[2] = maxabs(all); out[3] = std::sqrt(l2);
  orc_destroy(d);
  return 0;
}

static int golden_transform(int N, bool to_contra, double out[2]) {
  const double ax[3] = {0, 0, 1};
  orc_domain* d = orc_create(N, 42, 1.0, 9.80616, 1.0, ax);
  if (!d) return -1;
  const int np = d->npts();
  std::vector<double> ui, vi, ut, vt, uo(np), vo(np), eu, ev;
  double l2u = 0.0, l2v = 0.0;
  for (int lev = 0; lev < 3; ++lev) {
    set_vector(*d, field_cross_polar, !to_contra, ui, vi);
    set_vector(*d, field_cross_polar, to_contra, ut, vt);
    if (to_contra) co2contra(*d, ui.data(), vi.data(), uo.data(), vo.data());
    else contra2co(*d, ui.data(), vi.data(), uo.data(), vo.data());
    for (int k = 0; k < np; ++k) { uo[k] = uo[k] + (-1.0) * ut[k]; vo[k] = vo[k] + (-1.0) * vt[k]; }
    eu.insert(eu.end(), uo.begin(), uo.end());
    ev.insert(ev.end(), vo.begin(), vo.end());
    l2u += l2sq(*d, uo.data()); l2v += l2sq(*d, vo.data());
  }
  out[0] = maxabs(eu) + maxabs(ev);
  out[1] = std::sqrt(l2u) + std::sqrt(l2v);
  orc_destroy(d);
  return 0;
}
int orc_golden_co2contra(int N, double out[2]) { return golden_transform(N, true, out); }
int orc_golden_contra2co(int N, double out[2]) { return golden_transform(N, false, out); }

// The colocated A grid of the reference's pointwise operator tests
// (create_domain(domain, "cube", "A", N, nz)): N x N cell-centre points per
// panel, alpha_i = -pi/4 + (i + 1/2) hx, unit sphere, Omega = 1 about z.  The
// node's position, covariant / contravariant basis and Jacobian follow
// ecs_metric_mod.f90:326-478 as on the Ah grid.
struct AGridNode {
  double r[3], a1[3], a2[3], b1[3], b2[3], J;
};
static AGridNode agrid_node(int N, int p, int i, int j) {
  const double hx = 0.5 * PI / (double)N;
  const double al = -0.25 * PI + (i + 0.5) * hx, be = -0.25 * PI + (j + 0.5) * hx;
  AGridNode g;
  double v[3];
  r_proto(al, be, v); to_face(p, v, g.r);
  a1_proto(al, be, v); to_face(p, v, g.a1);
  a2_proto(al, be, v); to_face(p, v, g.a2);
  b1_proto(al, be, v); to_face(p, v, g.b1);
  b2_proto(al, be, v); to_face(p, v, g.b2);
  const double ta = std::tan(al), tb = std::tan(be);
  const double sg = std::sqrt(1.0 + ta * ta + tb * tb);
  g.J = (1.0 + ta * ta) * (1.0 + tb * tb) / (sg * sg * sg);
  return g;
}
static double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// test_coriolis with coriolis_colocated on the A grid (test_diffops_mod.f90:
// 651-722): cor = calc_coriolis of the contravariant VSH_curl_free_10 field
// (coriolis_colocated_mod.f90:36-61: cor_u = f vt J, cor_v = -f ut J) against
// the covariant components of the exact force 2 sin(phi) (v_phi, -v_lam)
// (test_fields_mod.f90:592-616); nz = 3 identical levels.  out = {sum of
// the maxabs, sum of the l2 norms} of (cor_u, cor_v) errors.
int orc_golden_coriolis(int N, double out[2]) {
  const double hx = 0.5 * PI / (double)N;
  double mu = 0.0, mv = 0.0, l2u = 0.0, l2v = 0.0;
  for (int lev = 0; lev < 3; ++lev)
    for (int p = 0; p < 6; ++p)
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          const AGridNode g = agrid_node(N, p, i, j);
          double V[3];
          field_vsh_curl_free_10(g.r[0], g.r[1], g.r[2], V);
          const double ut = dot3(V, g.b1), vt = dot3(V, g.b2);
          const double f = 2.0 * 1.0 * g.r[2] / std::sqrt(dot3(g.r, g.r));
          const double cu = f * vt * g.J, cv = -f * ut * g.J;
          // exact force: lam/phi components of V, rotated and scaled
          const double lam = std::atan2(g.r[1], g.r[0]);
          const double phi = std::asin(g.r[2] / std::sqrt(dot3(g.r, g.r)));
          const double el[3] = {-std::sin(lam), std::cos(lam), 0.0};
          const double ep[3] = {-std::sin(phi) * std::cos(lam), -std::sin(phi) * std::sin(lam), std::cos(phi)};
          const double vl = dot3(V, el), vp = dot3(V, ep);
          const double pc = 2.0 * std::sin(phi);
          const double fl = pc * vp, fp = -pc * vl;
          const double F[3] = {fl * el[0] + fp * ep[0], fl * el[1] + fp * ep[1], fl * el[2] + fp * ep[2]};
          const double eu = cu + (-1.0) * dot3(F, g.a1), ev = cv + (-1.0) * dot3(F, g.a2);
          mu = std::max(mu, std::fabs(eu));
          mv = std::max(mv, std::fabs(ev));
          l2u = l2u + eu * eu * g.J * hx * hx;
          l2v = l2v + ev * ev * g.J * hx * hx;
        }
  out[0] = mu + mv;
  out[1] = std::sqrt(l2u) + std::sqrt(l2v);
  return 0;
}

// test_KE with KE_colocated on the A grid (test_diffops_mod.f90:523-587):
// KE = (u ut + v vt) / 2 (KE_colocated_mod.f90:41-47) from the covariant and
// contravariant components of the VSH_curl_free_10 and cross-polar fields,
// against |V|^2 / 2 (test_fields_mod.f90:804-825); nz = 3.  out = {maxabs,
// l2} of the VSH error, then of the cross-polar error.
int orc_golden_ke(int N, double out[4]) {
  const double hx = 0.5 * PI / (double)N;
  for (int fld = 0; fld < 2; ++fld) {
    double m = 0.0, l2 = 0.0;
    for (int lev = 0; lev < 3; ++lev)
      for (int p = 0; p < 6; ++p)
        for (int j = 0; j < N; ++j)
          for (int i = 0; i < N; ++i) {
            const AGridNode g = agrid_node(N, p, i, j);
            double V[3];
            if (fld == 0) field_vsh_curl_free_10(g.r[0], g.r[1], g.r[2], V);
            else field_cross_polar(g.r[0], g.r[1], g.r[2], V);
            const double u = dot3(V, g.a1), v = dot3(V, g.a2);
            const double ut = dot3(V, g.b1), vt = dot3(V, g.b2);
            const double ke = (u * ut + v * vt) / 2.0;
            const double e = ke + (-1.0) * (0.5 * (V[0] * V[0] + V[1] * V[1] + V[2] * V[2]));
            m = std::max(m, std::fabs(e));
            l2 = l2 + e * e * g.J * hx * hx;
          }
    out[2 * fld] = m;
    out[2 * fld + 1] = std::sqrt(l2);
  }
  return 0;
}

// test_quadrature (test_quadrature/test_quadrature_mod.f90:18-80)
double orc_golden_quadrature(int N, int order, int max_order) {
  const double ax[3] = {0, 0, 1};
  orc_domain* d = orc_create(N, order, 1.0, 9.80616, 1.0, ax);
  if (!d) return -1.0;
  const int n = d->n, np = d->npts();
  std::vector<double> fu(np);
  double worst = 0.0;
  for (int o = 0; o <= max_order; ++o) {
    for (int p = 0; p < 6; ++p)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int id = p * n * n + j * n + i;
          const double a = alpha_of(*d, i), b = alpha_of(*d, j);
          fu[id] = 1.0 / d->J[id] * std::pow(a, o) * std::pow(b, o);
        }
    const int pw = o + 1;
    const double t = std::pow(0.25 * PI, pw) - std::pow(-0.25 * PI, pw);
    const double exact = 6.0 * t * t / (double)(pw * pw);
    worst = std::max(worst, std::fabs(exact - mass(*d, fu.data())));
  }
  orc_destroy(d);
  return worst;
}

// RK4 amplification on the diagonal test operator dv/dt = i*omega*v
// (test/test_time_steping/test_ts_mod.f90:7-73 with models/iomega_model):
// one rk4_mod.f90:20-42 step from v=1 must equal 1+z+z^2/2+z^3/6+z^4/24,
// z = dt*omega.  Returns sum |numeric - analytic| over the 10 modes.
double orc_golden_rk4_iomega(void) {
  typedef std::complex<double> C;
  const int n = 10;
  const double day = 24.0 * 3600.0, dt = 6.0 * 3600.0;
  std::vector<C> om(n), v0(n, C(1.0, 0.0)), k1(n), k2(n), k3(n), k4(n), y(n);
  // cmplx() without a kind argument yields default (single precision) parts
  for (int i = 0; i < n; ++i)
    om[i] = C((double)(float)(1.0 / (day * (i + 1))), (double)(float)(2.0 * PI * (i + 1) / day));
  auto A = [&](std::vector<C>& out, const std::vector<C>& in) {
    for (int i = 0; i < n; ++i) out[i] = om[i] * in[i];
  };
  A(k1, v0);
  for (int i = 0; i < n; ++i) y[i] = 1.0 * v0[i] + (0.5 * dt) * k1[i];
  A(k2, y);
  for (int i = 0; i < n; ++i) y[i] = 1.0 * v0[i] + (0.5 * dt) * k2[i];
  A(k3, y);
  for (int i = 0; i < n; ++i) y[i] = 1.0 * v0[i] + dt * k3[i];
  A(k4, y);
  double err = 0.0;
  for (int i = 0; i < n; ++i) {
    C x = v0[i];
    x = x + (dt / 6.0) * k1[i] + (dt / 3.0) * k2[i];
    x = x + (dt / 3.0) * k3[i] + (dt / 6.0) * k4[i];
    const C z = dt * om[i];
    const C z2 = z * z, z3 = z2 * z, z4 = z3 * z;
    const C tr = 1.0 + z + 0.5 * z2 + z3 / 6.0 + z4 / 24.0;
    err += std::abs(x - tr);
  }
  return err;
}

}  // extern "C"
