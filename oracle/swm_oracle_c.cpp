// swm_oracle_c.cpp -- FP64 CPU oracle of the C-grid SBP vector-invariant
// shallow-water operator (the &shallow_water_model_c family of the reference's
// namelist_swm:80-102: divergence_c_sbp42, gradient_c_sbp42, curl_c_sbp42,
// coriolis_Cgrid_sbp42, KE_Cgrid_sbp42, co2contra_c_sbp42, massflux_c_sbp42,
// SBP_C42_quadrature, and their sbp21 counterparts).
//
// TEST INFRASTRUCTURE ONLY (see swm_oracle.h).  Every routine names the
// reference file:line it restates.  One tile per panel, as on one GPU.
//
// Meshes (mesh_factory_mod.f90:25-133 with the C staggering of
// domain_factory_mod.f90:108-112), dense FP64 arrays, i fastest, then j, then
// panel; 0-based (i, j) is the reference's (i+1, j+1):
//   mesh 0 "p" (o, cell centres)  N   x N     alpha = -pi/4 + (i + 1/2) hx
//   mesh 1 "u" (x, x-faces)       N+1 x N     alpha = -pi/4 + i hx
//   mesh 2 "v" (y, y-faces)       N   x N+1   beta  = -pi/4 + j hx
//   mesh 3 "q" (xy, corners)      N+1 x N+1
// h lives on p, the covariant u on u, v on v, the curl on q.

#include "swm_oracle.h"
#include "swm_oracle_common.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

namespace {

using namespace orc_common;

// ---------------------------------------------------------------------------
// Staggered 1D SBP operators (sbp_operator_mod.f90:12-38 and sbp_apply
// 152-228; sbp_factory_mod.f90:38-179; the staggered tables of
// sbp_operators_collection_mod.f90:88-193).  Ql[r*nw + m] multiplies input m
// for left closure row r (0-based).  The right block is the mirror image of
// the left one times rsign (-1 for differences, +1 for interpolations), the
// interior stencil covers inputs k+inshift .. k+inshift+w-1 for output k.
// dnx = n_out - n_in.  proj and Aout are the boundary projection and the
// output-grid mass matrix of the SAT penalties.
// ---------------------------------------------------------------------------
struct Stag {
  int ne = 0, nw = 0;
  std::vector<double> Ql;
  std::vector<int> last;
  std::vector<double> Qin;
  int inshift = 0, dnx = 0;
  double rsign = 1.0;
  std::vector<double> proj, Aout;
};

enum StagId { W21_C2I, W21_I2C, W42_C2I, W42_I2C, D21_C2I, D21_I2C, D42_C2I, D42_I2C };

// The four staggered operators of one SBP order.
struct Ops {
  int order = 42;
  Stag Wc2i, Wi2c, Dc2i, Di2c;
};

Stag make_stag(StagId id) {
  Stag s;
  switch (id) {
    case W21_C2I:  // W21_stagered_interp_c2i
      s.ne = 1; s.nw = 1; s.Ql = {1.0}; s.last = {1};
      s.Qin = {0.5, 0.5}; s.inshift = -1; s.dnx = 1; s.rsign = 1.0;
      break;
    case W21_I2C:  // W21_stagered_interp_i2c
      s.ne = 1; s.nw = 2; s.Ql = {0.5, 0.5}; s.last = {2};
      s.Qin = {0.5, 0.5}; s.inshift = 0; s.dnx = -1; s.rsign = 1.0;
      break;
    case W42_C2I:  // W42_stagered_interp_c2i (the opt1 closure)
      s.ne = 4; s.nw = 5;
      s.Ql = {1.3630402181345285, -0.17804474904273135, -0.23303115631809243, 0.048035687226327554, 0.0,
              0.46340770044238916, 0.4765661872892848, 0.15664452409426372, -0.09661841182593758, 0.0,
              0.07545241951434666, 0.44794495248229815, 0.37775283649236274, 0.09884979151099299, 0.0,
              -0.04413695843145285, -0.04040344754874627, 0.649837488701711, 0.4980831989686297, -0.06338028169014084};
      s.last = {4, 4, 4, 5};
      s.Qin = {-1.0 / 16.0, 9.0 / 16.0, 9.0 / 16.0, -1.0 / 16.0}; s.inshift = -2; s.dnx = 1; s.rsign = 1.0;
      break;
    case W42_I2C:  // W42_stagered_interp_i2c (the opt1 closure)
      s.ne = 4; s.nw = 6;
      s.Ql = {0.4892964885611128, 0.48123107353632727, 0.0696483872440123, -0.040175949341450676, 0.0, 0.0,
              -0.07913099957454726, 0.6127279550862234, 0.5119370885511979, -0.045534044062872786, 0.0, 0.0,
              -0.0869982983587545, 0.1691760860218048, 0.3626427230326682, 0.6151794893042863, -0.06, 0.0,
              0.018680545032460714, -0.10869571330417979, 0.09884979151099299, 0.4911653767607321, 0.5625, -0.0625};
      s.last = {4, 4, 5, 6};
      s.Qin = {-1.0 / 16.0, 9.0 / 16.0, 9.0 / 16.0, -1.0 / 16.0}; s.inshift = -1; s.dnx = -1; s.rsign = 1.0;
      break;
    case D21_C2I:
      s.ne = 1; s.nw = 2; s.Ql = {-1.0, 1.0}; s.last = {2};
      s.Qin = {-1.0, 1.0}; s.inshift = -1; s.dnx = 1; s.rsign = -1.0;
      s.proj = {1.5, -0.5}; s.Aout = {0.5, 1.0};           // D21_A_interfaces
      break;
    case D21_I2C:
      s.ne = 1; s.nw = 2; s.Ql = {-1.0, 1.0}; s.last = {2};
      s.Qin = {-1.0, 1.0}; s.inshift = 0; s.dnx = -1; s.rsign = -1.0;
      s.proj = {1.5, -0.5}; s.Aout = {1.0, 1.0};           // D21_A_centers
      break;
    case D42_C2I:
      s.ne = 4; s.nw = 5;
      s.Ql = {-2.0, 3.0, -1.0, 0.0, 0.0,
              -1.0, 1.0, 0.0, 0.0, 0.0,
              1.0 / 24.0, -9.0 / 8.0, 9.0 / 8.0, -1.0 / 24.0, 0.0,
              -1.0 / 71.0, 6.0 / 71.0, -83.0 / 71.0, 81.0 / 71.0, -3.0 / 71.0};
      s.last = {3, 2, 4, 5};
      s.Qin = {1.0 / 24.0, -9.0 / 8.0, 9.0 / 8.0, -1.0 / 24.0}; s.inshift = -2; s.dnx = 1; s.rsign = -1.0;
      s.proj = {15.0 / 8.0, -5.0 / 4.0, 3.0 / 8.0};
      s.Aout = {7.0 / 18.0, 9.0 / 8.0, 1.0, 71.0 / 72.0, 1.0};  // D42_A_interfaces
      break;
    case D42_I2C:
      s.ne = 3; s.nw = 5;
      s.Ql = {-79.0 / 78.0, 27.0 / 26.0, -1.0 / 26.0, 1.0 / 78.0, 0.0,
              2.0 / 21.0, -9.0 / 7.0, 9.0 / 7.0, -2.0 / 21.0, 0.0,
              1.0 / 75.0, 0.0, -27.0 / 25.0, 83.0 / 75.0, -1.0 / 25.0};
      s.last = {4, 4, 5};
      s.Qin = {1.0 / 24.0, -9.0 / 8.0, 9.0 / 8.0, -1.0 / 24.0}; s.inshift = -1; s.dnx = -1; s.rsign = -1.0;
      s.proj = {15.0 / 8.0, -5.0 / 4.0, 3.0 / 8.0};
      s.Aout = {13.0 / 12.0, 7.0 / 8.0, 25.0 / 24.0, 1.0};  // D42_A_centers
      break;
  }
  return s;
}

// sbp_apply (sbp_operator_mod.f90:152-228) for output k (0-based) of a line
// of nout outputs over nin = nout - dnx inputs f[m*st].
inline double stag_point(const Stag& s, const double* f, int nout, int st, int k) {
  const int nin = nout - s.dnx;
  double acc = 0.0;
  if (k < s.ne) {
    const double* q = &s.Ql[k * s.nw];
    for (int m = 0; m < s.last[k]; ++m) acc += q[m] * f[m * st];
  } else if (k < nout - s.ne) {
    const int w = (int)s.Qin.size();
    for (int t = 0; t < w; ++t) acc += s.Qin[t] * f[(k + s.inshift + t) * st];
  } else {
    // Qr(nwst:nw, ir) * f(mx:nin): the outermost input first
    const int r = nout - 1 - k;
    const double* q = &s.Ql[r * s.nw];
    for (int m = s.last[r] - 1; m >= 0; --m) acc += (s.rsign * q[m]) * f[(nin - 1 - m) * st];
  }
  return acc;
}

// ---------------------------------------------------------------------------
// Meshes and the cross halos of the one-tile-per-panel exchanges.
// ---------------------------------------------------------------------------
struct Mesh {
  int nx = 0, ny = 0;
  double si = 0.5, sj = 0.5;  // shift_i, shift_j of mesh_factory_mod.f90:34-41
  std::vector<double> J, Qi1, Qi2, Qi3, Q1, Q2, Q3, rx, ry, rz, f, a1, a2, b1, b2;
  int size() const { return 6 * nx * ny; }
  int at(int p, int i, int j) const { return (p * ny + j) * nx + i; }
};

// Halo slot of panel p, side s (0 left i<0, 1 right i>=nx, 2 bottom j<0,
// 3 top j>=ny), depth d = 1..kDepth, along-side index k: the sender's dense
// index, whether the sender value is the other vector component, and the sign.
constexpr int kDepth = 5;  // 3 for the C-grid operators, 5 for the ECS_O corner formulas
struct HaloSrc {
  int idx = -1;
  bool other = false;
  double sign = 1.0;
};
struct Halo {
  int len[4] = {0, 0, 0, 0};
  std::vector<HaloSrc> slot[4];  // [p][d-1][k]
  const HaloSrc& get(int p, int s, int d, int k) const { return slot[s][(p * kDepth + d - 1) * len[s] + k]; }
};

// create_o_points_halo_exchange / create_symm_halo_vec_exchange_U/V_points
// (parallel/exchange_factory_mod.f90:13-156, 334-617) and the vector packing
// of buffer_mod.f90:278-475, restricted to the cross halos the C-grid SBP
// operators read: the neighbour's points are placed by transform_index with
// the receiving mesh's point counts, so the duplicated edge faces of u (v)
// land in the first x (y) halo layer.  kind: 0 scalar on mesh T, 1 the u
// component of a C vector (T = u), 2 the v component (T = v).
Halo build_halo(const Mesh& T, const Mesh& other, int kind) {
  Halo h;
  h.len[0] = h.len[1] = T.ny;
  h.len[2] = h.len[3] = T.nx;
  for (int s = 0; s < 4; ++s) h.slot[s].assign((size_t)6 * kDepth * h.len[s], HaloSrc{});
  for (int p = 0; p < 6; ++p)
    for (int q = 0; q < 6; ++q) {
      if (q == p) continue;
      int istep, jstep; bool dim_i;
      basis_orientation(p, q, istep, jstep, dim_i);  // (receiver, sender)
      const bool swap = kind != 0 && !dim_i;
      const Mesh& S = swap ? other : T;
      double sign = 1.0;
      if (kind == 1) sign = dim_i ? istep : jstep;
      if (kind == 2) sign = dim_i ? jstep : istep;
      for (int js = 1; js <= S.ny; ++js)
        for (int is = 1; is <= S.nx; ++is) {
          int it, jt;
          transform_index(q, is, js, p, T.nx, T.ny, it, jt);
          int s = -1, d = 0, k = 0;
          if (it <= 0 && it > -kDepth && jt >= 1 && jt <= T.ny) { s = 0; d = 1 - it; k = jt - 1; }
          else if (it > T.nx && it <= T.nx + kDepth && jt >= 1 && jt <= T.ny) { s = 1; d = it - T.nx; k = jt - 1; }
          else if (jt <= 0 && jt > -kDepth && it >= 1 && it <= T.nx) { s = 2; d = 1 - jt; k = it - 1; }
          else if (jt > T.ny && jt <= T.ny + kDepth && it >= 1 && it <= T.nx) { s = 3; d = jt - T.ny; k = it - 1; }
          if (s < 0) continue;
          HaloSrc& e = h.slot[s][(p * kDepth + d - 1) * h.len[s] + k];
          e.idx = S.at(q, is - 1, js - 1);
          e.other = swap;
          e.sign = sign;
        }
    }
  for (int s = 0; s < 4; ++s)
    for (const HaloSrc& e : h.slot[s])
      if (e.idx < 0) std::abort();  // every cross-halo slot has a sender
  return h;
}

// Value of field f of mesh M at extended 0-based (i, j) of panel p; g is the
// other component of a vector (nullptr for scalars).
inline double ext(const Mesh& M, const Halo& H, const double* f, const double* g, int p, int i, int j) {
  if (i >= 0 && i < M.nx && j >= 0 && j < M.ny) return f[M.at(p, i, j)];
  int s, d, k;
  if (i < 0) { s = 0; d = -i; k = j; }
  else if (i >= M.nx) { s = 1; d = i - M.nx + 1; k = j; }
  else if (j < 0) { s = 2; d = -j; k = i; }
  else { s = 3; d = j - M.ny + 1; k = i; }
  const HaloSrc& e = H.get(p, s, d, k);
  return e.sign * (e.other ? g[e.idx] : f[e.idx]);
}

}  // namespace

struct orcc_domain {
  int N = 0, order = 42;
  double hx = 0.0, scale = 1.0, grav = 9.80616, omega = 1.0, axis[3] = {0, 0, 1};
  Mesh m[4];               // p, u, v, q
  Halo ho, hu, hv, hq;     // scalar on p, C vector u / v, scalar on q
  Halo hau, hav;           // A vector (both components on p): u / v
  Ops ops;    // the operators of the model's SBP order
  Ops ops21;  // the 2/1 operators of the C-grid hyperdiffusion
  std::vector<double> Ac, Ai;
  // ECS_O halo: cubic weights [row 0..1][position -1..N+2][4] and stencil bases
  std::vector<double> ecs_w;
  std::vector<int> ecs_ind;
  // ecs_A_vec: the 2x2 maps [edge 0..3][depth 1..kDepth][position 1..N][4]
  std::vector<double> ecs_tm;
  // ECS_xy: cubic weights [row 0..kXyRows-1][position 1-kXyRows..n+kXyRows][4], bases
  std::vector<double> xy_w;
  std::vector<int> xy_ind;  // quadrature edge weights at centres / interfaces
};

namespace {

int nthreads() { return orc_get_threads(); }

void build_mesh(orcc_domain& d, Mesh& M, int nx, int ny, double si, double sj) {
  M.nx = nx; M.ny = ny; M.si = si; M.sj = sj;
  const int np = M.size();
  for (auto* v : {&M.J, &M.Qi1, &M.Qi2, &M.Qi3, &M.Q1, &M.Q2, &M.Q3, &M.rx, &M.ry, &M.rz, &M.f}) v->assign(np, 0.0);
  for (auto* v : {&M.a1, &M.a2, &M.b1, &M.b2}) v->assign(3 * (size_t)np, 0.0);
  for (int p = 0; p < 6; ++p)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int id = M.at(p, i, j);
        // get_alpha / get_beta: alpha_0 + (i - 1 + shift_i) hx with 1-based i
        const double al = -0.25 * PI + (i + si) * d.hx, be = -0.25 * PI + (j + sj) * d.hx;
        const double ta = std::tan(al), tb = std::tan(be);
        const double sg = std::sqrt(1.0 + ta * ta + tb * tb);
        M.J[id] = (1.0 + ta * ta) * (1.0 + tb * tb) / (sg * sg * sg);
        M.Qi1[id] = sg * sg / (1.0 + ta * ta);
        M.Qi2[id] = sg * sg * ta * tb / ((1.0 + ta * ta) * (1.0 + tb * tb));
        M.Qi3[id] = sg * sg / (1.0 + tb * tb);
        // ecs_Q (ecs_metric_mod.f90:401-419)
        const double s4 = sg * sg * sg * sg;
        M.Q1[id] = (1.0 + ta * ta) * (1.0 + ta * ta) * (1.0 + tb * tb) / s4;
        M.Q2[id] = -(1.0 + ta * ta) * (1.0 + tb * tb) * ta * tb / s4;
        M.Q3[id] = (1.0 + ta * ta) * (1.0 + tb * tb) * (1.0 + tb * tb) / s4;
        double v[3], w[3];
        r_proto(al, be, v); to_face(p, v, w);
        M.rx[id] = w[0]; M.ry[id] = w[1]; M.rz[id] = w[2];
        const double nn = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        const double pr = (d.axis[0] * w[0] + d.axis[1] * w[1] + d.axis[2] * w[2]) / nn;
        M.f[id] = 2.0 * d.omega * pr;  // calc_coriolis_parameter (coriolis_factory_mod.f90:151-172)
        a1_proto(al, be, v); to_face(p, v, &M.a1[3 * id]);
        a2_proto(al, be, v); to_face(p, v, &M.a2[3 * id]);
        b1_proto(al, be, v); to_face(p, v, &M.b1[3 * id]);
        b2_proto(al, be, v); to_face(p, v, &M.b2[3 * id]);
      }
}

// Fill out[k] = op applied along x (dir 0) or y (dir 1) from the input mesh
// I to the output mesh O (sbp_apply over every output point).
void stag_apply(const Stag& s, const Mesh& I, const double* f, const Mesh& O, double* out, int dir) {
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int pj = 0; pj < 6 * O.ny; ++pj) {
    const int p = pj / O.ny, j = pj % O.ny;
    for (int i = 0; i < O.nx; ++i) {
      if (dir == 0) out[O.at(p, i, j)] = stag_point(s, &f[I.at(p, 0, j)], O.nx, 1, i);
      else out[O.at(p, i, j)] = stag_point(s, &f[I.at(p, i, 0)], O.ny, I.nx, j);
    }
  }
}

// ------------------------------------------------------------- co2contra
// co2contra_c_sbp42 (co2contra/co2contra_Cgrid_mod.f90:292-437): the other
// covariant component is interpolated to the centres, multiplied by J Qi12
// there, interpolated to the faces and divided by J.  co2contra_c_sbp21
// (226-290) is the same chain with the 2nd-order W21 weights.
void co2contra(const orcc_domain& d, const Ops& o, const double* u, const double* v, double* ut, double* vt) {
  const Mesh &P = d.m[0], &U = d.m[1], &V = d.m[2];
  std::vector<double> a(P.size()), b(P.size()), t(U.size()), s(V.size());
  stag_apply(o.Wi2c, V, v, P, a.data(), 1);
  stag_apply(o.Wi2c, U, u, P, b.data(), 0);
  for (int k = 0; k < P.size(); ++k) {
    a[k] = P.J[k] * P.Qi2[k] * a[k];
    b[k] = P.J[k] * P.Qi2[k] * b[k];
  }
  stag_apply(o.Wc2i, P, a.data(), U, t.data(), 0);
  stag_apply(o.Wc2i, P, b.data(), V, s.data(), 1);
  for (int k = 0; k < U.size(); ++k) ut[k] = U.Qi1[k] * u[k] + t[k] / U.J[k];
  for (int k = 0; k < V.size(); ++k) vt[k] = V.Qi3[k] * v[k] + s[k] / V.J[k];
}

// massflux_c_sbp42 / _sbp21 (massflux/massflux_Cgrid_mod.f90:230-358):
// h interpolated to the faces times the contravariant velocity.
void massflux(const orcc_domain& d, const double* h, const double* ut, const double* vt, double* hu, double* hv) {
  const Mesh &P = d.m[0], &U = d.m[1], &V = d.m[2];
  stag_apply(d.ops.Wc2i, P, h, U, hu, 0);
  for (int k = 0; k < U.size(); ++k) hu[k] = ut[k] * hu[k];
  stag_apply(d.ops.Wc2i, P, h, V, hv, 1);
  for (int k = 0; k < V.size(); ++k) hv[k] = vt[k] * hv[k];
}

// KE_Cgrid_sbp42 / _sbp21 (kinetic_energy/KE_Cgrid_mod.f90:21-75).
void kinetic_energy(const orcc_domain& d, const double* u, const double* v, const double* ut, const double* vt,
                    double* ke) {
  const Mesh &P = d.m[0], &U = d.m[1], &V = d.m[2];
  std::vector<double> ku(U.size()), kv(V.size()), kuh(P.size()), kvh(P.size());
  for (int k = 0; k < U.size(); ++k) ku[k] = U.J[k] * (u[k] * ut[k]) / 2.0;
  for (int k = 0; k < V.size(); ++k) kv[k] = V.J[k] * (v[k] * vt[k]) / 2.0;
  stag_apply(d.ops.Wi2c, U, ku.data(), P, kuh.data(), 0);
  stag_apply(d.ops.Wi2c, V, kv.data(), P, kvh.data(), 1);
  for (int k = 0; k < P.size(); ++k) ke[k] = (kuh[k] + kvh[k]) / P.J[k];
}

// ------------------------------------------------------------------ grad
// gradient_c_sbp42 (gradient/grad_c_sbp42_mod.f90:44-139) with the 3-wide
// o-point halo; gradient_c_sbp21 (grad_c2_ecs_mod.f90:234-293) with 2.
void grad(const orcc_domain& d, const Ops& o, const double* f, double* gx, double* gy) {
  const Mesh &P = d.m[0], &U = d.m[1], &V = d.m[2];
  const int N = d.N;
  const double dx1 = 1.0 / (d.scale * d.hx);
  const double hs = d.hx * d.scale;
  const Stag& D = o.Dc2i;  // dedge / din of grad_c_sbp42 are D42_staggered_c2i
  const double sq1 = 7.0 / 18.0;
  auto F = [&](int p, int i, int j) { return ext(P, d.ho, f, nullptr, p, i, j); };
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int p = 0; p < 6; ++p) {
    // x: line j, output i = 0..N (faces), input f(i) cells, 0-based f(i) is F(i)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i <= N; ++i) {
        double g;
        if (o.order == 21) {
          if (i == 0) g = (0.5 * F(p, 1, j) + 0.5 * F(p, 0, j) - 1.5 * F(p, -1, j) + 0.5 * F(p, -2, j)) / hs;
          else if (i == N) g = (-0.5 * F(p, N - 2, j) - 0.5 * F(p, N - 1, j) + 1.5 * F(p, N, j) - 0.5 * F(p, N + 1, j)) / hs;
          else g = (F(p, i, j) - F(p, i - 1, j)) / hs;
        } else {
          const int n1 = i + 1;  // 1-based face index; n = N+1
          if (n1 <= 4) {
            double a = 0.0;
            for (int m = 0; m < D.last[i]; ++m) a += D.Ql[i * D.nw + m] * F(p, m, j);
            g = a * dx1;
            if (i == 0) {
              const double dh = (D.proj[0] * (F(p, 0, j) - F(p, -1, j)) + D.proj[1] * (F(p, 1, j) - F(p, -2, j)) +
                                 D.proj[2] * (F(p, 2, j) - F(p, -3, j))) * dx1;
              g = g + 0.5 * dh / sq1;
            }
          } else if (n1 <= N + 1 - 4) {
            double a = 0.0;
            for (int t = 0; t < 4; ++t) a += F(p, i - 2 + t, j) * D.Qin[t];
            g = a * dx1;
          } else {
            const int i2 = N + 1 - n1;  // 0-based mirrored row
            double a = 0.0;
            for (int m = 0; m < D.last[i2]; ++m) a += D.Ql[i2 * D.nw + m] * F(p, N - 1 - m, j);
            g = -a * dx1;
            if (i == N) {
              const double dh = (D.proj[0] * (F(p, N, j) - F(p, N - 1, j)) + D.proj[1] * (F(p, N + 1, j) - F(p, N - 2, j)) +
                                 D.proj[2] * (F(p, N + 2, j) - F(p, N - 3, j))) * dx1;
              g = g + 0.5 * dh / sq1;
            }
          }
        }
        gx[U.at(p, i, j)] = g;
      }
    // y: column i, output j = 0..N
    for (int j = 0; j <= N; ++j)
      for (int i = 0; i < N; ++i) {
        double g;
        if (o.order == 21) {
          if (j == 0) g = (0.5 * F(p, i, 1) + 0.5 * F(p, i, 0) - 1.5 * F(p, i, -1) + 0.5 * F(p, i, -2)) / hs;
          else if (j == N) g = (-0.5 * F(p, i, N - 2) - 0.5 * F(p, i, N - 1) + 1.5 * F(p, i, N) - 0.5 * F(p, i, N + 1)) / hs;
          else g = (F(p, i, j) - F(p, i, j - 1)) / hs;
        } else {
          const int n1 = j + 1;
          if (n1 <= 4) {
            double a = 0.0;
            for (int m = 0; m < D.last[j]; ++m) a += D.Ql[j * D.nw + m] * F(p, i, m);
            g = a * dx1;
            if (j == 0) {
              const double dh = (D.proj[0] * (F(p, i, 0) - F(p, i, -1)) + D.proj[1] * (F(p, i, 1) - F(p, i, -2)) +
                                 D.proj[2] * (F(p, i, 2) - F(p, i, -3))) * dx1;
              g = g + 0.5 * dh / sq1;
            }
          } else if (n1 <= N + 1 - 4) {
            double a = 0.0;
            for (int t = 0; t < 4; ++t) a += F(p, i, j - 2 + t) * D.Qin[t];
            g = a * dx1;
          } else {
            const int j2 = N + 1 - n1;
            double a = 0.0;
            for (int m = 0; m < D.last[j2]; ++m) a += D.Ql[j2 * D.nw + m] * F(p, i, N - 1 - m);
            g = -a * dx1;
            if (j == N) {
              const double dh = (D.proj[0] * (F(p, i, N) - F(p, i, N - 1)) + D.proj[1] * (F(p, i, N + 1) - F(p, i, N - 2)) +
                                 D.proj[2] * (F(p, i, N + 2) - F(p, i, N - 3))) * dx1;
              g = g + 0.5 * dh / sq1;
            }
          }
        }
        gy[V.at(p, i, j)] = g;
      }
  }
}

// ------------------------------------------------------------------- div
// divergence_c_sbp42 (divergence/div_c_sbp42_mod.f90:32-107): Gu = J u on
// the faces, the C-vector exchange, D42_staggered_i2c along each direction
// plus the "at_center" SAT penalty on the jump of the duplicated edge faces
// (sbp_operator_mod.f90:318-384), divided by J hx a.  divergence_c_sbp21
// (div_c2_mod.f90:76-177) uses the raw halo values times the local J.
void div(const orcc_domain& d, const Ops& o, const double* hu, const double* hv, double* out) {
  const Mesh &P = d.m[0], &U = d.m[1], &V = d.m[2];
  const int N = d.N;
  std::vector<double> gu(U.size()), gv(V.size());
  for (int k = 0; k < U.size(); ++k) gu[k] = hu[k] * U.J[k];
  for (int k = 0; k < V.size(); ++k) gv[k] = hv[k] * V.J[k];
  const Stag& D = o.Di2c;
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int pj = 0; pj < 6 * N; ++pj) {
    const int p = pj / N, j = pj % N;
    for (int i = 0; i < N; ++i) {
      double dx, dy;
      if (o.order == 21) {
        auto u = [&](int a, int b) { return ext(U, d.hu, hu, hv, p, a, b); };
        auto v = [&](int a, int b) { return ext(V, d.hv, hv, hu, p, a, b); };
        auto Ju = [&](int a, int b) { return U.J[U.at(p, a, b)]; };
        auto Jv = [&](int a, int b) { return V.J[V.at(p, a, b)]; };
        // 1-based i' = i+1; u(i') is 0-based u(i'-1)
        if (i == 0) dx = Ju(1, j) * u(1, j) - Ju(0, j) * (0.25 * u(0, j) + 0.75 * u(-1, j));
        else if (i == 1) dx = Ju(2, j) * u(2, j) - Ju(1, j) * u(1, j) - 0.25 * Ju(0, j) * (u(0, j) - u(-1, j));
        else if (i == N - 2) dx = Ju(N - 1, j) * u(N - 1, j) - Ju(N - 2, j) * u(N - 2, j) +
                                  0.25 * Ju(N, j) * (u(N, j) - u(N + 1, j));
        else if (i == N - 1) dx = Ju(N, j) * (0.75 * u(N + 1, j) + 0.25 * u(N, j)) - Ju(N - 1, j) * u(N - 1, j);
        else dx = Ju(i + 1, j) * u(i + 1, j) - Ju(i, j) * u(i, j);
        if (j == 0) dy = Jv(i, 1) * v(i, 1) - Jv(i, 0) * (0.25 * v(i, 0) + 0.75 * v(i, -1));
        else if (j == 1) dy = Jv(i, 2) * v(i, 2) - Jv(i, 1) * v(i, 1) - 0.25 * Jv(i, 0) * (v(i, 0) - v(i, -1));
        else if (j == N - 2) dy = Jv(i, N - 1) * v(i, N - 1) - Jv(i, N - 2) * v(i, N - 2) +
                                  0.25 * Jv(i, N) * (v(i, N) - v(i, N + 1));
        else if (j == N - 1) dy = Jv(i, N) * (0.75 * v(i, N + 1) + 0.25 * v(i, N)) - Jv(i, N - 1) * v(i, N - 1);
        else dy = Jv(i, j + 1) * v(i, j + 1) - Jv(i, j) * v(i, j);
      } else {
        auto Gu = [&](int a, int b) { return ext(U, d.hu, gu.data(), gv.data(), p, a, b); };
        auto Gv = [&](int a, int b) { return ext(V, d.hv, gv.data(), gu.data(), p, a, b); };
        dx = stag_point(D, &gu[U.at(p, 0, j)], N, 1, i);
        dy = stag_point(D, &gv[V.at(p, i, 0)], N, V.nx, j);
        const int ne = (int)D.proj.size();
        if (i < ne) dx = dx + 0.5 * (D.proj[i] / D.Aout[i]) * (Gu(0, j) - Gu(-1, j));
        if (i >= N - ne) {
          const int r = N - 1 - i;  // mirrored penalty_r
          dx = dx + 0.5 * (D.proj[r] / D.Aout[r]) * (Gu(N + 1, j) - Gu(N, j));
        }
        if (j < ne) dy = dy + 0.5 * (D.proj[j] / D.Aout[j]) * (Gv(i, 0) - Gv(i, -1));
        if (j >= N - ne) {
          const int r = N - 1 - j;
          dy = dy + 0.5 * (D.proj[r] / D.Aout[r]) * (Gv(i, N + 1) - Gv(i, N));
        }
      }
      out[P.at(p, i, j)] = (dx + dy) / (P.J[P.at(p, i, j)] * d.hx * d.scale);
    }
  }
}

// Ah-type scalar sync of the corner points (halo/halo_Ah_scalar_sync_mod.f90:
// 38-93): edge points are the average of their two copies, cube corners of
// their three.
void sync_q(const orcc_domain& d, double* f) {
  const Mesh& Q = d.m[3];
  const int n = Q.nx, e = n - 1;
  std::vector<double> ring(6 * 4 * (size_t)n);
  for (int p = 0; p < 6; ++p)
    for (int k = 0; k < n; ++k) {
      ring[(p * 4 + 0) * n + k] = ext(Q, d.hq, f, nullptr, p, -1, k);
      ring[(p * 4 + 1) * n + k] = ext(Q, d.hq, f, nullptr, p, n, k);
      ring[(p * 4 + 2) * n + k] = ext(Q, d.hq, f, nullptr, p, k, -1);
      ring[(p * 4 + 3) * n + k] = ext(Q, d.hq, f, nullptr, p, k, n);
    }
  for (int p = 0; p < 6; ++p) {
    const double* L = &ring[(p * 4 + 0) * n];
    const double* R = &ring[(p * 4 + 1) * n];
    const double* B = &ring[(p * 4 + 2) * n];
    const double* T = &ring[(p * 4 + 3) * n];
    auto at = [&](int i, int j) -> double& { return f[Q.at(p, i, j)]; };
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

// ------------------------------------------------------------------ curl
// curl_c_sbp42 / _sbp21 (curl/curl_c_sbp_mod.f90:21-127): D_staggered_c2i of
// the covariant components onto the corners, the SAT penalties on the jumps
// across the panel edges, division by J hx a, then the Ah scalar sync
// (curl_factory_mod.f90:56-88).
void curl(const orcc_domain& d, const Ops& o, const double* u, const double* v, double* out) {
  const Mesh &U = d.m[1], &V = d.m[2], &Q = d.m[3];
  const int N = d.N, nq = N + 1;
  const Stag& D = o.Dc2i;
  const int np = (int)D.proj.size();
  const double al = D.Aout[0];  // Al_out(1) = Ar_out(end)
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int pj = 0; pj < 6 * nq; ++pj) {
    const int p = pj / nq, j = pj % nq;
    auto vv = [&](int a, int b) { return ext(V, d.hv, v, u, p, a, b); };
    auto uu = [&](int a, int b) { return ext(U, d.hu, u, v, p, a, b); };
    for (int i = 0; i < nq; ++i) {
      double dvx = stag_point(D, &v[V.at(p, 0, j)], nq, 1, i);
      if (i == 0) {
        double dv = 0.0;
        for (int m = 0; m < np; ++m) dv = dv + D.proj[m] * (vv(m, j) - vv(-1 - m, j));
        dvx = dvx + 0.5 * dv / al;
      }
      if (i == N) {
        double dv = 0.0;
        for (int m = 0; m < np; ++m) dv = dv + D.proj[m] * (vv(N + m, j) - vv(N - 1 - m, j));
        dvx = dvx + 0.5 * dv / al;
      }
      double duy = stag_point(D, &u[U.at(p, i, 0)], nq, U.nx, j);
      if (j == 0) {
        double du = 0.0;
        for (int m = 0; m < np; ++m) du = du + D.proj[m] * (uu(i, m) - uu(i, -1 - m));
        duy = duy + 0.5 * du / al;
      }
      if (j == N) {
        double du = 0.0;
        for (int m = 0; m < np; ++m) du = du + D.proj[m] * (uu(i, N + m) - uu(i, N - 1 - m));
        duy = duy + 0.5 * du / al;
      }
      out[Q.at(p, i, j)] = (dvx - duy) / (Q.J[Q.at(p, i, j)] * d.hx * d.scale);
    }
  }
  sync_q(d, out);
}

// -------------------------------------------------------------- coriolis
// coriolis_Cgrid_sbp42 / _sbp21 (coriolis/coriolis_Cgrid_mod.f90:38-118 with
// the interpolators of interpolator_2d/*: uv2pvec, w2h, pvec2uv).
void coriolis(const orcc_domain& d, const double* hu, const double* hv, const double* h, const double* cu,
              double* cor_u, double* cor_v) {
  const Mesh &P = d.m[0], &U = d.m[1], &V = d.m[2], &Q = d.m[3];
  std::vector<double> gu(U.size()), gv(V.size()), gup(P.size()), gvp(P.size());
  std::vector<double> fu(U.size()), fv(V.size()), fuh(P.size()), fvh(P.size()), cp(P.size());
  std::vector<double> cup(P.size()), cvp(P.size());
  for (int k = 0; k < U.size(); ++k) gu[k] = U.J[k] * hu[k];
  for (int k = 0; k < V.size(); ++k) gv[k] = V.J[k] * hv[k];
  stag_apply(d.ops.Wi2c, U, gu.data(), P, gup.data(), 0);
  stag_apply(d.ops.Wi2c, V, gv.data(), P, gvp.data(), 1);
  // interp_w2h (interpolator_w2h_mod.f90:25-67)
  stag_apply(d.ops.Wi2c, Q, cu, V, fv.data(), 0);
  stag_apply(d.ops.Wi2c, Q, cu, U, fu.data(), 1);
  stag_apply(d.ops.Wi2c, U, fu.data(), P, fuh.data(), 0);
  stag_apply(d.ops.Wi2c, V, fv.data(), P, fvh.data(), 1);
  for (int k = 0; k < P.size(); ++k) {
    cp[k] = 0.5 * fuh[k] + 0.5 * fvh[k];
    cup[k] = (P.f[k] + cp[k]) * gvp[k] / h[k];
    cvp[k] = -(P.f[k] + cp[k]) * gup[k] / h[k];
  }
  stag_apply(d.ops.Wc2i, P, cup.data(), U, cor_u, 0);
  stag_apply(d.ops.Wc2i, P, cvp.data(), V, cor_v, 1);
  (void)Q;
}

// ------------------------------------------------------------- grad_perp
// grad_perp_c_sbp21 / _sbp42 (grad_perp/grad_perp_c_sbp_mod.f90:20-95,
// grad_perp_factory_mod.f90:24-55): D_staggered_i2c of the corner field w
// along y onto the x-faces and along x onto the y-faces, each with the
// "at_center" SAT penalty (sbp_operator_mod.f90:343-391) on the jump between
// the panel's edge point and the neighbour's copy of it in the first halo
// layer; gu = -(.) / (a hx J_u), gv = (.) / (a hx J_v).
void grad_perp(const orcc_domain& d, const Ops& o, const double* w, double* gu, double* gv) {
  const Mesh &U = d.m[1], &V = d.m[2], &Q = d.m[3];
  const int N = d.N;
  const Stag& D = o.Di2c;
  const int ne = (int)D.proj.size();
  auto W = [&](int p, int i, int j) { return ext(Q, d.hq, w, nullptr, p, i, j); };
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int p = 0; p < 6; ++p) {
    for (int j = 0; j < N; ++j)  // x-faces: along y
      for (int i = 0; i <= N; ++i) {
        double g = stag_point(D, &w[Q.at(p, i, 0)], N, Q.nx, j);
        if (j < ne) g = g + 0.5 * (D.proj[j] / D.Aout[j]) * (W(p, i, 0) - W(p, i, -1));
        if (j >= N - ne) {
          const int r = N - 1 - j;
          g = g + 0.5 * (D.proj[r] / D.Aout[r]) * (W(p, i, N + 1) - W(p, i, N));
        }
        const int e = U.at(p, i, j);
        gu[e] = -g / (d.scale * d.hx * U.J[e]);
      }
    for (int j = 0; j <= N; ++j)  // y-faces: along x
      for (int i = 0; i < N; ++i) {
        double g = stag_point(D, &w[Q.at(p, 0, j)], N, 1, i);
        if (i < ne) g = g + 0.5 * (D.proj[i] / D.Aout[i]) * (W(p, 0, j) - W(p, -1, j));
        if (i >= N - ne) {
          const int r = N - 1 - i;
          g = g + 0.5 * (D.proj[r] / D.Aout[r]) * (W(p, N + 1, j) - W(p, N, j));
        }
        const int e = V.at(p, i, j);
        gv[e] = g / (d.scale * d.hx * V.J[e]);
      }
  }
}

// ------------------------------------------------------------- contra2co
// transform2co of co2contra_c_sbp21_new / _sbp42_new (co2contra/
// co2contra_Cgrid_mod.f90:135-203, the interpolators interp2d_uv2pvec_C and
// interp2d_pvec2uv_C of interpolator2d_factory_mod.f90:47-58): the
// contravariant components interpolated to the centres, times J Q12 there,
// swapped, interpolated back to the faces, divided by J and added to
// Q11 u^1 (Q22 u^2).
void contra2co(const orcc_domain& d, const Ops& o, const double* ut, const double* vt, double* u, double* v) {
  const Mesh &P = d.m[0], &U = d.m[1], &V = d.m[2];
  std::vector<double> uh(P.size()), vh(P.size()), a(U.size()), b(V.size());
  stag_apply(o.Wi2c, U, ut, P, uh.data(), 0);
  stag_apply(o.Wi2c, V, vt, P, vh.data(), 1);
  for (int k = 0; k < P.size(); ++k) {
    const double x = uh[k] * P.J[k] * P.Q2[k];
    const double y = vh[k] * P.J[k] * P.Q2[k];
    uh[k] = y;
    vh[k] = x;
  }
  stag_apply(o.Wc2i, P, uh.data(), U, a.data(), 0);
  stag_apply(o.Wc2i, P, vh.data(), V, b.data(), 1);
  for (int k = 0; k < U.size(); ++k) u[k] = U.Q1[k] * ut[k] + a[k] / U.J[k];
  for (int k = 0; k < V.size(); ++k) v[k] = V.Q3[k] * vt[k] + b[k] / V.J[k];
}

// ---------------------------------------------------------- hyperdiffusion
// diff_coeff^(2 diff_order) with its sign, diff_order 2: -(c^4), c = coeff a hx
// (hordiff_factory_mod.f90:96-100, 132-136, 243-246).
double diff_c4(const orcc_domain& d, double coeff) {
  const double c = coeff * d.scale * d.hx;
  const double c2 = c * c;
  return -(c2 * c2);
}

// The C-grid vector hyperdiffusion (hordiff/hordiff_Cgrid_mod.f90:59-140)
// with the 2/1 operators of hordiff_factory_mod.f90:53-139.  parts: 1 the
// divergence part (hordiff_c_biharm_div), 2 the curl part
// (hordiff_c_biharm_curl), 3 both (hordiff_c_biharm_curl_div):
//   div part   c4 grad div co2contra grad div co2contra (u, v)
//   curl part  c4 contra2co grad_perp curl contra2co grad_perp curl (u, v)
// summed as u_tend = c4 A + 1.0 (c4 B).
void hordiff_uv(const orcc_domain& d, int parts, double coeff, const double* u, const double* v, double* tu,
                double* tv) {
  const Ops& o = d.ops21;
  const Mesh &P = d.m[0], &U = d.m[1], &V = d.m[2], &Q = d.m[3];
  const double c4 = diff_c4(d, coeff);
  std::vector<double> ut(U.size()), vt(V.size()), a(U.size()), b(V.size()), dv(P.size()), cq(Q.size());
  std::vector<double> cu(U.size(), 0.0), cv(V.size(), 0.0);
  if (parts & 2) {
    curl(d, o, u, v, cq.data());
    grad_perp(d, o, cq.data(), ut.data(), vt.data());
    contra2co(d, o, ut.data(), vt.data(), a.data(), b.data());
    curl(d, o, a.data(), b.data(), cq.data());
    grad_perp(d, o, cq.data(), ut.data(), vt.data());
    contra2co(d, o, ut.data(), vt.data(), a.data(), b.data());
    for (int k = 0; k < U.size(); ++k) cu[k] = c4 * a[k];
    for (int k = 0; k < V.size(); ++k) cv[k] = c4 * b[k];
  }
  if (parts & 1) {
    co2contra(d, o, u, v, ut.data(), vt.data());
    div(d, o, ut.data(), vt.data(), dv.data());
    grad(d, o, dv.data(), a.data(), b.data());
    co2contra(d, o, a.data(), b.data(), ut.data(), vt.data());
    div(d, o, ut.data(), vt.data(), dv.data());
    grad(d, o, dv.data(), ut.data(), vt.data());
    if (parts & 2) {
      for (int k = 0; k < U.size(); ++k) cu[k] = cu[k] + 1.0 * (c4 * ut[k]);
      for (int k = 0; k < V.size(); ++k) cv[k] = cv[k] + 1.0 * (c4 * vt[k]);
    } else {
      for (int k = 0; k < U.size(); ++k) cu[k] = c4 * ut[k];
      for (int k = 0; k < V.size(); ++k) cv[k] = c4 * vt[k];
    }
  }
  std::copy(cu.begin(), cu.end(), tu);
  std::copy(cv.begin(), cv.end(), tv);
}

// hordiff_scalar_C (hordiff/hordiff_scalar_mod.f90:33-53 with
// divgrad_laplace_c_sbp21, laplace/divgrad_laplace_mod.f90:23-33):
// th = c4 L(L(h)), L = div co2contra grad.
void hordiff_h(const orcc_domain& d, double coeff, const double* h, double* th) {
  const Ops& o = d.ops21;
  const Mesh &P = d.m[0], &U = d.m[1], &V = d.m[2];
  const double c4 = diff_c4(d, coeff);
  std::vector<double> f(h, h + P.size()), gx(U.size()), gy(V.size()), gxt(U.size()), gyt(V.size());
  for (int rep = 0; rep < 2; ++rep) {
    grad(d, o, f.data(), gx.data(), gy.data());
    co2contra(d, o, gx.data(), gy.data(), gxt.data(), gyt.data());
    div(d, o, gxt.data(), gyt.data(), f.data());
  }
  for (int k = 0; k < P.size(); ++k) th[k] = c4 * f[k];
}

// ------------------------------------------------------------------ ECS_O
// Weights of the ECS_O halo (equiang_cs/ecs_halo_factory_mod.f90:164-196,
// init_halo_interp): the virtual point at position i (1-based, -1..N+2) of
// halo row r (1, 2) lies on the neighbour panel's grid line r at the angle
// atan(tan(alpha_i) / tan(pi/4 + (r - 1/2) hx)); ind is the neighbour cell
// below it and the four cubic Lagrange weights take the neighbour's points
// ind-1 .. ind+2.  Returns false if a stencil used by the edge interpolation
// would leave the panel (never for N >= 12).
bool build_ecs_weights(orcc_domain& d) {
  const int N = d.N, ni = N + 4;
  d.ecs_w.assign((size_t)2 * ni * 4, 0.0);
  d.ecs_ind.assign((size_t)2 * ni, 0);
  for (int r = 1; r <= 2; ++r)
    for (int i = -1; i <= N + 2; ++i) {
      const double zb = 0.25 * PI + (r - 0.5) * d.hx;
      double za = -0.25 * PI + (i - 0.5) * d.hx;
      const double zx = std::tan(za) / std::tan(zb);
      za = std::atan(zx);
      const int ind = (int)std::floor((za + 0.25 * PI - 0.5 * d.hx) / d.hx) + 1;
      const double x = (za + 0.25 * PI) / d.hx - (ind - 0.5);
      double* w = &d.ecs_w[((size_t)(r - 1) * ni + (i + 1)) * 4];
      w[0] = -x * (x - 1.0) * (x - 2.0) / 6.0;
      w[1] = (x + 1.0) * (x - 1.0) * (x - 2.0) / 2.0;
      w[2] = -(x + 1.0) * x * (x - 2.0) / 2.0;
      w[3] = (x + 1.0) * x * (x - 1.0) / 6.0;
      d.ecs_ind[(size_t)(r - 1) * ni + (i + 1)] = ind;
      const bool used = r == 1 ? (i >= 2 && i <= N - 1) : (i >= 1 && i <= N);
      if (used && (ind - 1 < 1 || ind + 2 > N)) return false;
    }
  return true;
}

// ECS_O halo of width hw (1 or 2) of one panel (ecs_halo_mod.f90:95-475 after
// the 'full' o-point exchange): E is the extended panel, 1-based (i, j) in
// [1-hw, N+hw]^2, row-major with width N + 2 hw.  The interior is f; the
// cross halos are the exchanged neighbour values interpolated along each
// edge (ecs_ext_halo_1e; the first row leaves its two end points to the
// corners); the points next to and in each cube corner come from the corner
// formulas of ecs_halo_1corner on the exchanged values.  No formula reads the
// exchange's corner regions, which the one-tile-per-panel exchange leaves
// unfilled.
// X(i1, j1) gives the exchanged value at a halo point (and the field inside
// the panel); the vector halo passes its edge-transformed components.
template <class Xf>
void ecs_o_panel_x(const orcc_domain& d, Xf X, int hw, double* E) {
  const int N = d.N, W = N + 2 * hw, ni = N + 4;
  auto out = [&](int i1, int j1) -> double& { return E[(size_t)(j1 - 1 + hw) * W + (i1 - 1 + hw)]; };
  auto w = [&](int m, int i, int r) { return d.ecs_w[((size_t)(r - 1) * ni + (i + 1)) * 4 + (m + 1)]; };
  auto ind = [&](int i, int r) { return d.ecs_ind[(size_t)(r - 1) * ni + (i + 1)]; };
  for (int j = 1; j <= N; ++j)
    for (int i = 1; i <= N; ++i) out(i, j) = X(i, j);
  // corners first, from the exchanged values (ecs_halo_corners)
  const int ist[4] = {0, N + 1, N + 1, 0}, idr[4] = {1, -1, -1, 1};
  const int jst[4] = {0, 0, N + 1, N + 1}, jdr[4] = {1, 1, -1, -1};
  double cs[4][6] = {};
  for (int c = 0; c < 4; ++c) {
    auto fc = [&](int i, int j) { return X(ist[c] + idr[c] * i, jst[c] + jdr[c] * j); };
    // the weights of corner 1, mirrored for the corners at i = N+1
    auto pw = [&](int m, int i, int r) { return idr[c] == 1 ? w(m, i, r) : w(1 - m, N + 1 - i, r); };
    const double zw = pw(-1, 1, 1), zw2 = zw * zw, zw3 = zw2 * zw;
    const double z0 = pw(0, 1, 1), z1 = pw(1, 1, 1), z2 = pw(2, 1, 1);
    double* q = cs[c];
    double zx = z0 * fc(0, 1) + z1 * fc(0, 2) + z2 * fc(0, 3);
    double zy = z0 * fc(1, 0) + z1 * fc(1, -1) + z2 * fc(1, -2);
    double zz = z0 * fc(1, 1) + z1 * fc(2, 1) + z2 * fc(3, 1);
    q[0] = (zx + zw * zy + zw2 * zz) / (1.0 - zw3);
    const double zfy1 = (zy + zw * zz + zw2 * zx) / (1.0 - zw3);
    zx = z0 * fc(1, 0) + z1 * fc(2, 0) + z2 * fc(3, 0);
    zy = z0 * fc(0, 1) + z1 * fc(-1, 1) + z2 * fc(-2, 1);
    zz = z0 * fc(1, 1) + z1 * fc(1, 2) + z2 * fc(1, 3);
    q[1] = (zx + zw * zy + zw2 * zz) / (1.0 - zw3);
    const double zfy2 = (zy + zw * zz + zw2 * zx) / (1.0 - zw3);
    double zff1 = pw(-1, 1, 2) * fc(2, 0) + pw(0, 1, 2) * fc(2, -1) + pw(1, 1, 2) * fc(2, -2) + pw(2, 1, 2) * fc(2, -3);
    double zff2 = pw(-1, 1, 2) * fc(0, 2) + pw(0, 1, 2) * fc(-1, 2) + pw(1, 1, 2) * fc(-2, 2) + pw(2, 1, 2) * fc(-3, 2);
    q[2] = 0.5 * (pw(-1, 0, 1) * zff1 + pw(0, 0, 1) * zfy1 + pw(1, 0, 1) * fc(0, 1) + pw(2, 0, 1) * fc(0, 2) +
                  pw(-1, 0, 1) * zff2 + pw(0, 0, 1) * zfy2 + pw(1, 0, 1) * fc(1, 0) + pw(2, 0, 1) * fc(2, 0));
    if (hw > 1) {
      zff1 = pw(-1, 2, 1) * fc(1, 0) + pw(0, 2, 1) * fc(1, -1) + pw(1, 2, 1) * fc(1, -2) + pw(2, 2, 1) * fc(1, -3);
      const double zff11 =
          pw(-1, 2, 2) * fc(2, -1) + pw(0, 2, 2) * fc(2, -2) + pw(1, 2, 2) * fc(2, -3) + pw(2, 2, 2) * fc(2, -4);
      zff2 = pw(-1, 2, 1) * fc(0, 1) + pw(0, 2, 1) * fc(-1, 1) + pw(1, 2, 1) * fc(-2, 1) + pw(2, 2, 1) * fc(-3, 1);
      const double zff22 =
          pw(-1, 2, 2) * fc(-1, 2) + pw(0, 2, 2) * fc(-2, 2) + pw(1, 2, 2) * fc(-3, 2) + pw(2, 2, 2) * fc(-4, 2);
      q[3] = pw(-1, 0, 2) * zff1 + pw(0, 0, 2) * fc(-1, 1) + pw(1, 0, 2) * fc(-1, 2) + pw(2, 0, 2) * fc(-1, 3);
      q[4] = pw(-1, 0, 2) * zff2 + pw(0, 0, 2) * fc(1, -1) + pw(1, 0, 2) * fc(2, -1) + pw(2, 0, 2) * fc(3, -1);
      q[5] = 0.5 * (pw(-1, -1, 2) * zff11 + pw(0, -1, 2) * zff1 + pw(1, -1, 2) * fc(-1, 1) + pw(2, -1, 2) * fc(-1, 2) +
                    pw(-1, -1, 2) * zff22 + pw(0, -1, 2) * zff2 + pw(1, -1, 2) * fc(1, -1) + pw(2, -1, 2) * fc(2, -1));
    }
  }
  // edges: rows r = 1..hw of each cross halo (ecs_halo_edges_x / _y)
  for (int r = 1; r <= hw; ++r)
    for (int i = (r == 1 ? 2 : 1); i <= (r == 1 ? N - 1 : N); ++i) {
      const int b = ind(i, r);
      auto itp = [&](auto G) {
        double s = w(-1, i, r) * G(b - 1);
        s = s + w(0, i, r) * G(b);
        s = s + w(1, i, r) * G(b + 1);
        s = s + w(2, i, r) * G(b + 2);
        return s;
      };
      out(i, 1 - r) = itp([&](int k) { return X(k, 1 - r); });
      out(i, N + r) = itp([&](int k) { return X(k, N + r); });
      out(1 - r, i) = itp([&](int k) { return X(1 - r, k); });
      out(N + r, i) = itp([&](int k) { return X(N + r, k); });
    }
  // corner points (ecs_halo_corners_put): corner-relative (0,1), (1,0), (0,0),
  // and for hw 2 (-1,0), (0,-1), (-1,-1)
  const int ci[6] = {0, 1, 0, -1, 0, -1}, cj[6] = {1, 0, 0, 0, -1, -1};
  for (int c = 0; c < 4; ++c)
    for (int k = 0; k < (hw > 1 ? 6 : 3); ++k) out(ist[c] + idr[c] * ci[k], jst[c] + jdr[c] * cj[k]) = cs[c][k];
}

void ecs_o_panel(const orcc_domain& d, const double* f, int p, int hw, double* E) {
  const Mesh& P = d.m[0];
  ecs_o_panel_x(d, [&](int i1, int j1) { return ext(P, d.ho, f, nullptr, p, i1 - 1, j1 - 1); }, hw, E);
}

// gradient_a2_ecs (gradient/grad_a2_mod.f90:19-69 with grad_factory_mod.f90:
// 105-121): the ECS_O halo of width 1, then central differences of the cell
// values, gx = 0.5 (f(i+1) - f(i-1)) / (hx a), covariant, at the centres.
void grad_a2_ecs(const orcc_domain& d, const double* f, double* gx, double* gy) {
  const Mesh& P = d.m[0];
  const int N = d.N, hw = 1, W = N + 2;
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int p = 0; p < 6; ++p) {
    std::vector<double> E((size_t)W * W, 0.0);
    ecs_o_panel(d, f, p, hw, E.data());
    auto e = [&](int i1, int j1) { return E[(size_t)j1 * W + i1]; };  // 0-based extended
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        const int ii = i + 1, jj = j + 1;
        gx[P.at(p, i, j)] = 0.5 * (e(ii + 1, jj) - e(ii - 1, jj)) / (d.hx * d.scale);
        gy[P.at(p, i, j)] = 0.5 * (e(ii, jj + 1) - e(ii, jj - 1)) / (d.hx * d.scale);
      }
  }
}

// gradient_c2_ecs (gradient/grad_c2_ecs_mod.f90:33-51, 95-144 with
// grad_factory_mod.f90:44-57): the ECS_O halo of width 1, then the first
// differences of the cell values onto the faces, gx = (f(i) - f(i-1)) / (hx a)
// on the x-faces, gy likewise on the y-faces; covariant.
void grad_c2_ecs(const orcc_domain& d, const double* f, double* gx, double* gy) {
  const Mesh &U = d.m[1], &V = d.m[2];
  const int N = d.N, W = N + 2;
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int p = 0; p < 6; ++p) {
    std::vector<double> E((size_t)W * W, 0.0);
    ecs_o_panel(d, f, p, 1, E.data());
    auto e = [&](int i1, int j1) { return E[(size_t)j1 * W + i1]; };  // 1-based, hw 1
    for (int j1 = 1; j1 <= N; ++j1)
      for (int i1 = 1; i1 <= N + 1; ++i1) gx[U.at(p, i1 - 1, j1 - 1)] = (e(i1, j1) - e(i1 - 1, j1)) / (d.hx * d.scale);
    for (int j1 = 1; j1 <= N + 1; ++j1)
      for (int i1 = 1; i1 <= N; ++i1) gy[V.at(p, i1 - 1, j1 - 1)] = (e(i1, j1) - e(i1, j1 - 1)) / (d.hx * d.scale);
  }
}

// ---------------------------------------------------------------- ecs_A_vec
// The maps of the A-grid vector halo (equiang_cs/ecs_halo_vec_a_factory_mod.f90
// :108-170, init_transform_matrix): at position i and depth j of edge e
// (bottom, top, left, right), the neighbour's exchanged contravariant
// components (already turned to this panel's axes by the exchange) live at the
// neighbour's point (alpha_s, beta_s); rotated into this panel's frame, its
// basis vectors a1s, a2s are projected on this panel's extended dual basis
// b1t, b2t at the same point: TM = [a1s.b1t, a2s.b1t; a1s.b2t, a2s.b2t].
void build_ecs_tm(orcc_domain& d) {
  const int N = d.N;
  d.ecs_tm.assign((size_t)4 * kDepth * N * 4, 0.0);
  const int ab_shift[4] = {0, 0, 1, 1}, b_sign[4] = {1, -1, 1, -1};
  auto rot = [](int e, const double v[3], double o[3]) {
    switch (e) {
      case 0: o[0] = v[0]; o[1] = -v[2]; o[2] = v[1]; break;
      case 1: o[0] = v[0]; o[1] = v[2]; o[2] = -v[1]; break;
      case 2: o[0] = -v[2]; o[1] = v[1]; o[2] = v[0]; break;
      default: o[0] = v[2]; o[1] = v[1]; o[2] = -v[0]; break;
    }
  };
  auto dot = [](const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
  for (int e = 0; e < 4; ++e)
    for (int j = 1; j <= kDepth; ++j)
      for (int i = 1; i <= N; ++i) {
        const double al = -0.25 * PI + (i - 0.5) * d.hx;
        const double be = b_sign[e] * (0.25 * PI - (j - 0.5) * d.hx);
        const double as = ab_shift[e] ? be : al, bs = ab_shift[e] ? al : be;
        double v[3], a1s[3], a2s[3], r[3], b1t[3], b2t[3];
        a1_proto(as, bs, v); rot(e, v, a1s);
        a2_proto(as, bs, v); rot(e, v, a2s);
        r_proto(as, bs, v); rot(e, v, r);
        const double at = std::atan(r[0] / r[2]), bt = std::atan(r[1] / r[2]);
        b1_proto(at, bt, b1t);
        b2_proto(at, bt, b2t);
        double* T = &d.ecs_tm[(((size_t)e * kDepth + (j - 1)) * N + (i - 1)) * 4];
        T[0] = dot(a1s, b1t); T[1] = dot(a2s, b1t); T[2] = dot(a1s, b2t); T[3] = dot(a2s, b2t);
      }
}

// The ecs_A_vec halo of width hw (ecs_halo_vec_a_mod.f90:34-158): the 'full'
// vector exchange, the maps TM on the exchanged rows, then the ECS_O
// interpolation of each component.  Contravariant components at the centres.
void ecs_a_vec_panel(const orcc_domain& d, const double* u, const double* v, int p, int hw, double* Eu, double* Ev) {
  const Mesh& P = d.m[0];
  const int N = d.N;
  auto XV = [&](int c, int i1, int j1) -> double {
    if (i1 >= 1 && i1 <= N && j1 >= 1 && j1 <= N) return (c == 0 ? u : v)[P.at(p, i1 - 1, j1 - 1)];
    int e, dd, pos;
    if (j1 < 1) { e = 0; dd = 1 - j1; pos = i1; }
    else if (j1 > N) { e = 1; dd = j1 - N; pos = i1; }
    else if (i1 < 1) { e = 2; dd = 1 - i1; pos = j1; }
    else { e = 3; dd = i1 - N; pos = j1; }
    const double eu = ext(P, d.hau, u, v, p, i1 - 1, j1 - 1), ev = ext(P, d.hav, v, u, p, i1 - 1, j1 - 1);
    const double* T = &d.ecs_tm[(((size_t)e * kDepth + (dd - 1)) * N + (pos - 1)) * 4];
    return c == 0 ? T[0] * eu + T[1] * ev : T[2] * eu + T[3] * ev;
  };
  ecs_o_panel_x(d, [&](int i1, int j1) { return XV(0, i1, j1); }, hw, Eu);
  ecs_o_panel_x(d, [&](int i1, int j1) { return XV(1, i1, j1); }, hw, Ev);
}

// divergence_a2_ecs (divergence/div_a2_mod.f90:19-72 with div_factory_mod.f90:
// 90-112): the ecs_A_vec halo of width 1, then the central difference of J u^i
// over 2 J hx a, J on the extended grid lines beyond the edges.
void div_a2_ecs(const orcc_domain& d, const double* u, const double* v, double* out) {
  const Mesh& P = d.m[0];
  const int N = d.N, hw = 1, W = N + 2;
  auto Jx = [&](int i1, int j1) {
    const double al = -0.25 * PI + ((i1 - 1) + 0.5) * d.hx, be = -0.25 * PI + ((j1 - 1) + 0.5) * d.hx;
    const double ta = std::tan(al), tb = std::tan(be);
    const double sg = std::sqrt(1.0 + ta * ta + tb * tb);
    return (1.0 + ta * ta) * (1.0 + tb * tb) / (sg * sg * sg);
  };
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int p = 0; p < 6; ++p) {
    std::vector<double> Eu((size_t)W * W, 0.0), Ev((size_t)W * W, 0.0);
    ecs_a_vec_panel(d, u, v, p, hw, Eu.data(), Ev.data());
    auto eu = [&](int i1, int j1) { return Eu[(size_t)j1 * W + i1]; };  // 0-based extended = 1-based + 0
    auto ev = [&](int i1, int j1) { return Ev[(size_t)j1 * W + i1]; };
    for (int j1 = 1; j1 <= N; ++j1)
      for (int i1 = 1; i1 <= N; ++i1)
        out[P.at(p, i1 - 1, j1 - 1)] =
            (Jx(i1 + 1, j1) * eu(i1 + 1, j1) - Jx(i1 - 1, j1) * eu(i1 - 1, j1) + Jx(i1, j1 + 1) * ev(i1, j1 + 1) -
             Jx(i1, j1 - 1) * ev(i1, j1 - 1)) /
            (2.0 * Jx(i1, j1) * d.hx * d.scale);
  }
}

// ------------------------------------------------------------------ ECS_xy
// The ECS_xy halo of the corner (node) mesh, the Ah grid's points
// (equiang_cs/ecs_halo_xy_mod.f90:38-217 with ecs_halo_factory_mod.f90:198-
// 228, init_halo_xy_interp): n = N+1 nodes a side, the exchange places the
// neighbour's copy of the shared edge row in the first halo layer, so halo row
// r is interpolated from the neighbour's row r + 1 layers out.  Widths up to
// kXyRows (the exchange is kDepth deep).
constexpr int kXyRows = kDepth - 1;

void build_xy_weights(orcc_domain& d) {
  const int n = d.N + 1, ni = n + 2 * kXyRows;
  d.xy_w.assign((size_t)kXyRows * ni * 4, 0.0);
  d.xy_ind.assign((size_t)kXyRows * ni, 0);
  for (int r = 1; r <= kXyRows; ++r)
    for (int i = 1 - kXyRows; i <= n + kXyRows; ++i) {
      const double zb = 0.25 * PI + r * d.hx;
      double za = -0.25 * PI + (i - 1.0) * d.hx;
      za = std::atan(std::tan(za) / std::tan(zb));
      const int b = std::min(std::max(2, (int)std::floor((za + 0.25 * PI) / d.hx) + 1), n - 2);
      const double x = (za + 0.25 * PI) / d.hx - (b - 1.0);
      double* w = &d.xy_w[((size_t)(r - 1) * ni + (i - 1 + kXyRows)) * 4];
      w[0] = -x * (x - 1.0) * (x - 2.0) / 6.0;
      w[1] = (x + 1.0) * (x - 1.0) * (x - 2.0) / 2.0;
      w[2] = -(x + 1.0) * x * (x - 2.0) / 2.0;
      w[3] = (x + 1.0) * x * (x - 1.0) / 6.0;
      d.xy_ind[(size_t)(r - 1) * ni + (i - 1 + kXyRows)] = b;
    }
}

// One panel's ECS_xy halo of width hw on the extended tile E ((n+2hw)^2,
// row-major, the reference's 1-based (i, j) at row j+hw-1, column i+hw-1).
// The reference works in place; each step's inputs are restated here from
// the exchanged values X:
//  - the cube-corner nodes become the average of their three copies, and the
//    corner diagonal (1-r, 1-r) the average of the two strips' points r+1
//    layers out next to the corner, which also stand in for those points;
//  - the other edge nodes become the average with their duplicate;
//  - halo row r of an edge is the cubic interpolation (ecs_ext_halo_1e of the
//    xy module) of the neighbour's row r+1 layers out, whose end points are
//    the corner diagonals, at positions max(1-hw, 2-r) .. min(n+hw, n+r-1).
void ecs_xy_panel(const orcc_domain& d, const double* f, int p, int hw, double* E) {
  const Mesh& Q = d.m[3];
  const int n = d.N + 1, W = n + 2 * hw, ni = n + 2 * kXyRows;
  auto X = [&](int i1, int j1) { return ext(Q, d.hq, f, nullptr, p, i1 - 1, j1 - 1); };
  auto out = [&](int i1, int j1) -> double& { return E[(size_t)(j1 - 1 + hw) * W + (i1 - 1 + hw)]; };
  auto w = [&](int m, int i, int r) { return d.xy_w[((size_t)(r - 1) * ni + (i - 1 + kXyRows)) * 4 + (m + 1)]; };
  auto ind = [&](int i, int r) { return d.xy_ind[(size_t)(r - 1) * ni + (i - 1 + kXyRows)]; };
  for (int j = 1; j <= n; ++j)
    for (int i = 1; i <= n; ++i) out(i, j) = X(i, j);
  // corner diagonals of corners 1..4 (at (1,1), (n,1), (n,n), (1,n))
  std::vector<double> dg(4 * (size_t)(hw + 1), 0.0);
  auto D = [&](int c, int r) -> double& { return dg[(size_t)c * (hw + 1) + r]; };
  for (int r = 1; r <= hw; ++r) {
    D(0, r) = 0.5 * (X(-r, 1) + X(1, -r));
    D(1, r) = 0.5 * (X(n + r + 1, 1) + X(n, -r));
    D(2, r) = 0.5 * (X(n + r + 1, n) + X(n, n + r + 1));
    D(3, r) = 0.5 * (X(1, n + r + 1) + X(-r, n));
  }
  // the panel's edge nodes: corners from three copies, the rest from two
  out(1, 1) = (X(1, 1) + X(1, 0) + X(0, 1)) / 3.0;
  out(n, 1) = (X(n, 1) + X(n, 0) + X(n + 1, 1)) / 3.0;
  out(n, n) = (X(n, n) + X(n, n + 1) + X(n + 1, n)) / 3.0;
  out(1, n) = (X(1, n) + X(0, n) + X(1, n + 1)) / 3.0;
  for (int k = 2; k <= n - 1; ++k) {
    out(k, 1) = 0.5 * (X(k, 1) + X(k, 0));
    out(k, n) = 0.5 * (X(k, n) + X(k, n + 1));
    out(1, k) = 0.5 * (X(1, k) + X(0, k));
    out(n, k) = 0.5 * (X(n, k) + X(n + 1, k));
  }
  // halo rows: the source row with its corner-diagonal end points
  for (int r = 1; r <= hw; ++r) {
    const int lo = std::max(1 - hw, 2 - r), hi = std::min(n + hw, n + r - 1);
    auto S1 = [&](int k) { return k == 1 ? D(0, r) : k == n ? D(1, r) : X(k, -r); };         // bottom
    auto S2 = [&](int k) { return k == 1 ? D(3, r) : k == n ? D(2, r) : X(k, n + r + 1); };  // top
    auto S3 = [&](int k) { return k == 1 ? D(0, r) : k == n ? D(3, r) : X(-r, k); };         // left
    auto S4 = [&](int k) { return k == 1 ? D(1, r) : k == n ? D(2, r) : X(n + r + 1, k); };  // right
    for (int k = lo; k <= hi; ++k) {
      const int b = ind(k, r);
      auto itp = [&](auto S) {
        double s = w(-1, k, r) * S(b - 1);
        s = s + w(0, k, r) * S(b);
        s = s + w(1, k, r) * S(b + 1);
        s = s + w(2, k, r) * S(b + 2);
        return s;
      };
      out(k, 1 - r) = itp(S1);
      out(k, n + r) = itp(S2);
      out(1 - r, k) = itp(S3);
      out(n + r, k) = itp(S4);
    }
    out(1 - r, 1 - r) = D(0, r);
    out(n + r, 1 - r) = D(1, r);
    out(n + r, n + r) = D(2, r);
    out(1 - r, n + r) = D(3, r);
  }
}

// laplace_ch_halo2 / laplace_ch_halo4 (laplace/laplace_ch_halo_mod.f90:15-179
// with laplace_factory_mod.f90:110-126): on the node mesh with the ECS_xy
// halo (width 1 / 3), the divergence of the contravariant gradient at second
// / fourth order, then the Ah-type edge sync.  The metric is the ECS metric at
// the nodes and at the half-shifted points (mesh_y at (i+1/2, j), mesh_x at
// (i, j+1/2)), extended beyond the edges.
void laplace_ch(const orcc_domain& d, int order, const double* f, double* out) {
  const Mesh& Q = d.m[3];
  const int N = d.N, n = N + 1, hw = order == 2 ? 1 : 3, W = n + 2 * hw;
  const double hx = d.hx, a = d.scale;
  struct Mt { double J, qi1, qi2, qi3; };
  auto met = [&](double si, double sj) {  // 1-based node coordinates, may be fractional / outside
    const double al = -0.25 * PI + (si - 1.0) * hx, be = -0.25 * PI + (sj - 1.0) * hx;
    const double ta = std::tan(al), tb = std::tan(be);
    const double sg = std::sqrt(1.0 + ta * ta + tb * tb);
    Mt m;
    m.J = (1.0 + ta * ta) * (1.0 + tb * tb) / (sg * sg * sg);
    m.qi1 = sg * sg / (1.0 + ta * ta);
    m.qi2 = sg * sg * ta * tb / ((1.0 + ta * ta) * (1.0 + tb * tb));
    m.qi3 = sg * sg / (1.0 + tb * tb);
    return m;
  };
  std::vector<double> raw(Q.size());
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (int p = 0; p < 6; ++p) {
    std::vector<double> E((size_t)W * W, 0.0);
    ecs_xy_panel(d, f, p, hw, E.data());
    auto F = [&](int i1, int j1) { return E[(size_t)(j1 - 1 + hw) * W + (i1 - 1 + hw)]; };
    auto xy = [&](int i1, int j1) { return met(i1, j1); };
    auto my = [&](int i1, int j1) { return met(i1 + 0.5, j1); };  // mesh_y: (i+1/2, j)
    auto mx = [&](int i1, int j1) { return met(i1, j1 + 0.5); };  // mesh_x: (i, j+1/2)
    for (int j = 1; j <= n; ++j)
      for (int i = 1; i <= n; ++i) {
        double v;
        if (order == 2) {
          auto gx = [&](int ii, int jj) { return (F(ii + 1, jj) - F(ii, jj)) / (hx * a); };
          auto gy = [&](int ii, int jj) { return (F(ii, jj + 1) - F(ii, jj)) / (hx * a); };
          auto gxt = [&](int ii, int jj) {
            const double gh0 = 0.5 * (gy(ii, jj - 1) + gy(ii, jj)) * xy(ii, jj).qi2 * xy(ii, jj).J;
            const double gh1 = 0.5 * (gy(ii + 1, jj - 1) + gy(ii + 1, jj)) * xy(ii + 1, jj).qi2 * xy(ii + 1, jj).J;
            return my(ii, jj).qi1 * gx(ii, jj) + 0.5 * (gh0 + gh1) / my(ii, jj).J;
          };
          // the reference's own index pairing in gyt's second term: Qi12 at
          // (i+1, j) times J at (i, j+1) (laplace_ch_halo_mod.f90:87).  It
          // makes the order-2 operator converge at first order; with both at
          // (i, j+1) it would be second order.  Kept, for parity.
          auto gyt = [&](int ii, int jj) {
            const double gh0 = 0.5 * (gx(ii - 1, jj) + gx(ii, jj)) * xy(ii, jj).qi2 * xy(ii, jj).J;
            const double gh1 = 0.5 * (gx(ii - 1, jj + 1) + gx(ii, jj + 1)) * xy(ii + 1, jj).qi2 * xy(ii, jj + 1).J;
            return mx(ii, jj).qi3 * gy(ii, jj) + 0.5 * (gh0 + gh1) / mx(ii, jj).J;
          };
          v = (my(i, j).J * gxt(i, j) - my(i - 1, j).J * gxt(i - 1, j) + mx(i, j).J * gyt(i, j) -
               mx(i, j - 1).J * gyt(i, j - 1)) /
              (xy(i, j).J * hx * a);
        } else {
          auto gx = [&](int ii, int jj) {
            return (-F(ii + 2, jj) + 27.0 * F(ii + 1, jj) - 27.0 * F(ii, jj) + F(ii - 1, jj)) / (24.0 * hx * a);
          };
          auto gy = [&](int ii, int jj) {
            return (-F(ii, jj + 2) + 27.0 * F(ii, jj + 1) - 27.0 * F(ii, jj) + F(ii, jj - 1)) / (24.0 * hx * a);
          };
          auto gxh = [&](int ii, int jj) {
            return (-gx(ii - 2, jj) + 9.0 * gx(ii - 1, jj) + 9.0 * gx(ii, jj) - gx(ii + 1, jj)) / 16.0 * xy(ii, jj).qi2 *
                   xy(ii, jj).J;
          };
          auto gyh = [&](int ii, int jj) {
            return (-gy(ii, jj - 2) + 9.0 * gy(ii, jj - 1) + 9.0 * gy(ii, jj) - gy(ii, jj + 1)) / 16.0 * xy(ii, jj).qi2 *
                   xy(ii, jj).J;
          };
          auto gxt = [&](int ii, int jj) {
            return my(ii, jj).qi1 * gx(ii, jj) +
                   (-gyh(ii + 2, jj) + 9.0 * gyh(ii + 1, jj) + 9.0 * gyh(ii, jj) - gyh(ii - 1, jj)) / (16.0 * my(ii, jj).J);
          };
          auto gyt = [&](int ii, int jj) {
            return mx(ii, jj).qi3 * gy(ii, jj) +
                   (-gxh(ii, jj + 2) + 9.0 * gxh(ii, jj + 1) + 9.0 * gxh(ii, jj) - gxh(ii, jj - 1)) / (16.0 * mx(ii, jj).J);
          };
          const double dx = (-my(i + 1, j).J * gxt(i + 1, j) + 27.0 * my(i, j).J * gxt(i, j) -
                             27.0 * my(i - 1, j).J * gxt(i - 1, j) + my(i - 2, j).J * gxt(i - 2, j)) /
                            24.0;
          const double dy = (-mx(i, j + 1).J * gyt(i, j + 1) + 27.0 * mx(i, j).J * gyt(i, j) -
                             27.0 * mx(i, j - 1).J * gyt(i, j - 1) + mx(i, j - 2).J * gyt(i, j - 2)) /
                            24.0;
          v = (dx / hx + dy / hx) / (xy(i, j).J * a);
        }
        raw[Q.at(p, i - 1, j - 1)] = v;
      }
  }
  std::copy(raw.begin(), raw.end(), out);
  sync_q(d, out);
}

// operator_swm_t%apply, vector-invariant branch
// (models/shallow_water/operator/operator_swm_mod.f90:61-113).
void apply(const orcc_domain& d, const double* hs, const double* h, const double* u, const double* v, double* th,
           double* tu, double* tv) {
  const Mesh &P = d.m[0], &U = d.m[1], &V = d.m[2], &Q = d.m[3];
  std::vector<double> ut(U.size()), vt(V.size()), hu(U.size()), hv(V.size()), ke(P.size());
  std::vector<double> gx(U.size()), gy(V.size()), cu(Q.size()), cor_u(U.size()), cor_v(V.size()), dv(P.size());
  co2contra(d, d.ops, u, v, ut.data(), vt.data());
  massflux(d, h, ut.data(), vt.data(), hu.data(), hv.data());
  kinetic_energy(d, u, v, ut.data(), vt.data(), ke.data());
  for (int k = 0; k < P.size(); ++k) ke[k] = ke[k] + d.grav * h[k] + d.grav * (hs ? hs[k] : 0.0);
  grad(d, d.ops, ke.data(), gx.data(), gy.data());
  curl(d, d.ops, u, v, cu.data());
  coriolis(d, hu.data(), hv.data(), h, cu.data(), cor_u.data(), cor_v.data());
  for (int k = 0; k < U.size(); ++k) tu[k] = -1.0 * gx[k] + 1.0 * cor_u[k];
  for (int k = 0; k < V.size(); ++k) tv[k] = -1.0 * gy[k] + 1.0 * cor_v[k];
  div(d, d.ops, hu.data(), hv.data(), dv.data());
  for (int k = 0; k < P.size(); ++k) th[k] = -1.0 * dv[k];
}

// rk4_t%step (time_schemes/rk4_mod.f90:20-42) on the staggered state.
void rk4(const orcc_domain& d, const double* hs, double* h, double* u, double* v, double dt, int nsteps) {
  const int n[3] = {d.m[0].size(), d.m[1].size(), d.m[2].size()};
  double* F0[3] = {h, u, v};
  std::vector<double> k[4][3], y[3];
  for (int c = 0; c < 3; ++c) {
    y[c].assign(n[c], 0.0);
    for (int s = 0; s < 4; ++s) k[s][c].assign(n[c], 0.0);
  }
  auto A = [&](int s, double* yh, double* yu, double* yv) {
    apply(d, hs, yh, yu, yv, k[s][0].data(), k[s][1].data(), k[s][2].data());
  };
  auto assign = [&](double s2, int s) {
    for (int c = 0; c < 3; ++c)
      for (int m = 0; m < n[c]; ++m) y[c][m] = 1.0 * F0[c][m] + s2 * k[s][c][m];
  };
  for (int st = 0; st < nsteps; ++st) {
    A(0, h, u, v);
    assign(0.5 * dt, 0);
    A(1, y[0].data(), y[1].data(), y[2].data());
    assign(0.5 * dt, 1);
    A(2, y[0].data(), y[1].data(), y[2].data());
    assign(dt, 2);
    A(3, y[0].data(), y[1].data(), y[2].data());
    const double c6 = dt / 6.0, c3 = dt / 3.0;
    for (int c = 0; c < 3; ++c)
      for (int m = 0; m < n[c]; ++m) {
        double x = F0[c][m];
        x = x + c6 * k[0][c][m] + c3 * k[1][c][m];
        x = x + c3 * k[2][c][m] + c6 * k[3][c][m];
        F0[c][m] = x;
      }
  }
}

// explicit_Eul1_t%step (explicit_Eul1_mod.f90:20-30) of operator_swm_diff_t
// (operator_swm_diff_mod.f90:25-46): v0 = v0 + dt D(v0).
void diffusion_step(const orcc_domain& d, int parts, double cuv, double ch, double* h, double* u, double* v,
                    double dt) {
  const int n[3] = {d.m[0].size(), d.m[1].size(), d.m[2].size()};
  std::vector<double> th(n[0]), tu(n[1]), tv(n[2]);
  hordiff_uv(d, parts, cuv, u, v, tu.data(), tv.data());
  hordiff_h(d, ch, h, th.data());
  for (int k = 0; k < n[0]; ++k) h[k] = h[k] + dt * th[k];
  for (int k = 0; k < n[1]; ++k) u[k] = u[k] + dt * tu[k];
  for (int k = 0; k < n[2]; ++k) v[k] = v[k] + dt * tv[k];
}

// SBP_C42 / SBP_C21 quadrature (quadrature_factory_mod.f90:90-160 and
// sbp_quadrature_mod.f90:21-40): centre or interface edge weights per
// direction according to the mesh's point type.
double mass(const orcc_domain& d, int mesh, const double* f) {
  const Mesh& M = d.m[mesh];
  auto weights = [&](int n, bool iface) {
    const std::vector<double>& e = iface ? d.Ai : d.Ac;
    std::vector<double> w(n, 1.0);
    const int ne = (int)e.size();
    for (int k = 0; k < std::min(ne, n); ++k) w[k] = e[k];
    for (int k = std::max(n - ne, 0); k < n; ++k) w[k] = e[n - 1 - k];
    return w;
  };
  const std::vector<double> ax = weights(M.nx, mesh == 1 || mesh == 3);
  const std::vector<double> ay = weights(M.ny, mesh == 2 || mesh == 3);
  double tot = 0.0;
  for (int p = 0; p < 6; ++p) {
    double acc = 0.0;
    for (int j = 0; j < M.ny; ++j)
      for (int i = 0; i < M.nx; ++i) {
        const int id = M.at(p, i, j);
        acc = acc + f[id] * M.J[id] * d.hx * d.hx * ax[i] * ay[j];
      }
    tot = tot + acc;
  }
  return tot;
}

// l2norm (vec_math_mod.f90:50-90), summed over the given number of levels
// before the square root.
double l2sq(const Mesh& M, double hx, const double* f) {
  double tot = 0.0;
  for (int p = 0; p < 6; ++p) {
    double acc = 0.0;
    for (int j = 0; j < M.ny; ++j)
      for (int i = 0; i < M.nx; ++i) {
        const int id = M.at(p, i, j);
        acc = acc + f[id] * f[id] * M.J[id] * hx * hx;
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

// set_vector_test_field (test_fields_mod.f90): u on the u mesh from its
// basis vector 1, v on the v mesh from its basis vector 2.
template <class Gen>
void set_vector(const orcc_domain& d, Gen gen, bool contravariant, std::vector<double>& u, std::vector<double>& v) {
  const Mesh &U = d.m[1], &V = d.m[2];
  u.assign(U.size(), 0.0);
  v.assign(V.size(), 0.0);
  for (int k = 0; k < U.size(); ++k) {
    double w[3];
    gen(U.rx[k], U.ry[k], U.rz[k], w);
    const double* e = contravariant ? &U.b1[3 * k] : &U.a1[3 * k];
    u[k] = w[0] * e[0] + w[1] * e[1] + w[2] * e[2];
  }
  for (int k = 0; k < V.size(); ++k) {
    double w[3];
    gen(V.rx[k], V.ry[k], V.rz[k], w);
    const double* e = contravariant ? &V.b2[3 * k] : &V.a2[3 * k];
    v[k] = w[0] * e[0] + w[1] * e[1] + w[2] * e[2];
  }
}

orcc_domain* create(int N, int order, double radius, double grav, double omega, const double axis[3]) {
  if (N < 12 || (order != 21 && order != 42)) return nullptr;
  orcc_domain* d = new orcc_domain;
  d->N = N; d->order = order;
  d->scale = radius; d->grav = grav; d->omega = omega;
  const double an = std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
  for (int c = 0; c < 3; ++c) d->axis[c] = axis[c] / an;
  d->hx = (0.25 * PI - (-0.25 * PI)) / (double)N;
  build_mesh(*d, d->m[0], N, N, 0.5, 0.5);
  build_mesh(*d, d->m[1], N + 1, N, 0.0, 0.5);
  build_mesh(*d, d->m[2], N, N + 1, 0.5, 0.0);
  build_mesh(*d, d->m[3], N + 1, N + 1, 0.0, 0.0);
  d->ho = build_halo(d->m[0], d->m[0], 0);
  d->hu = build_halo(d->m[1], d->m[2], 1);
  d->hv = build_halo(d->m[2], d->m[1], 2);
  d->hq = build_halo(d->m[3], d->m[3], 0);
  if (!build_ecs_weights(*d)) {
    delete d;
    return nullptr;
  }
  d->hau = build_halo(d->m[0], d->m[0], 1);
  d->hav = build_halo(d->m[0], d->m[0], 2);
  build_ecs_tm(*d);
  build_xy_weights(*d);
  d->ops21.order = 21;
  d->ops21.Wc2i = make_stag(W21_C2I); d->ops21.Wi2c = make_stag(W21_I2C);
  d->ops21.Dc2i = make_stag(D21_C2I); d->ops21.Di2c = make_stag(D21_I2C);
  if (order == 42) {
    d->ops.order = 42;
    d->ops.Wc2i = make_stag(W42_C2I); d->ops.Wi2c = make_stag(W42_I2C);
    d->ops.Dc2i = make_stag(D42_C2I); d->ops.Di2c = make_stag(D42_I2C);
    d->Ac = {13.0 / 12.0, 7.0 / 8.0, 25.0 / 24.0, 1.0};
    d->Ai = {7.0 / 18.0, 9.0 / 8.0, 1.0, 71.0 / 72.0, 1.0};
  } else {
    d->ops = d->ops21;
    d->Ac = {1.0, 1.0};
    d->Ai = {0.5, 1.0};
  }
  return d;
}

}  // namespace

extern "C" {

orcc_domain* orcc_create(int N, int sbp_order, double radius, double grav, double omega, const double axis[3]) {
  return create(N, sbp_order, radius, grav, omega, axis);
}
void orcc_destroy(orcc_domain* d) { delete d; }
int orcc_size(const orcc_domain* d, int mesh) { return (mesh < 0 || mesh > 3) ? -1 : d->m[mesh].size(); }

void orcc_points(const orcc_domain* d, int mesh, double* x, double* y, double* z) {
  const Mesh& M = d->m[mesh];
  for (int k = 0; k < M.size(); ++k) { x[k] = M.rx[k]; y[k] = M.ry[k]; z[k] = M.rz[k]; }
}
void orcc_metric(const orcc_domain* d, int mesh, double* J, double* Qi1, double* Qi2, double* Qi3, double* f) {
  const Mesh& M = d->m[mesh];
  for (int k = 0; k < M.size(); ++k) {
    J[k] = M.J[k]; Qi1[k] = M.Qi1[k]; Qi2[k] = M.Qi2[k]; Qi3[k] = M.Qi3[k]; f[k] = M.f[k];
  }
}
void orcc_bases(const orcc_domain* d, int mesh, double* a1, double* a2, double* b1, double* b2) {
  const Mesh& M = d->m[mesh];
  for (size_t k = 0; k < 3 * (size_t)M.size(); ++k) { a1[k] = M.a1[k]; a2[k] = M.a2[k]; b1[k] = M.b1[k]; b2[k] = M.b2[k]; }
}

void orcc_co2contra(const orcc_domain* d, const double* u, const double* v, double* ut, double* vt) {
  co2contra(*d, d->ops, u, v, ut, vt);
}
void orcc_massflux(const orcc_domain* d, const double* h, const double* ut, const double* vt, double* hu, double* hv) {
  massflux(*d, h, ut, vt, hu, hv);
}
void orcc_ke(const orcc_domain* d, const double* u, const double* v, const double* ut, const double* vt, double* ke) {
  kinetic_energy(*d, u, v, ut, vt, ke);
}
void orcc_grad(const orcc_domain* d, const double* f, double* gx, double* gy) { grad(*d, d->ops, f, gx, gy); }
void orcc_div(const orcc_domain* d, const double* hu, const double* hv, double* out) { div(*d, d->ops, hu, hv, out); }
void orcc_curl(const orcc_domain* d, const double* u, const double* v, double* out) { curl(*d, d->ops, u, v, out); }
void orcc_coriolis(const orcc_domain* d, const double* hu, const double* hv, const double* h, const double* cu,
                   double* cor_u, double* cor_v) {
  coriolis(*d, hu, hv, h, cu, cor_u, cor_v);
}
void orcc_apply(const orcc_domain* d, const double* hs, const double* h, const double* u, const double* v,
                double* th, double* tu, double* tv) {
  apply(*d, hs, h, u, v, th, tu, tv);
}
void orcc_rk4(const orcc_domain* d, const double* hs, double* h, double* u, double* v, double dt, int nsteps) {
  rk4(*d, hs, h, u, v, dt, nsteps);
}
void orcc_grad_perp(const orcc_domain* d, const double* w, double* gu, double* gv) {
  grad_perp(*d, d->ops, w, gu, gv);
}
void orcc_contra2co(const orcc_domain* d, const double* ut, const double* vt, double* u, double* v) {
  contra2co(*d, d->ops, ut, vt, u, v);
}
void orcc_hordiff(const orcc_domain* d, int parts, double uv_coeff, double h_coeff, const double* h, const double* u,
                  const double* v, double* th, double* tu, double* tv) {
  hordiff_uv(*d, parts, uv_coeff, u, v, tu, tv);
  hordiff_h(*d, h_coeff, h, th);
}
void orcc_model_step(const orcc_domain* d, const double* hs, double* h, double* u, double* v, double dt, int nsteps,
                     int parts, double uv_coeff, double h_coeff) {
  for (int s = 0; s < nsteps; ++s) {
    rk4(*d, hs, h, u, v, dt, 1);
    diffusion_step(*d, parts, uv_coeff, h_coeff, h, u, v, dt);
  }
}
int orcc_ecs_o_halo(const orcc_domain* d, const double* f, int halo_width, double* ext) {
  if (halo_width < 1 || halo_width > 2) return -1;
  const size_t W = (size_t)d->N + 2 * halo_width;
  for (int p = 0; p < 6; ++p) ecs_o_panel(*d, f, p, halo_width, ext + p * W * W);
  return 0;
}
void orcc_grad_a2_ecs(const orcc_domain* d, const double* f, double* gx, double* gy) { grad_a2_ecs(*d, f, gx, gy); }
int orcc_ecs_a_vec_halo(const orcc_domain* d, const double* u, const double* v, int halo_width, double* eu,
                        double* ev) {
  if (halo_width < 1 || halo_width > 2) return -1;
  const size_t W = (size_t)d->N + 2 * halo_width;
  for (int p = 0; p < 6; ++p) ecs_a_vec_panel(*d, u, v, p, halo_width, eu + p * W * W, ev + p * W * W);
  return 0;
}
void orcc_div_a2_ecs(const orcc_domain* d, const double* u, const double* v, double* out) { div_a2_ecs(*d, u, v, out); }
void orcc_grad_c2_ecs(const orcc_domain* d, const double* f, double* gx, double* gy) { grad_c2_ecs(*d, f, gx, gy); }
int orcc_ecs_xy_halo(const orcc_domain* d, const double* f, int halo_width, double* ext) {
  if (halo_width < 1 || halo_width > kXyRows) return -1;
  const size_t W = (size_t)d->N + 1 + 2 * halo_width;
  for (int p = 0; p < 6; ++p) ecs_xy_panel(*d, f, p, halo_width, ext + p * W * W);
  return 0;
}
int orcc_laplace_ch(const orcc_domain* d, int order, const double* f, double* out) {
  if (order != 2 && order != 4) return -1;
  laplace_ch(*d, order, f, out);
  return 0;
}
double orcc_mass(const orcc_domain* d, int mesh, const double* f) { return mass(*d, mesh, f); }
double orcc_l2norm(const orcc_domain* d, int mesh, const double* f) {
  return std::sqrt(l2sq(d->m[mesh], d->hx, f));
}

// Analytic fields of the known-answer tests on the C meshes (as
// orc_vector_test_field / orc_scalar_test_field on the Ah grid): vector kinds
// 0 solid rotation (axis cycles with level), 1 cross-polar flow, 2 gradient
// of x/y/z (cycles), 3 curl-free VSH; u on the u mesh, v on the v mesh.
// Scalar kinds 10 x/y/z (cycles), 11 cross-polar divergence, 12 cross-polar
// vorticity, on the given mesh.
int orcc_vector_test_field(const orcc_domain* d, int kind, int level, int contravariant, double* u, double* v) {
  std::vector<double> a, b;
  const bool ct = contravariant != 0;
  switch (kind) {
    case 0: set_vector(*d, [level](double x, double y, double z, double w[3]) { field_solid_rotation(level, x, y, z, w); }, ct, a, b); break;
    case 1: set_vector(*d, field_cross_polar, ct, a, b); break;
    case 2: set_vector(*d, [level](double x, double y, double z, double w[3]) { field_xyz_grad(level, x, y, z, w); }, ct, a, b); break;
    case 3: set_vector(*d, field_vsh_curl_free_10, ct, a, b); break;
    default: return -1;
  }
  std::copy(a.begin(), a.end(), u);
  std::copy(b.begin(), b.end(), v);
  return 0;
}

int orcc_scalar_test_field(const orcc_domain* d, int kind, int level, int mesh, double* f) {
  if (mesh < 0 || mesh > 3) return -1;
  const Mesh& M = d->m[mesh];
  for (int k = 0; k < M.size(); ++k) {
    const double x = M.rx[k], y = M.ry[k], z = M.rz[k];
    if (kind == 10) f[k] = field_xyz(level, x, y, z);
    else if (kind == 11) f[k] = field_cross_polar_div(x, y, z);
    else if (kind == 12) f[k] = field_cross_polar_zeta(x, y, z);
    else return -1;
  }
  return 0;
}

// The reference's known-answer tests on the C grid at N, nz = 3 identical
// levels apart from the solid-rotation axis (test_diff_ops/
// test_diffops_mod.f90): kind 0 test_div (71-125), 1 test_grad (127-178),
// 2 test_curl (466-522), 3 test_coriolis_vec_inv (723-789), 4 test_KE
// (523-594), 5 test_co2contra (231-278).  Unit sphere, Omega = 1 about z.
int orcc_golden(int kind, int N, int order, double* out) {
  const double ax[3] = {0, 0, 1};
  orcc_domain* d = create(N, order, 1.0, 9.80616, 1.0, ax);
  if (!d) return -1;
  const Mesh &P = d->m[0], &U = d->m[1], &V = d->m[2], &Q = d->m[3];
  std::vector<double> u, v, ut, vt, a(std::max(P.size(), Q.size())), b(V.size()), c(U.size());
  std::vector<double> all, allx, ally;
  double l2 = 0.0, l2x = 0.0, l2y = 0.0;
  int rc = 0;
  switch (kind) {
    case 0: {  // div of the contravariant solid rotation (per-level axis) and of the cross-polar flow
      for (int lev = 0; lev < 3; ++lev) {
        set_vector(*d, [lev](double x, double y, double z, double w[3]) { field_solid_rotation(lev, x, y, z, w); },
                   true, u, v);
        div(*d, d->ops, u.data(), v.data(), a.data());
        std::vector<double> e(a.begin(), a.begin() + P.size());
        for (double& x : e) x = d->scale * x;
        all.insert(all.end(), e.begin(), e.end());
        l2 += l2sq(P, d->hx, e.data());
      }
      out[0] = maxabs(all); out[1] = std::sqrt(l2);
      all.clear(); l2 = 0.0;
      for (int lev = 0; lev < 3; ++lev) {
        set_vector(*d, field_cross_polar, true, u, v);
        div(*d, d->ops, u.data(), v.data(), a.data());
        std::vector<double> e(P.size());
        for (int k = 0; k < P.size(); ++k) e[k] = d->scale * a[k] - 1.0 * field_cross_polar_div(P.rx[k], P.ry[k], P.rz[k]);
        all.insert(all.end(), e.begin(), e.end());
        l2 += l2sq(P, d->hx, e.data());
      }
      out[2] = maxabs(all); out[3] = std::sqrt(l2);
      break;
    }
    case 1: {  // covariant gradient of x, y, z (per level)
      std::vector<double> f(P.size()), tx, ty;
      for (int lev = 0; lev < 3; ++lev) {
        for (int k = 0; k < P.size(); ++k) f[k] = field_xyz(lev, P.rx[k], P.ry[k], P.rz[k]);
        set_vector(*d, [lev](double x, double y, double z, double w[3]) { field_xyz_grad(lev, x, y, z, w); }, false,
                   tx, ty);
        grad(*d, d->ops, f.data(), c.data(), b.data());
        for (int k = 0; k < U.size(); ++k) c[k] = d->scale * c[k] - 1.0 * tx[k];
        for (int k = 0; k < V.size(); ++k) b[k] = d->scale * b[k] - 1.0 * ty[k];
        allx.insert(allx.end(), c.begin(), c.end());
        ally.insert(ally.end(), b.begin(), b.end());
        l2x += l2sq(U, d->hx, c.data());
        l2y += l2sq(V, d->hx, b.data());
      }
      out[0] = maxabs(allx) + maxabs(ally);
      out[1] = std::sqrt(l2x) + std::sqrt(l2y);
      break;
    }
    case 2: {  // curl of the curl-free VSH field and of the cross-polar flow
      for (int fld = 0; fld < 2; ++fld) {
        all.clear(); l2 = 0.0;
        for (int lev = 0; lev < 3; ++lev) {
          if (fld == 0) set_vector(*d, field_vsh_curl_free_10, false, u, v);
          else set_vector(*d, field_cross_polar, false, u, v);
          curl(*d, d->ops, u.data(), v.data(), a.data());
          std::vector<double> e(Q.size());
          for (int k = 0; k < Q.size(); ++k) {
            e[k] = d->scale * a[k];
            if (fld == 1) e[k] = e[k] - 1.0 * field_cross_polar_zeta(Q.rx[k], Q.ry[k], Q.rz[k]);
          }
          all.insert(all.end(), e.begin(), e.end());
          l2 += l2sq(Q, d->hx, e.data());
        }
        out[2 * fld] = maxabs(all); out[2 * fld + 1] = std::sqrt(l2);
      }
      break;
    }
    case 3: {  // Coriolis force of the contravariant VSH field, h = 1, curl = 0
      std::vector<double> h(P.size(), 1.0), cz(Q.size(), 0.0), tu(U.size()), tv(V.size());
      for (int lev = 0; lev < 3; ++lev) {
        set_vector(*d, field_vsh_curl_free_10, true, u, v);
        coriolis(*d, u.data(), v.data(), h.data(), cz.data(), c.data(), b.data());
        // exact force 2 sin(phi) (v_phi, -v_lam) (coriolis_force_field_generator_t)
        auto force = [](double x, double y, double z, double w[3]) {
          double V3[3];
          field_vsh_curl_free_10(x, y, z, V3);
          const double r = std::sqrt(x * x + y * y + z * z);
          const double lam = std::atan2(y, x), phi = std::asin(z / r);
          const double el[3] = {-std::sin(lam), std::cos(lam), 0.0};
          const double ep[3] = {-std::sin(phi) * std::cos(lam), -std::sin(phi) * std::sin(lam), std::cos(phi)};
          const double vl = V3[0] * el[0] + V3[1] * el[1] + V3[2] * el[2];
          const double vp = V3[0] * ep[0] + V3[1] * ep[1] + V3[2] * ep[2];
          const double pc = 2.0 * std::sin(phi);
          const double fl = pc * vp, fp = -pc * vl;
          for (int q = 0; q < 3; ++q) w[q] = fl * el[q] + fp * ep[q];
        };
        set_vector(*d, force, false, tu, tv);
        for (int k = 0; k < U.size(); ++k) c[k] = c[k] + (-1.0) * tu[k];
        for (int k = 0; k < V.size(); ++k) b[k] = b[k] + (-1.0) * tv[k];
        allx.insert(allx.end(), c.begin(), c.end());
        ally.insert(ally.end(), b.begin(), b.end());
        l2x += l2sq(U, d->hx, c.data());
        l2y += l2sq(V, d->hx, b.data());
      }
      out[0] = maxabs(allx) + maxabs(ally);
      out[1] = std::sqrt(l2x) + std::sqrt(l2y);
      break;
    }
    case 4: {  // kinetic energy against |V|^2/2 at the centres
      for (int fld = 0; fld < 2; ++fld) {
        all.clear(); l2 = 0.0;
        for (int lev = 0; lev < 3; ++lev) {
          if (fld == 0) {
            set_vector(*d, field_vsh_curl_free_10, false, u, v);
            set_vector(*d, field_vsh_curl_free_10, true, ut, vt);
          } else {
            set_vector(*d, field_cross_polar, false, u, v);
            set_vector(*d, field_cross_polar, true, ut, vt);
          }
          kinetic_energy(*d, u.data(), v.data(), ut.data(), vt.data(), a.data());
          std::vector<double> e(P.size());
          for (int k = 0; k < P.size(); ++k) {
            double W[3];
            if (fld == 0) field_vsh_curl_free_10(P.rx[k], P.ry[k], P.rz[k], W);
            else field_cross_polar(P.rx[k], P.ry[k], P.rz[k], W);
            e[k] = 1.0 * a[k] + (-1.0) * (0.5 * (W[0] * W[0] + W[1] * W[1] + W[2] * W[2]));
          }
          all.insert(all.end(), e.begin(), e.end());
          l2 += l2sq(P, d->hx, e.data());
        }
        out[2 * fld] = maxabs(all); out[2 * fld + 1] = std::sqrt(l2);
      }
      break;
    }
    case 5: {  // co2contra of the covariant cross-polar flow
      for (int lev = 0; lev < 3; ++lev) {
        set_vector(*d, field_cross_polar, false, u, v);
        set_vector(*d, field_cross_polar, true, ut, vt);
        co2contra(*d, d->ops, u.data(), v.data(), c.data(), b.data());
        for (int k = 0; k < U.size(); ++k) c[k] = c[k] + (-1.0) * ut[k];
        for (int k = 0; k < V.size(); ++k) b[k] = b[k] + (-1.0) * vt[k];
        allx.insert(allx.end(), c.begin(), c.end());
        ally.insert(ally.end(), b.begin(), b.end());
        l2x += l2sq(U, d->hx, c.data());
        l2y += l2sq(V, d->hx, b.data());
      }
      out[0] = maxabs(allx) + maxabs(ally);
      out[1] = std::sqrt(l2x) + std::sqrt(l2y);
      break;
    }
    case 6: {  // transform2co of the contravariant cross-polar flow
      for (int lev = 0; lev < 3; ++lev) {
        set_vector(*d, field_cross_polar, true, ut, vt);
        set_vector(*d, field_cross_polar, false, u, v);
        contra2co(*d, d->ops, ut.data(), vt.data(), c.data(), b.data());
        for (int k = 0; k < U.size(); ++k) c[k] = c[k] + (-1.0) * u[k];
        for (int k = 0; k < V.size(); ++k) b[k] = b[k] + (-1.0) * v[k];
        allx.insert(allx.end(), c.begin(), c.end());
        ally.insert(ally.end(), b.begin(), b.end());
        l2x += l2sq(U, d->hx, c.data());
        l2y += l2sq(V, d->hx, b.data());
      }
      out[0] = maxabs(allx) + maxabs(ally);
      out[1] = std::sqrt(l2x) + std::sqrt(l2y);
      break;
    }
    case 9: {  // gradient_c2_ecs of x, y, z onto the faces
      std::vector<double> f(P.size()), tx, ty;
      for (int lev = 0; lev < 3; ++lev) {
        for (int k = 0; k < P.size(); ++k) f[k] = field_xyz(lev, P.rx[k], P.ry[k], P.rz[k]);
        set_vector(*d, [lev](double x, double y, double z, double w[3]) { field_xyz_grad(lev, x, y, z, w); }, false,
                   tx, ty);
        grad_c2_ecs(*d, f.data(), c.data(), b.data());
        for (int k = 0; k < U.size(); ++k) c[k] = d->scale * c[k] - 1.0 * tx[k];
        for (int k = 0; k < V.size(); ++k) b[k] = d->scale * b[k] - 1.0 * ty[k];
        allx.insert(allx.end(), c.begin(), c.end());
        ally.insert(ally.end(), b.begin(), b.end());
        l2x += l2sq(U, d->hx, c.data());
        l2y += l2sq(V, d->hx, b.data());
      }
      out[0] = maxabs(allx) + maxabs(ally);
      out[1] = std::sqrt(l2x) + std::sqrt(l2y);
      break;
    }
    case 8: {  // divergence_a2_ecs of the contravariant solid rotation and cross-polar flow at the centres
      std::vector<double> ua(P.size()), va(P.size()), dv(P.size());
      auto setp = [&](auto gen) {
        for (int k = 0; k < P.size(); ++k) {
          double W3[3];
          gen(P.rx[k], P.ry[k], P.rz[k], W3);
          const double* b1 = &P.b1[3 * k];
          const double* b2 = &P.b2[3 * k];
          ua[k] = W3[0] * b1[0] + W3[1] * b1[1] + W3[2] * b1[2];
          va[k] = W3[0] * b2[0] + W3[1] * b2[1] + W3[2] * b2[2];
        }
      };
      for (int fld = 0; fld < 2; ++fld) {
        all.clear(); l2 = 0.0;
        for (int lev = 0; lev < 3; ++lev) {
          if (fld == 0) setp([lev](double x, double y, double z, double w[3]) { field_solid_rotation(lev, x, y, z, w); });
          else setp(field_cross_polar);
          div_a2_ecs(*d, ua.data(), va.data(), dv.data());
          std::vector<double> e(P.size());
          for (int k = 0; k < P.size(); ++k) {
            e[k] = d->scale * dv[k];
            if (fld == 1) e[k] = e[k] - 1.0 * field_cross_polar_div(P.rx[k], P.ry[k], P.rz[k]);
          }
          all.insert(all.end(), e.begin(), e.end());
          l2 += l2sq(P, d->hx, e.data());
        }
        out[2 * fld] = maxabs(all); out[2 * fld + 1] = std::sqrt(l2);
      }
      break;
    }
    case 7: {  // gradient_a2_ecs of x, y, z on the cell centres (the A grid's points)
      std::vector<double> f(P.size()), tx(P.size()), ty(P.size()), gx(P.size()), gy(P.size());
      for (int lev = 0; lev < 3; ++lev) {
        for (int k = 0; k < P.size(); ++k) {
          f[k] = field_xyz(lev, P.rx[k], P.ry[k], P.rz[k]);
          double W3[3];
          field_xyz_grad(lev, P.rx[k], P.ry[k], P.rz[k], W3);
          const double* a1 = &P.a1[3 * k];
          const double* a2 = &P.a2[3 * k];
          tx[k] = W3[0] * a1[0] + W3[1] * a1[1] + W3[2] * a1[2];
          ty[k] = W3[0] * a2[0] + W3[1] * a2[1] + W3[2] * a2[2];
        }
        grad_a2_ecs(*d, f.data(), gx.data(), gy.data());
        for (int k = 0; k < P.size(); ++k) {
          gx[k] = d->scale * gx[k] - 1.0 * tx[k];
          gy[k] = d->scale * gy[k] - 1.0 * ty[k];
        }
        allx.insert(allx.end(), gx.begin(), gx.end());
        ally.insert(ally.end(), gy.begin(), gy.end());
        l2x += l2sq(P, d->hx, gx.data());
        l2y += l2sq(P, d->hx, gy.data());
      }
      out[0] = maxabs(allx) + maxabs(ally);
      out[1] = std::sqrt(l2x) + std::sqrt(l2y);
      break;
    }
    default:
      rc = -1;
  }
  delete d;
  return rc;
}

}  // extern "C"
