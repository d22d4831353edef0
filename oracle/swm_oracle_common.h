// swm_oracle_common.h -- pieces shared by the Ah-grid oracle
// (swm_oracle.cpp) and the C-grid oracle (swm_oracle_c.cpp): the cube
// topology, the ECS metric on the prototype face and the analytic test
// fields of the reference's known-answer tests.
//
// TEST INFRASTRUCTURE ONLY (see swm_oracle.h).
#ifndef SWM_ORACLE_COMMON_H
#define SWM_ORACLE_COMMON_H

#include <algorithm>
#include <cmath>

namespace orc_common {

inline constexpr double PI = 3.141592653589793238462643383279502884;  // acos(-1._8)

// ---------------------------------------------------------------------------
// Cube topology: panel frames ex, ey, inward normal n and integer origin r.
// topology/cubed_sphere_topology_mod.f90:29-55 (same six frames).
// ---------------------------------------------------------------------------
inline constexpr int TEX[6][3] = {{-1, 0, 0}, {0, 0, -1}, {1, 0, 0}, {0, 0, 1}, {1, 0, 0}, {1, 0, 0}};
inline constexpr int TEY[6][3] = {{0, 1, 0}, {0, 1, 0}, {0, 1, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, -1}};
inline constexpr int TN[6][3]  = {{0, 0, 1}, {-1, 0, 0}, {0, 0, -1}, {1, 0, 0}, {0, 1, 0}, {0, -1, 0}};
inline constexpr int TR[6][3]  = {{1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 0, 0}, {0, 0, 0}, {0, 1, 1}};

inline int dot3i(const int* a, const int* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Unfolded frame of target panel pt extended across the edge it shares with
// source panel ps (cubed_sphere_topology_mod.f90:80-148 and 180-239).
struct Unfold {
  int exl[3], eyl[3], rl[3], shift[2];
};

inline Unfold unfold(int ps, int pt, int nx, int ny) {
  Unfold u{};
  const int d_right = dot3i(TEX[pt], TN[ps]);
  const int d_bt = dot3i(TEY[pt], TN[ps]);
  const int d_opp = dot3i(TN[pt], TN[ps]);
  for (int c = 0; c < 3; ++c) {
    if (d_right == -1) {  // source lies right of target
      u.exl[c] = TN[pt][c]; u.eyl[c] = TEY[pt][c]; u.rl[c] = TR[pt][c] + TEX[pt][c];
    } else if (d_right == 1) {  // left
      u.exl[c] = -TN[pt][c]; u.eyl[c] = TEY[pt][c]; u.rl[c] = TR[pt][c] + TN[pt][c];
    } else if (d_bt == 1) {  // bottom
      u.exl[c] = TEX[pt][c]; u.eyl[c] = -TN[pt][c]; u.rl[c] = TR[pt][c] + TN[pt][c];
    } else if (d_bt == -1) {  // top
      u.exl[c] = TEX[pt][c]; u.eyl[c] = TN[pt][c]; u.rl[c] = TR[pt][c] + TEY[pt][c];
    } else if (d_opp == -1) {  // opposite
      u.exl[c] = -TEX[pt][c]; u.eyl[c] = TEY[pt][c];
      u.rl[c] = TR[pt][c] + TEX[pt][c] + TN[pt][c];
    }
  }
  if (d_right == -1) { u.shift[0] = nx; u.shift[1] = 0; }
  else if (d_right == 1) { u.shift[0] = -nx; u.shift[1] = 0; }
  else if (d_bt == 1) { u.shift[0] = 0; u.shift[1] = -ny; }
  else if (d_bt == -1) { u.shift[0] = 0; u.shift[1] = ny; }
  else { u.shift[0] = 2 * nx; u.shift[1] = 0; }
  return u;
}

// transform_index: 1-based node of panel ps -> (possibly halo) index of pt.
inline void transform_index(int ps, int is, int js, int pt, int nx, int ny, int& it, int& jt) {
  if (ps == pt) { it = is; jt = js; return; }
  Unfold u = unfold(ps, pt, nx, ny);
  int dr[3];
  for (int c = 0; c < 3; ++c) dr[c] = TR[ps][c] - u.rl[c];
  const int ex_ex = dot3i(TEX[ps], u.exl), ex_ey = dot3i(TEY[ps], u.exl), ex_r = dot3i(dr, u.exl);
  const int ey_ex = dot3i(TEX[ps], u.eyl), ey_ey = dot3i(TEY[ps], u.eyl), ey_r = dot3i(dr, u.eyl);
  it = (is - 1) * ex_ex + (js - 1) * ex_ey + (nx - 1) * ex_r + 1 + u.shift[0];
  jt = (is - 1) * ey_ex + (js - 1) * ey_ey + (ny - 1) * ey_r + 1 + u.shift[1];
}

// find_basis_orientation(pn_source, pn_target): loop direction and the
// swapped/negated component order used when packing vectors.
inline void basis_orientation(int ps, int pt, int& istep, int& jstep, bool& dim_i) {
  if (ps == pt) { istep = 1; jstep = 1; dim_i = true; return; }
  Unfold u = unfold(ps, pt, 2, 2);
  const int ex_ex = dot3i(TEX[ps], u.exl), ex_ey = dot3i(TEY[ps], u.exl);
  const int ey_ex = dot3i(TEX[ps], u.eyl), ey_ey = dot3i(TEY[ps], u.eyl);
  if (ex_ex != 0) { dim_i = true; istep = ex_ex; jstep = ey_ey; }
  else { dim_i = false; istep = ex_ey; jstep = ey_ex; }
}

// ---------------------------------------------------------------------------
// ECS metric on the prototype face (equiang_cs/ecs_metric_mod.f90:326-478).
// ---------------------------------------------------------------------------
inline void r_proto(double a, double b, double r[3]) {
  const double ta = std::tan(a), tb = std::tan(b);
  const double d = std::sqrt(1.0 + ta * ta + tb * tb);
  r[0] = ta / d; r[1] = tb / d; r[2] = 1.0 / d;
}
inline void a1_proto(double a, double b, double v[3]) {
  const double ta = std::tan(a), tb = std::tan(b);
  const double p = std::pow(1.0 + ta * ta + tb * tb, 1.5);
  v[0] = (1.0 + ta * ta) * (1.0 + tb * tb) / p;
  v[1] = -ta * tb * (1.0 + ta * ta) / p;
  v[2] = -ta * (1.0 + ta * ta) / p;
}
inline void a2_proto(double a, double b, double v[3]) {
  const double ta = std::tan(a), tb = std::tan(b);
  const double p = std::pow(1.0 + ta * ta + tb * tb, 1.5);
  v[0] = -ta * tb * (1.0 + tb * tb) / p;
  v[1] = (1.0 + ta * ta) * (1.0 + tb * tb) / p;
  v[2] = -tb * (1.0 + tb * tb) / p;
}
inline void b1_proto(double a, double b, double v[3]) {
  const double ta = std::tan(a), tb = std::tan(b);
  const double s = std::sqrt(1.0 + ta * ta + tb * tb);
  v[0] = (1.0 + tb * tb - (ta * tb) * (ta * tb) / (1.0 + ta * ta)) / s;
  v[1] = 0.0;
  v[2] = -ta * (1.0 + tb * tb / (1.0 + ta * ta)) / s;
}
inline void b2_proto(double a, double b, double v[3]) {
  const double ta = std::tan(a), tb = std::tan(b);
  const double s = std::sqrt(1.0 + ta * ta + tb * tb);
  v[0] = 0.0;
  v[1] = ((1.0 + ta * ta) - (ta * tb) * (ta * tb) / (1.0 + tb * tb)) / s;
  v[2] = -tb * (ta * ta / (1.0 + tb * tb) + 1.0) / s;
}
// ecs_proto2realface with the identity rotation matrix.
inline void to_face(int p, const double v[3], double out[3]) {
  for (int c = 0; c < 3; ++c) out[c] = TEX[p][c] * v[0] + TEY[p][c] * v[1] - TN[p][c] * v[2];
}

// ---------------------------------------------------------------------------
// Analytic test fields (test_fields/test_fields_mod.f90, latlon_functions_mod,
// sph_coords_mod).  Level k (0,1,2) matters for the fields that cycle axes.
// ---------------------------------------------------------------------------
inline void field_solid_rotation(int k, double x, double y, double z, double v[3]) {
  const double ax[3] = {k == 0 ? 1.0 : 0.0, k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0};
  v[0] = ax[1] * z - ax[2] * y;
  v[1] = -ax[0] * z + ax[2] * x;
  v[2] = ax[0] * y - ax[1] * x;
}
inline void field_cross_polar(double x, double y, double z, double v[3]) {
  const double r2 = x * x + y * y + z * z;
  const double cphi = std::sqrt((x * x + y * y) / r2);
  const double sphi = z / std::sqrt(r2);
  const double rho = std::max(std::sqrt(x * x + y * y), (double)1e-14f);
  const double clam = x / rho;
  double slam = y / rho;
  if (x * x + y * y == 0.0) slam = 1.0;
  const double u = sphi * (sphi * sphi - 3.0 * cphi * cphi) * slam - 0.5 * cphi;
  const double w = sphi * sphi * clam;
  v[0] = -slam * u - sphi * clam * w;
  v[1] = clam * u - sphi * slam * w;
  v[2] = cphi * w;
}
inline double field_cross_polar_div(double x, double y, double z) { return -x * z / (x * x + y * y + z * z); }
inline double field_cross_polar_zeta(double x, double y, double z) {
  return (16.0 * (1 - z * z) * y - 13.0 * y - z) / (x * x + y * y + z * z);
}
inline double field_xyz(int k, double x, double y, double z) {
  return (k == 0 ? 1.0 : 0.0) * x + (k == 1 ? 1.0 : 0.0) * y + (k == 2 ? 1.0 : 0.0) * z;
}
inline void field_xyz_grad(int k, double x, double y, double z, double v[3]) {
  const double e[3] = {k == 0 ? 1.0 : 0.0, k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0};
  const double r = std::sqrt(x * x + y * y + z * z);
  const double nv[3] = {x / r, y / r, z / r};
  const double s = nv[0] * e[0] + nv[1] * e[1] + nv[2] * e[2];
  for (int c = 0; c < 3; ++c) v[c] = e[c] - nv[c] * s;
}
inline void field_vsh_curl_free_10(double x, double y, double z, double v[3]) {
  double lam = std::atan2(y, x);
  const double phi = std::atan2(z, std::sqrt(x * x + y * y));
  lam = lam + PI * (1.0 - (lam >= 0.0 ? 1.0 : -1.0));
  const double vl = 0.0, vp = -std::cos(phi);
  v[0] = -std::sin(lam) * vl - std::sin(phi) * std::cos(lam) * vp;
  v[1] = std::cos(lam) * vl - std::sin(phi) * std::sin(lam) * vp;
  v[2] = std::cos(phi) * vp;
}

}  // namespace orc_common

#endif
