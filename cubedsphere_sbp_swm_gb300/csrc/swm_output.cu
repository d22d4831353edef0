// swm_output.cu -- lat-lon output of Ah fields: the interpolator of the
// reference's lat-lon regrid (regridders/regrid_factory_mod.f90:9-301,
// regrid_to_latlon_mod.f90:54-165) and its application on the GPU.
//
// Set-up (host, FP64, once per grid): every point of the Nlon x Nlat grid is
// mapped to (panel, alpha, beta) by the ECS rule (the panel whose outer
// normal has the largest projection, ecs_metric_mod.f90:480-506), given a
// 2x2 (linear) or 4x4 (cubic) stencil of panel nodes clipped to the panel,
// and Lagrange weights in each direction.  For vectors, the dot products of
// the lat-lon unit vectors with b1, b2 (covariant components) or a1, a2
// (contravariant) at the point rotate the interpolated components into
// (east, north) components.  The set-up runs on the host with the same
// arithmetic as the reference so that points that fall on grid lines pick
// the same stencil.
//
// Regrid (device): one thread per lat-lon point gathers its stencil from
// the pitched panel fields (FP64, or an FP32 (hi, lo) pair summed in FP64)
// and writes FP64 and, for the file outputers, FP32 values.
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "swm_ops.cuh"

namespace swm {
namespace {

constexpr double kPiO = 3.14159265358979323846;

// Panel frames: first and second proto-face axes and the inner normal
// (cubed_sphere_topology_mod.f90:29-79); a proto-face vector v maps to
// ex*v0 + ey*v1 - n*v2.
const int kEX[6][3] = {{-1, 0, 0}, {0, 0, -1}, {1, 0, 0}, {0, 0, 1}, {1, 0, 0}, {1, 0, 0}};
const int kEY[6][3] = {{0, 1, 0}, {0, 1, 0}, {0, 1, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, -1}};
const int kN[6][3] = {{0, 0, 1}, {-1, 0, 0}, {0, 0, -1}, {1, 0, 0}, {0, 1, 0}, {0, -1, 0}};

void face_vec(int p, const double v[3], double out[3]) {
  for (int c = 0; c < 3; ++c) out[c] = kEX[p][c] * v[0] + kEY[p][c] * v[1] - kN[p][c] * v[2];
}

// Cartesian basis vectors at (alpha, beta) on the proto face
// (ecs_metric_mod.f90:326-478): covariant a1, a2 and contravariant b1, b2.
void basis_proto(double a, double b, bool contravariant_components, double e1[3], double e2[3]) {
  const double ta = std::tan(a), tb = std::tan(b);
  if (contravariant_components) {   // a1, a2
    const double p = std::pow(1.0 + ta * ta + tb * tb, 1.5);
    e1[0] = (1.0 + ta * ta) * (1.0 + tb * tb) / p;
    e1[1] = -ta * tb * (1.0 + ta * ta) / p;
    e1[2] = -ta * (1.0 + ta * ta) / p;
    e2[0] = -ta * tb * (1.0 + tb * tb) / p;
    e2[1] = (1.0 + ta * ta) * (1.0 + tb * tb) / p;
    e2[2] = -tb * (1.0 + tb * tb) / p;
  } else {                           // b1, b2
    const double s = std::sqrt(1.0 + ta * ta + tb * tb);
    e1[0] = (1.0 + tb * tb - (ta * tb) * (ta * tb) / (1.0 + ta * ta)) / s;
    e1[1] = 0.0;
    e1[2] = -ta * (1.0 + tb * tb / (1.0 + ta * ta)) / s;
    e2[0] = 0.0;
    e2[1] = ((1.0 + ta * ta) - (ta * tb) * (ta * tb) / (1.0 + tb * tb)) / s;
    e2[2] = -tb * (ta * ta / (1.0 + tb * tb) + 1.0) / s;
  }
}

template <class T>
__global__ void latlon_kernel(FieldGeom g, LatLonDev L, int nf, const T* fa, const T* fb,
                              const float* la, const float* lb, double* out, float* out32) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = L.nlon * L.nlat;
  if (q >= np) return;
  const int w = L.w;
  const long long base = L.base[q];
  double wx[4], wy[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    wx[a] = a < w ? L.wx[a * np + q] : 0.0;
    wy[a] = a < w ? L.wy[a * np + q] : 0.0;
  }
  double v[2] = {0.0, 0.0};
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    if (c >= nf) break;
    const T* F = (c ? fb : fa) + base;
    const float* Lo = c ? lb : la;
    if (Lo) Lo += base;
    double acc = 0.0;
    for (int j1 = 0; j1 < w; ++j1)
      for (int i1 = 0; i1 < w; ++i1) {
        const long long o = (long long)j1 * g.P + i1;
        const double p = Lo ? (double)F[o] + (double)Lo[o] : (double)F[o];
        acc = acc + wx[i1] * wy[j1] * p;
      }
    v[c] = acc;
  }
  if (nf == 2) {   // rotate to lat-lon components
    const double zu = v[0], zv = v[1];
    v[0] = L.rot[0 * np + q] * zu + L.rot[2 * np + q] * zv;   // u2u*zu + v2u*zv
    v[1] = L.rot[1 * np + q] * zu + L.rot[3 * np + q] * zv;   // u2v*zu + v2v*zv
  }
  for (int c = 0; c < nf; ++c) {
    if (out) out[c * np + q] = v[c];
    if (out32) out32[c * np + q] = (float)v[c];
  }
}

}  // namespace

int latlon_setup(int N, int nlon, int nlat, int width, int contravariant, const FieldGeom& g,
                 LatLonHost& h) {
  if (nlon < 1 || nlat < 2 || (width != 2 && width != 4)) return -1;
  const int np = nlon * nlat, n = N + 1;
  h.nlon = nlon; h.nlat = nlat; h.w = width;
  h.base.assign(np, 0);
  h.wx.assign((size_t)4 * np, 0.0);
  h.wy.assign((size_t)4 * np, 0.0);
  h.rot.assign((size_t)4 * np, 0.0);
  const double hx = (0.25 * kPiO - (-0.25 * kPiO)) / (double)N;
  const double alpha0 = -0.25 * kPiO;
  const double hlon = 2.0 * kPiO / (double)nlon, hlat = kPiO / (nlat - 1.0);
  auto rows = [&](int j0, int j1) {
    for (int j = j0; j < j1; ++j)
      for (int i = 0; i < nlon; ++i) {
        const int q = j * nlon + i;
        const double lat = -0.5 * kPiO + hlat * j, lon = hlon * i;
        const double r[3] = {std::cos(lat) * std::cos(lon), std::cos(lat) * std::sin(lon),
                             std::sin(lat)};
        int p = 0;
        double best = 0.0;
        for (int pp = 0; pp < 6; ++pp) {
          const double rn = -(r[0] * kN[pp][0] + r[1] * kN[pp][1] + r[2] * kN[pp][2]);
          if (rn > best) { p = pp; best = rn; }
        }
        const double a = std::atan((kEX[p][0] * r[0] + kEX[p][1] * r[1] + kEX[p][2] * r[2]) / best);
        const double b = std::atan((kEY[p][0] * r[0] + kEY[p][1] * r[1] + kEY[p][2] * r[2]) / best);
        const double zdx = (a - alpha0) / hx + 1.0, zdy = (b - alpha0) / hx + 1.0;
        int ir = std::min((int)std::floor(zdx) + width / 2, n);
        const int x1 = std::max(ir - width + 1, 1);
        ir = std::min((int)std::floor(zdy) + width / 2, n);
        const int y1 = std::max(ir - width + 1, 1);
        h.base[q] = (long long)p * g.ps + (long long)(y1 - 1) * g.P + (x1 - 1);
        const double dx = zdx - x1, dy = zdy - y1;
        double* WX = &h.wx[q];
        double* WY = &h.wy[q];
        if (width == 2) {
          WX[0] = 1.0 - dx; WX[np] = dx;
          WY[0] = 1.0 - dy; WY[np] = dy;
        } else {
          WX[0] = -(dx - 1.0) * (dx - 2.0) * (dx - 3.0) / 6.0;
          WX[np] = dx * (dx - 2.0) * (dx - 3.0) / 2.0;
          WX[2 * np] = -dx * (dx - 1.0) * (dx - 3.0) / 2.0;
          WX[3 * np] = dx * (dx - 1.0) * (dx - 2.0) / 6.0;
          WY[0] = -(dy - 1.0) * (dy - 2.0) * (dy - 3.0) / 6.0;
          WY[np] = dy * (dy - 2.0) * (dy - 3.0) / 2.0;
          WY[2 * np] = -dy * (dy - 1.0) * (dy - 3.0) / 2.0;
          WY[3 * np] = dy * (dy - 1.0) * (dy - 2.0) / 6.0;
        }
        const double iv[3] = {-std::sin(lon), std::cos(lon), 0.0};
        const double jv[3] = {-std::sin(lat) * std::cos(lon), -std::sin(lat) * std::sin(lon),
                              std::cos(lat)};
        double e1p[3], e2p[3], e1[3], e2[3];
        basis_proto(a, b, contravariant != 0, e1p, e2p);
        face_vec(p, e1p, e1);
        face_vec(p, e2p, e2);
        h.rot[q] = iv[0] * e1[0] + iv[1] * e1[1] + iv[2] * e1[2];            // u2u
        h.rot[np + q] = jv[0] * e1[0] + jv[1] * e1[1] + jv[2] * e1[2];       // u2v
        h.rot[2 * np + q] = iv[0] * e2[0] + iv[1] * e2[1] + iv[2] * e2[2];   // v2u
        h.rot[3 * np + q] = jv[0] * e2[0] + jv[1] * e2[1] + jv[2] * e2[2];   // v2v
      }
  };
  const int nt = std::max(1, std::min((int)std::thread::hardware_concurrency(), 32));
  if (nt == 1 || nlat < 64) {
    rows(0, nlat);
  } else {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back(rows, (int)((long long)nlat * t / nt), (int)((long long)nlat * (t + 1) / nt));
    for (auto& t : th) t.join();
  }
  return 0;
}

template <class T>
cudaError_t launch_latlon(const FieldGeom& g, const LatLonDev& L, int nf, const T* fa, const T* fb,
                          const float* la, const float* lb, double* out, float* out32,
                          cudaStream_t st) {
  if (nf != 1 && nf != 2) return cudaErrorInvalidValue;
  const int np = L.nlon * L.nlat;
  latlon_kernel<T><<<(np + 255) / 256, 256, 0, st>>>(g, L, nf, fa, fb, la, lb, out, out32);
  return cudaGetLastError();
}
template cudaError_t launch_latlon<double>(const FieldGeom&, const LatLonDev&, int, const double*,
                                           const double*, const float*, const float*, double*,
                                           float*, cudaStream_t);
template cudaError_t launch_latlon<float>(const FieldGeom&, const LatLonDev&, int, const float*,
                                          const float*, const float*, const float*, double*,
                                          float*, cudaStream_t);

}  // namespace swm
