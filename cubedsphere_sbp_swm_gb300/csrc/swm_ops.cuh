// swm_ops.cuh -- host-callable launchers of the per-operator (unfused) FP64
// kernels, the FP64 geometry precompute, state linear combinations and the
// deterministic FP64 reductions.  Implemented in swm_ops.cu.
#pragma once

#include "swm_device.cuh"

#include <vector>

namespace swm {

struct FieldGeom {
  int n, P;
  long long ps, fs;   // panel stride, field stride (elements)
};

// Geometry (FP64): metric fields J, Qi1, Qi2, Qi3, f, rJ into m64 (NMETRIC
// fields of fs doubles) and sync weights qb|qt|ql|qr into qw (4n doubles).
cudaError_t launch_geometry(const FieldGeom& g, int N, double radius, double omega,
                            const double axis[3], double* m64, double* qw, cudaStream_t st);
// Cartesian contravariant basis vectors: 6 fields b1x b1y b1z b2x b2y b2z
cudaError_t launch_basis(const FieldGeom& g, double hx, double* b, cudaStream_t st);
// FP64 -> FP32 copy of nfields fields
cudaError_t launch_to_f32(const double* src, float* dst, long long count, cudaStream_t st);

// Per-operator FP64 kernels on (pitched) fields.
cudaError_t launch_co2contra(const FieldGeom& g, const double* m64, const double* u,
                             const double* v, double* ut, double* vt, cudaStream_t st);
cudaError_t launch_massflux(const FieldGeom& g, const double* h, const double* ut,
                            const double* vt, double* hu, double* hv, cudaStream_t st);
cudaError_t launch_ke(const FieldGeom& g, const double* u, const double* v, const double* ut,
                      const double* vt, double* ke, cudaStream_t st);
// ke += grav*h + grav*hs (hs nullable)
cudaError_t launch_ke_update(const FieldGeom& g, double grav, const double* h, const double* hs,
                             double* ke, cudaStream_t st);
// pre-sync SBP gradient: gx = Dx f / (hx a), gy = Dy f / (hx a)
cudaError_t launch_grad_presync(const FieldGeom& g, int order, double ghs, const double* f,
                                double* gx, double* gy, cudaStream_t st);
// pre-sync SBP divergence (Dx(J u) + Dy(J v)) / (J hx a); curl_form: the
// input is covariant and the operator uses (v/J, -u/J).
cudaError_t launch_div_presync(const FieldGeom& g, int order, double hx_a, const double* m64,
                               const double* u, const double* v, int curl_form, double* out,
                               cudaStream_t st);
cudaError_t launch_coriolis(const FieldGeom& g, const double* m64, const double* hu,
                            const double* hv, const double* h, const double* curl,
                            double* cor_u, double* cor_v, cudaStream_t st);
// out[k] = value for k < count
cudaError_t launch_fill(long long count, double value, double* out, cudaStream_t st);
// out = s1*a + s2*b over count elements (b nullable)
cudaError_t launch_axpby(long long count, double s1, const double* a, double s2, const double* b,
                         double* out, cudaStream_t st);
// Cube-edge syncs of pitched FP64 fields: gather the boundary values into
// the edge buffer, then apply the reference's averaging.
cudaError_t launch_sync_scalar(const FieldGeom& g, const Topology& tp, double* f, double* edge,
                               cudaStream_t st);
cudaError_t launch_sync_vector(const FieldGeom& g, const Topology& tp, const double* qw,
                               double* gx, double* gy, double* edge, cudaStream_t st);
// the same syncs on fields of either precision (edge buffer of that precision)
template <class T>
cudaError_t launch_sync_scalar_t(const FieldGeom& g, const Topology& tp, T* f, T* edge,
                                 cudaStream_t st);
template <class T>
cudaError_t launch_sync_vector_t(const FieldGeom& g, const Topology& tp, const double* qw, T* gx,
                                 T* gy, T* edge, cudaStream_t st);

// Transposed SBP first-derivative operator D^T: t[c*kr + r] = D[r][c] for
// the columns c < ct next to the left end (rows r < kr); the right end is
// the sign-flipped mirror and the interior the negated interior stencil
// (qin, inshift as in SbpC).  Needs n >= 2*kr.
struct SbpT {
  int ct, kr, nin, inshift;
  double t[9 * 12];
  double qin[7];
};

// Tangent-linear and adjoint pieces of the FP64 model operator (swm_adjoint.cu).
// y, dx, dk, lk, out: 3 fields (h, u, v); w: 5 fields (dK, d(h ut), d(h vt),
// dut, dvt); A: 6 fields.
cudaError_t launch_tl_pre(const FieldGeom& g, const double* m64, double grav, const double* y,
                          const double* dx, double* w, cudaStream_t st);
cudaError_t launch_tl_post(const FieldGeom& g, const double* m64, const double* y,
                           const double* zeta, const double* w, const double* dgx,
                           const double* dgy, const double* dz, const double* ddiv, double* dk,
                           cudaStream_t st);
// Adjoint stage pieces, FP64 or FP32 (order = SBP order of the context;
// m = metric of the element type; qw = FP64 sync weights):
// zeta = pre-sync curl rJ (Dx v - Dy u) of the state y, boundary values also
// into the EV_ZETA slots of the edge buffer Z;
template <class T>
cudaError_t launch_zeta_pre(const FieldGeom& g, int order, const T* m, const T* y, T* zeta, T* Z,
                            cudaStream_t st);
// A (6 fields) from lk = alpha*lam + beta*mu (mu nullable), boundary
// cotangents pulled into the edge buffer C;
template <class T>
cudaError_t launch_ad_pre(const FieldGeom& g, const Topology& tp, const double* qw, const T* m,
                          const T* y, const T* zeta, const T* Z, const T* lam, const T* mu, T alpha,
                          T beta, T* A, T* C, cudaStream_t st);
// the transposed cube-edge syncs of A's first four fields from C;
template <class T>
cudaError_t launch_adsync_gather(const FieldGeom& g, const Topology& tp, const T* m, const T* C,
                                 T* A, cudaStream_t st);
// out = F'(y)^T lk (out nullable); acc_out = acc_in + out (both nullable,
// may alias)
template <class T>
cudaError_t launch_ad_main(const FieldGeom& g, int order, const SbpT& t, const T* m, T ghs, T grav,
                           const T* y, const T* A, T* out, const T* acc_in, T* acc_out,
                           cudaStream_t st);
// transposed-table width of an SBP order (must match make_sbpT)
int adjoint_table_ct(int order);

// Deterministic FP64 reductions over the valid nodes of a field.
// kind: 0 sum(a*b), 1 SBP mass sum(a*J*hx^2*Ax*Ay), 2 min(a), 3 max(a),
//       4 SBP mass of a*b.
cudaError_t launch_reduce(const FieldGeom& g, int kind, const double* a, const double* b,
                          const double* J, const double* Aw, double hx2, double* partial,
                          int nblocks, double* result, cudaStream_t st);
constexpr int REDUCE_BLOCKS = 264;

// Per-node integrands of the SWM diagnostics (operator_swm_mod.f90:211-260):
// ke_u = 0.5*(h*ut)*u, ke_v = 0.5*(h*vt)*v, pe = 0.5*g*(h+hs)^2,
// ens = 0.5*(zeta+f)^2/h.
cudaError_t launch_diag_integrands(const FieldGeom& g, const double* m64, double grav,
                                   const double* h, const double* u, const double* v,
                                   const double* hs, const double* zeta, double* ke_u,
                                   double* ke_v, double* pe, double* ens, cudaStream_t st);

// State combinations for the FP32 compensated representation: out = s1*(a_hi
// + a_lo) + s2*(b_hi + b_lo) (b nullable) in double-float arithmetic on FP32
// instructions; out may alias a or b.  fill: (hi, lo) = value.
cudaError_t launch_axpby_f32pair(long long count, double s1, const float* ahi, const float* alo,
                                 double s2, const float* bhi, const float* blo, float* ohi,
                                 float* olo, cudaStream_t st);
cudaError_t launch_fill_f32pair(long long count, double value, float* ohi, float* olo,
                                cudaStream_t st);
// FP64 <-> (hi, lo) FP32 pair conversions
cudaError_t launch_split_f64(long long count, const double* src, float* hi, float* lo,
                             cudaStream_t st);
cudaError_t launch_join_f32pair(long long count, const float* hi, const float* lo, double* dst,
                                cudaStream_t st);
// Packed FP64 fields (6*n*n values each, panel-major, row-major inside a
// panel) <-> nf pitched state fields at field stride fs.  lo == nullptr: the
// state is FP64 (hi holds doubles); otherwise hi/lo are the FP32 pair, split
// on unpack and summed in FP64 on pack.
struct PackedFields {
  double* f[3];
};
cudaError_t launch_unpack_state(const FieldGeom& g, int nf, const PackedFields& src, void* hi,
                                float* lo, cudaStream_t st);
cudaError_t launch_pack_state(const FieldGeom& g, int nf, const void* hi, const float* lo,
                              const PackedFields& dst, cudaStream_t st);

// Hyperdiffusion (swm_diffusion.cu): narrow-stencil SBP Laplacians of order
// narrow = 42 or 63, on fields of element type T.  Per-context coefficient
// tables of one order: interior stencil coefficients (narrow_width fields
// each for x and y; FP64 contexts), the variable coefficients (2 fields;
// FP32 contexts form the interior coefficients from them) and the closure
// rows (narrow_closure_count values each for x and y), built in FP64.
template <class T>
struct NarrowTables {
  int narrow;
  T *cx, *cy, *clx, *cly;
  T* b;   // the variable coefficients J*Qi11 (field 0) and J*Qi22 (field 1)
};
int narrow_rows(int narrow);
int narrow_cols(int narrow);
int narrow_width(int narrow);
long long narrow_closure_count(int narrow, int n);
template <class T>
cudaError_t launch_narrow_tables(const FieldGeom& g, const NarrowTables<T>& t, const double* m,
                                 cudaStream_t st);
// Edge-synced Laplacian of nf = 1, 3 or 4 fields f into out (all at field
// stride g.fs, out must not overlap f); mt: metric of element type T;
// hs = hx * radius; edge: edge buffer of element type T; d1x, d1y: nf work
// fields each (FP64; FP32 passes null).  The tables' launcher must have run
// first (it sets the FP32 tile kernel's shared memory).
template <class T>
cudaError_t launch_laplace(const FieldGeom& g, const Topology& tp, const NarrowTables<T>& t, int nf,
                           const T* f, const T* mt, double hs, T* d1x, T* d1y, T* out, T* edge,
                           cudaStream_t st);
// cart (3 fields) = b1*u + b2*v; b12 from launch_basis
// cart = b1*u + b2*v (3 fields) and, when h_out is given, h_out = h
template <class T>
cudaError_t launch_to_cart(const FieldGeom& g, const T* b12, const T* h, const T* u, const T* v,
                           T* h_out, T* cart, cudaStream_t st);
// tu, tv = projections of cuv*L (3 Cartesian fields) on b1, b2; th = ch*Lh
template <class T>
cudaError_t launch_diff_tendency(const FieldGeom& g, const T* b12, double cuv, const T* L, T* tu,
                                 T* tv, double ch, const T* Lh, T* th, cudaStream_t st);
// FP32 (hi, lo) += dt * t, over count elements
// The FP32 diffusion step's state update from the twice-applied Laplacians
// (L: 3 Cartesian fields, Lh: h): tendencies cuv*L projected on b1, b2 and
// ch*Lh, the covariant sync of the velocity tendency, and the (hi, lo) pair
// update by dt, in two launches; tu, tv: work fields for the panel-boundary
// nodes.  edge_in (nullable): the edge buffer of the Laplacian that wrote
// Lh (slot 0) and L (slots 1..3) when their panel-side values are not yet
// synced (launch_biharmonic_f32); edge must be another buffer.
cudaError_t launch_diff_update_f32(const FieldGeom& g, const Topology& tp, const double* qw,
                                   const float* b12, double cuv, const float* L, double ch,
                                   const float* Lh, double dt, float* hi, float* lo, float* tu,
                                   float* tv, float* edge, const float* edge_in, cudaStream_t st);
// The FP32 biharmonic L(L(f)) of the 4 fields [h, x, y, z] of the 4/2
// narrow order in two tile launches and no sync launch: f is overwritten with the
// result, whose panel-side values are left for the consumer to sync from
// edge_b; L is a work area of 4 fields, edge_a another edge buffer.
cudaError_t launch_biharmonic_f32(const FieldGeom& g, const Topology& tp,
                                  const NarrowTables<float>& t, float* f, float* L, const float* mt,
                                  double hs, float* edge_a, float* edge_b, cudaStream_t st);
template <class T>
cudaError_t launch_pair_axpy(long long count, double dt, const T* t, float* hi, float* lo,
                             cudaStream_t st);
cudaError_t launch_f64_to_f32(long long count, const double* s, float* d, cudaStream_t st);


// Lat-lon output (swm_output.cu).  Interpolator of an Nlon x Nlat grid with
// stencil width w (2 linear, 4 cubic): per point the pitched offset of its
// stencil's first node, w weights per direction (point-major planes) and
// the rotation u2u, u2v, v2u, v2v to lat-lon components.
struct LatLonHost {
  int nlon = 0, nlat = 0, w = 0;
  std::vector<long long> base;
  std::vector<double> wx, wy, rot;   // 4 planes of nlon*nlat each
};
struct LatLonDev {
  int nlon, nlat, w;
  const long long* base;
  const double *wx, *wy, *rot;
};
// host set-up (regrid_factory_mod.f90:195-299; rotation of 121-160 for
// covariant or contravariant components); -1 on bad arguments
int latlon_setup(int N, int nlon, int nlat, int width, int contravariant, const FieldGeom& g,
                 LatLonHost& h);
// nf = 1: out = regrid of fa; nf = 2: the vector (fa, fb) regridded and
// rotated, out = (u plane, v plane).  la/lb: FP32 low parts (nullable);
// out (FP64) and out32 (FP32) nullable.
template <class T>
cudaError_t launch_latlon(const FieldGeom& g, const LatLonDev& L, int nf, const T* fa, const T* fb,
                          const float* la, const float* lb, double* out, float* out32,
                          cudaStream_t st);

}  // namespace swm
