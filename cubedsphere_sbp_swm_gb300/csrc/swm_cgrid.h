// swm_cgrid.h -- the C-grid SBP vector-invariant operator family on the GPU
// (the reference's &shallow_water_model_c, namelist_swm:80-102: divergence_c,
// gradient_c, curl_c, coriolis_Cgrid, KE_Cgrid, co2contra_c, massflux_c and
// the SBP_C quadrature at SBP order 21 or 42), FP64.
//
// Fields use the context's pitched layout (FieldGeom): element (p, j, i) at
// p*ps + j*P + i, each mesh occupying the leading rows / columns of the
// (N+1) x P panel slab:
//   mesh p (cell centres)  i < N,   j < N       h, kinetic energy, divergence
//   mesh u (x-faces)       i <= N,  j < N       covariant / contravariant u
//   mesh v (y-faces)       i < N,   j <= N      covariant / contravariant v
//   mesh q (corners)       i <= N,  j <= N      curl (the Ah node layout)
// Points outside a field's mesh are never written and stay as allocated.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "swm_ops.cuh"

namespace swm {

enum CMesh { CMESH_P = 0, CMESH_U = 1, CMESH_V = 2, CMESH_Q = 3 };

struct CGrid;

// Builds the metric of the four meshes, the cross-halo tables of the
// one-tile-per-panel exchanges and the work fields; order 21 or 42.
// fp32: also keep FP32 copies of the metric for the FP32 form's passes.
int cgrid_create(const FieldGeom& g, int N, int order, double radius, double grav, double omega,
                 const double axis[3], bool fp32, cudaStream_t st, CGrid** out, std::string& why);
// Only the cross-halo tables and ECS weights of the four meshes (the same
// field layout), for the ECS_xy halo and laplace_ch of an Ah-grid context,
// whose node mesh is the corner mesh.
int cgrid_create_tables(const FieldGeom& g, int N, double radius, cudaStream_t st, CGrid** out, std::string& why);
void cgrid_destroy(CGrid* c);
int cgrid_order(const CGrid* c);
// points per panel row (nx) and rows (ny) of a mesh
void cgrid_mesh_dims(const CGrid* c, int mesh, int* nx, int* ny);

// Unfused operators of the reference's plugin interface.  Each enqueues on
// st; tp / edge are the context's topology and edge buffer (corner sync).
cudaError_t cgrid_co2contra(CGrid* c, const double* u, const double* v, double* ut, double* vt,
                            cudaStream_t st);
cudaError_t cgrid_massflux(CGrid* c, const double* h, const double* ut, const double* vt, double* hu,
                           double* hv, cudaStream_t st);
cudaError_t cgrid_ke(CGrid* c, const double* u, const double* v, const double* ut, const double* vt,
                     double* ke, cudaStream_t st);
cudaError_t cgrid_grad(CGrid* c, const double* f, double* gx, double* gy, cudaStream_t st);
cudaError_t cgrid_div(CGrid* c, const double* hu, const double* hv, double* div, cudaStream_t st);
cudaError_t cgrid_curl(CGrid* c, const Topology& tp, double* edge, const double* u, const double* v,
                       double* curl, cudaStream_t st);
cudaError_t cgrid_coriolis(CGrid* c, const double* hu, const double* hv, const double* h,
                           const double* curl, double* cor_u, double* cor_v, cudaStream_t st);

// operator_swm_t%apply (vector-invariant form): tendencies (th, tu, tv) of
// the state (h, u, v); each state is 3 fields spaced g.fs apart.  hs nullable.
cudaError_t cgrid_apply(CGrid* c, const Topology& tp, double* edge, const double* hs, const double* in,
                        double* out, cudaStream_t st);
// One rk4_t%step of the state y0 in place (rk4_mod.f90:20-42).
cudaError_t cgrid_rk4(CGrid* c, const Topology& tp, double* edge, const double* hs, double* y0,
                      double dt, cudaStream_t st);
// The FP32 form (contexts created with fp32): the same passes in FP32 on
// FP32 states; the RK4 step keeps the state as an FP32 (hi, lo) pair and
// adds the stage increments with an exact two-sum.
cudaError_t cgrid_apply32(CGrid* c, const Topology& tp, float* edge, const float* hs, const float* in,
                          float* out, cudaStream_t st);
cudaError_t cgrid_rk4_32(CGrid* c, const Topology& tp, float* edge, const float* hs, float* hi, float* lo,
                         double dt, cudaStream_t st);
// A mesh field in the dense host layout (6 panels of ny rows of nx points)
// to / from its pitched device field: FP64 (lo == nullptr), or the FP32
// (hi, lo) pair, split from / joined into FP64.
cudaError_t cgrid_unpack(CGrid* c, int mesh, const double* dense, void* field, float* lo, cudaStream_t st);
cudaError_t cgrid_pack(CGrid* c, int mesh, const void* field, const float* lo, double* dense, cudaStream_t st);
// grad_perp_c_sbp21 / _sbp42 of a corner field (grad_perp_c_sbp_mod.f90:
// 20-95) and the transform2co of co2contra_c_sbp21_new / _sbp42_new
// (co2contra_Cgrid_mod.f90:135-203), at the context's order.
cudaError_t cgrid_grad_perp(CGrid* c, const double* w, double* gu, double* gv, cudaStream_t st);
cudaError_t cgrid_contra2co(CGrid* c, const double* ut, const double* vt, double* u, double* v, cudaStream_t st);
// The hyperdiffusion of operator_swm_diff_t with the C-grid names
// (hordiff_factory_mod.f90:19-36): parts 1 hordiff_c_biharm_div, 2
// hordiff_c_biharm_curl, 3 hordiff_c_biharm_curl_div for (u, v), and
// hordiff_scalar_C for h, with the 2/1 operators at any order.  c4uv, c4h:
// -(c^4) of the two coefficients.  cgrid_diffusion*: the tendency of the
// state in into out (distinct); cgrid_diffusion_step*: one explicit Euler
// step in place (FP32: on the (hi, lo) pair, with an exact two-sum).  The three
// parts run as three branches (the stream st and two side streams of the
// context, forked and joined with events).  cgrid_diffusion_prepare
// allocates their work fields, streams and events; call it once, outside
// any stream capture, before the others (they return cudaErrorInvalidValue
// until then).
cudaError_t cgrid_diffusion_prepare(CGrid* c);
cudaError_t cgrid_diffusion(CGrid* c, const Topology& tp, double* edge, int parts, double c4uv, double c4h,
                            const double* in, double* out, cudaStream_t st);
cudaError_t cgrid_diffusion_step(CGrid* c, const Topology& tp, double* edge, int parts, double c4uv, double c4h,
                                 double* y0, double dt, cudaStream_t st);
cudaError_t cgrid_diffusion32(CGrid* c, const Topology& tp, float* edge, int parts, double c4uv, double c4h,
                              const float* in, float* out, cudaStream_t st);
cudaError_t cgrid_diffusion_step32(CGrid* c, const Topology& tp, float* edge, int parts, double c4uv, double c4h,
                                   float* hi, float* lo, double dt, cudaStream_t st);
// The ECS_O scalar halo of a cell-centre field (equiang_cs/ecs_halo_mod.f90:
// 95-475, create_halo_procedure "ECS_O") and gradient_a2_ecs (gradient/
// grad_a2_mod.f90:19-69) on the centre mesh, which is the A grid's mesh.
// cgrid_ecs_o_halo: the extended tiles (6 x (N+2hw)^2, hw 1 or 2, row-major)
// into host memory, synchronously.
cudaError_t cgrid_grad_a2_ecs(CGrid* c, const double* f, double* gx, double* gy, cudaStream_t st);
cudaError_t cgrid_ecs_o_halo(CGrid* c, const double* f, int halo_width, double* ext_host, cudaStream_t st);
// The ecs_A_vec halo of contravariant (u, v) on the centres (equiang_cs/
// ecs_halo_vec_a_mod.f90:34-158) into two host arrays laid out as above, and
// divergence_a2_ecs (divergence/div_a2_mod.f90:19-72).
cudaError_t cgrid_ecs_a_vec_halo(CGrid* c, const double* u, const double* v, int halo_width, double* eu_host,
                                 double* ev_host, cudaStream_t st);
cudaError_t cgrid_div_a2_ecs(CGrid* c, const double* u, const double* v, double* div, cudaStream_t st);
// gradient_c2_ecs (gradient/grad_c2_ecs_mod.f90:33-51, 95-144): f on the
// centres, gx on the x-faces, gy on the y-faces, with the ECS_O halo.
cudaError_t cgrid_grad_c2_ecs(CGrid* c, const double* f, double* gx, double* gy, cudaStream_t st);
// The ECS_xy halo of a corner-mesh (Ah node) field (equiang_cs/
// ecs_halo_xy_mod.f90:38-217), width 1..4, its extended (N+1+2hw)^2 tiles to
// host memory (synchronous); and laplace_ch_halo2 / laplace_ch_halo4
// (laplace/laplace_ch_halo_mod.f90:15-179) of a corner-mesh field, edge-synced.
cudaError_t cgrid_ecs_xy_halo(CGrid* c, const double* f, int halo_width, double* ext_host, cudaStream_t st);
cudaError_t cgrid_laplace_ch(CGrid* c, const Topology& tp, double* edge, int order, const double* f, double* out,
                             cudaStream_t st);
// The scratch and metric tables cgrid_laplace_ch allocates on first use, made
// ahead (outside any stream capture).
cudaError_t cgrid_laplace_ch_prepare(CGrid* c, cudaStream_t st);
// SBP_C quadrature of one field of a mesh into *result (device pointer).
cudaError_t cgrid_mass(CGrid* c, int mesh, const double* f, double* result, cudaStream_t st);

}  // namespace swm
