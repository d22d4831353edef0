/*
 * swm_gpu.h -- C-ABI of the GB300 shallow-water hot path.
 *
 * Drop-in boundary for the reference's Fortran plugin surface
 * (vvshashkin/cubedsphere_sbp_swm).  Every entry point below names the
 * reference interface it replaces (file:line inside the reference project).
 * A Fortran caller binds these with iso_c_binding; Python/C++ callers use
 * plain pointers and sizes.  No torch or CUDA types appear in the signatures.
 *
 * Conventions
 *  - Every function returns SWM_OK (0) or a negative SWM_E_* code; the
 *    message of the last failure is swm_last_error(ctx) (or
 *    swm_last_error(NULL) for failures without a context).  Nothing aborts,
 *    traps or exits: the reference's parcomm_global%abort paths
 *    (parallel/parcomm_mod.f90:73-83) become error codes.
 *  - Host arrays use the reference layout of one tile per panel: for each of
 *    the 6 panels an (N+1) x (N+1) FP64 array p(1:N+1, 1:N+1) with i (alpha)
 *    fastest, panels stored one after another (6*(N+1)^2 doubles).  N is the
 *    number of cells per panel edge as in the reference namelist
 *    (domain/config_domain_mod.f90), so panel edge nodes are duplicated on
 *    both panels exactly as in the reference Ah grid.
 *  - Device memory belongs to the context; every call is ordered on the
 *    context's CUDA stream.  A context is not thread-safe (the reference
 *    operators are not re-entrant either: they share work fields).
 */
#ifndef SWM_GPU_H
#define SWM_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWM_OK             0
#define SWM_E_INVALID     -1  /* bad argument, size or handle */
#define SWM_E_UNSUPPORTED -2  /* unknown operator / scheme name or option */
#define SWM_E_CUDA        -3  /* CUDA runtime failure */
#define SWM_E_NOMEM       -4  /* device or host allocation failed */
#define SWM_E_DEVICE      -5  /* a kernel raised its device error flag */
#define SWM_E_IO          -6  /* an output file could not be opened or written */

/* Arithmetic of the hot path. */
#define SWM_FP64_PLAIN 0   /* FP64 end to end; parity path (1e-12 rel. L2/step) */
#define SWM_FP32_FUSED 1   /* FP32 stencils, compensated RK4 stage sums, FP64
                              metric precompute and FP64 global integrals */

typedef struct swm_ctx swm_ctx;      /* domain + operator + time scheme */
typedef struct swm_state swm_state;  /* stvec_swm_t: (h, u, v) on the device */
typedef struct swm_field swm_field;  /* grid_field_t: one FP64 field */
typedef struct swm_latlon swm_latlon;  /* lat-lon interpolator of a context */

/* Model configuration: the &domain, &metric and &shallow_water_model keys
 * the hot path needs (domain/config_domain_mod.f90:26-58,
 * metric/config_metric_mod.f90:37-63, models/shallow_water/config/
 * config_swm_mod.f90:8-107).  Physical constants are explicit. */
typedef struct swm_config {
  int    N;                 /* cells per panel edge (>= 16) */
  int    sbp_order;         /* 21, 42, 43 or 63 (SBP d21/d42/d43/d63) */
  double radius;            /* sphere radius a [m]   (metric "scale") */
  double grav;              /* gravity g [m s^-2] */
  double omega;             /* rotation rate [s^-1] */
  double rotation_axis[3];  /* normalised internally */
  int    precision;         /* SWM_FP64_PLAIN or SWM_FP32_FUSED */
  int    device;            /* CUDA device ordinal */
} swm_config;

/* ---------------------------------------------------------------------- */
/* Construction                                                            */
/* ---------------------------------------------------------------------- */

/* create_domain + create_swm_operator + create_timescheme("rk4") in one:
 * domain/domain_factory_mod.f90:44-136,
 * models/shallow_water/operator/operator_swm_factory_mod.f90:43-131,
 * time_schemes/timescheme_factory_mod.f90:42-59.  Uses the operator names
 * that match cfg->sbp_order (divergence_ahXX_sbp, gradient_ahXX_sbp_ecs,
 * curl_divergence_ahXX_sbp, coriolis_colocated, KE_colocated,
 * co2contra_colocated, massflux_colocated, SBP_AhXX_quadrature). */
int swm_ctx_create(const swm_config* cfg, swm_ctx** out);

/* As swm_ctx_create, with the operator names of the &shallow_water_model
 * namelist (config_swm_mod.f90:70-104).  Two operator families:
 *   Ah grid (staggering "Ah"): divergence_ahXX_sbp, gradient_ahXX_sbp_ecs,
 *     curl_divergence_ahXX_sbp (XX 42, 43, 63), coriolis_colocated,
 *     KE_colocated, co2contra_colocated, massflux_colocated,
 *     SBP_AhXX_quadrature; FP64 or the FP32 fused form;
 *   C grid (staggering "C", the &shallow_water_model_c namelist,
 *     namelist_swm:80-102): divergence_c_sbpNN, gradient_c_sbpNN,
 *     curl_c_sbpNN, coriolis_Cgrid_sbpNN, KE_Cgrid_sbpNN,
 *     co2contra_c_sbpNN (or co2contra_c_sbpNN_new, the same map),
 *     massflux_c_sbpNN, SBP_CNN_quadrature with NN 21 or 42, one order
 *     throughout; FP64 or the FP32 form (FP32 passes on an FP32 (hi, lo)
 *     state pair).  h lives on the cell centres, u on the x-faces, v on the
 *     y-faces (domain_factory_mod.f90:108-112).
 * Other names, or operators of different SBP orders, return
 * SWM_E_UNSUPPORTED.  A C-grid context provides the state algebra and
 * transfers, apply, the RK4 step, the hyperdiffusion and the model step,
 * orography, fields and the single operators below; the other entry points
 * return SWM_E_UNSUPPORTED on it. */
int swm_ctx_create_named(const swm_config* cfg, const char* div_op_name,
                         const char* grad_op_name, const char* curl_op_name,
                         const char* coriolis_op_name, const char* KE_op_name,
                         const char* co2contra_op_name,
                         const char* massflux_op_name,
                         const char* quadrature_name, swm_ctx** out);

void        swm_ctx_destroy(swm_ctx* ctx);
const char* swm_last_error(const swm_ctx* ctx);
int         swm_ctx_synchronize(swm_ctx* ctx);
/* The context's cudaStream_t, for callers that interleave their own work. */
void*       swm_ctx_stream(swm_ctx* ctx);
/* Number of nodes per field, 6*(N+1)^2 (the Ah grid; see swm_mesh_dims). */
size_t      swm_ctx_npts(const swm_ctx* ctx);

/* Staggering of a context and its meshes (mesh_p, mesh_u, mesh_v, mesh_q of
 * domain_t).  On the Ah grid all four are the (N+1) x (N+1) node mesh; on
 * the C grid p is N x N cell centres, u (N+1) x N x-faces, v N x (N+1)
 * y-faces, q (N+1) x (N+1) corners.  Host arrays of a mesh are 6 panels of
 * ny rows of nx points, i fastest. */
#define SWM_GRID_AH 0
#define SWM_GRID_C  1
#define SWM_MESH_P 0
#define SWM_MESH_U 1
#define SWM_MESH_V 2
#define SWM_MESH_Q 3
int swm_ctx_grid(const swm_ctx* ctx);                      /* SWM_GRID_* or -1 */
int swm_mesh_dims(const swm_ctx* ctx, int mesh, int* nx, int* ny);

/* Orography h_surf (operator_swm_factory_mod.f90:120-121; zero if never set). */
int swm_set_orography(swm_ctx* ctx, const double* h_surf_host);

/* ---------------------------------------------------------------------- */
/* State vector: stvec_t (stvec_mod.f90:10-28), stvec_swm_t                 */
/* (models/shallow_water/stvec/stvec_swm_mod.f90:10-106)                    */
/* ---------------------------------------------------------------------- */
int  swm_state_create(swm_ctx* ctx, swm_state** out);   /* create_stvec_swm */
int  swm_state_create_similar(swm_ctx* ctx, const swm_state* src,
                              swm_state** out);          /* %create_similar */
void swm_state_free(swm_state* s);
int  swm_state_upload(swm_ctx* ctx, swm_state* s, const double* h,
                      const double* u, const double* v);
int  swm_state_download(swm_ctx* ctx, const swm_state* s, double* h,
                        double* u, double* v);
/* Asynchronous transfers (no reference counterpart): the same packed host
 * layout as swm_state_upload / swm_state_download, moved by the copy engines
 * on two transfer streams of the context (one per direction) through device
 * staging buffers, so that transfers overlap the context's kernels and each
 * other.  Both return at once.
 *   upload_async: s holds the arrays' values for every call queued after
 *     it; the arrays must stay unchanged until swm_ctx_synchronize returns.
 *   download_async: copies s as the calls queued before it leave it (s may
 *     be changed right after the call); the arrays hold the values once
 *     swm_ctx_synchronize returns.
 * Page-locked host arrays give the overlap; pageable ones work but block. */
int  swm_state_upload_async(swm_ctx* ctx, swm_state* s, const double* h,
                            const double* u, const double* v);
int  swm_state_download_async(swm_ctx* ctx, const swm_state* s, double* h,
                              double* u, double* v);
/* this = s1                       (%assign_s1) */
int swm_assign_s1(swm_ctx* ctx, swm_state* s, double s1);
/* this = s1*v1                    (%assign_s1v1) */
int swm_assign_s1v1(swm_ctx* ctx, swm_state* s, double s1, const swm_state* v1);
/* this = s1*v1 + s2*v2            (%assign_s1v1s2v2, stvec_swm_mod.f90:38-62) */
int swm_assign_s1v1s2v2(swm_ctx* ctx, swm_state* s, double s1,
                        const swm_state* v1, double s2, const swm_state* v2);
/* this = this + s1*v1             (%update_s1v1, stvec_swm_mod.f90:88-106) */
int swm_update_s1v1(swm_ctx* ctx, swm_state* s, double s1, const swm_state* v1);
/* this = this + s1*v1 + s2*v2     (%update_s1v1s2v2, stvec_swm_mod.f90:63-87) */
int swm_update_s1v1s2v2(swm_ctx* ctx, swm_state* s, double s1,
                        const swm_state* v1, double s2, const swm_state* v2);
/* algebraic dot / norm2 over all nodes of h, u, v (%algebraic_dot/norm2) */
int swm_dot(swm_ctx* ctx, const swm_state* a, const swm_state* b, double* out);
int swm_norm2(swm_ctx* ctx, const swm_state* a, double* out);

/* ---------------------------------------------------------------------- */
/* Operator and time scheme                                                */
/* ---------------------------------------------------------------------- */
/* vout = A(vin): operator_t%apply (operator_mod.f90:18-25), implemented by
 * operator_swm_t%apply (operator_swm_mod.f90:61-113) as one fused kernel
 * pass plus the cube-edge pass. */
int swm_apply(swm_ctx* ctx, swm_state* vout, const swm_state* vin);
/* Same result through the unfused FP64 per-operator kernels in the
 * reference's call order (co2contra, massflux, KE, grad+sync, curl+sync,
 * coriolis, div+sync).  FP64 contexts only. */
int swm_apply_unfused(swm_ctx* ctx, swm_state* vout, const swm_state* vin);
/* nsteps of rk4_t%step (time_schemes/rk4_mod.f90:20-42) on v0, in place,
 * with the stage combinations folded into the RHS kernels and the step
 * replayed as a CUDA graph. */
int swm_rk4_step(swm_ctx* ctx, swm_state* v0, double dt, int nsteps);

/* ---------------------------------------------------------------------- */
/* Hyperdiffusion split step                                              */
/* ---------------------------------------------------------------------- */
/* The reference drivers follow every RK4 step with one explicit Euler step
 * of operator_swm_diff_t (operator_swm_diff_mod.f90:25-46; ts2_mod.f90:
 * 143-146, barotropic_inst_mod.f90:163-168).  swm_diffusion_set takes the
 * namelist's hordiff_uv_name / uv_diff_coeff / hordiff_h_name /
 * h_diff_coeff (config_swm_mod.f90:24-27, operator_swm_diff_factory_mod.f90
 * :27-30).  Supported names on the Ah grid: "hordiff_vec_xyz_Ah_sbp_NN_narrow"
 * for (u, v) and "hordiff_scalar_Ah_sbp_NN_narrow" for h, NN = 21, 42 or 63
 * (hordiff_factory_mod.f90:27-46).  The operator is -(c^4) L(L(.)) with L
 * the narrow-stencil SBP Laplacian and c = coeff*radius*hx, on h and on the
 * Cartesian components of the velocity.  "hordiff_vec_xyz_Ah" and
 * "hordiff_scalar_Ah" (hordiff_factory_mod.f90:33-40, 196-223) are the same
 * with L = laplace_ch_halo4 and its ECS_xy halo, and "hordiff_vec_Ah" that L
 * on the covariant components as scalars, then the covariant vector sync;
 * these three on FP64 contexts.  On the C grid
 * (hordiff_factory_mod.f90:19-36, 53-139, 196-247): "hordiff_c_biharm_div",
 * "hordiff_c_biharm_curl" or "hordiff_c_biharm_curl_div" for (u, v) --
 * -(c^4) grad div co2contra grad div co2contra and / or -(c^4) contra2co
 * grad_perp curl contra2co grad_perp curl -- and "hordiff_scalar_C" for h,
 * -(c^4) L(L(h)) with L = div co2contra grad, all with the sbp21 operators
 * whatever the context's order.  Other names give SWM_E_UNSUPPORTED.  FP64
 * contexts compute the tendency in FP64; FP32 contexts compute it in FP32
 * from the high part of the state and add dt times it to the (hi, lo) pair
 * with an exact two-sum. */
int swm_diffusion_set(swm_ctx* ctx, const char* hordiff_uv_name, double uv_diff_coeff,
                      const char* hordiff_h_name, double h_diff_coeff);
/* vout = D(vin): operator_swm_diff_t%apply (operator_swm_diff_mod.f90:
 * 25-46). */
int swm_apply_diffusion(swm_ctx* ctx, swm_state* vout, const swm_state* vin);
/* nsteps of explicit_Eul1_t%step (explicit_Eul1_mod.f90:20-30) with the
 * diffusion operator: v0 += dt * D(v0); one CUDA graph per step. */
int swm_diffusion_step(swm_ctx* ctx, swm_state* v0, double dt, int nsteps);
/* nsteps of the drivers' time step (ts2_mod.f90:143-146): rk4_t%step then
 * the diffusion step, both as one CUDA graph per step; without
 * swm_diffusion_set the same as swm_rk4_step. */
int swm_model_step(swm_ctx* ctx, swm_state* v0, double dt, int nsteps);
/* out = L(in): laplace_operator_t%calc_laplace of laplace_ah_sbp21_narrow /
 * _sbp42_narrow / _sbp63_narrow (laplace_Ah_sbp42_narrow_mod.f90:23-58,
 * laplace_Ah_sbp21_narrow_mod.f90:23-243, laplace_factory_mod.f90:179-250)
 * on FP64 fields, edge-synced; out may be in.  narrow_order = 21, 42 or 63. */
int swm_laplace(swm_ctx* ctx, swm_field* out, const swm_field* in, int narrow_order);

/* get_diagnostics (operator_swm_mod.f90:115-155): out[7] = hmin, hmax,
 * mass, TE, KE, PE, Enstrophy, all FP64 with SBP quadrature. */
int swm_diagnostics(swm_ctx* ctx, const swm_state* v, double out[7]);

/* ---------------------------------------------------------------------- */
/* Fields and single operators (grid_field_t, grid_field_mod.f90:7-65)     */
/* FP64, reference semantics, one kernel pass each (parity mode).          */
/* ---------------------------------------------------------------------- */
int  swm_field_create(swm_ctx* ctx, swm_field** out);   /* on mesh p */
/* a field on one of the context's meshes (create_grid_field on mesh_p/u/v/q) */
int  swm_field_create_mesh(swm_ctx* ctx, int mesh, swm_field** out);
void swm_field_free(swm_field* f);
int  swm_field_upload(swm_ctx* ctx, swm_field* f, const double* host);
int  swm_field_download(swm_ctx* ctx, const swm_field* f, double* host);

/* co2contra_colocated%transform (co2contra_colocated_mod.f90:20-60) */
int swm_op_co2contra(swm_ctx* ctx, swm_field* ut, swm_field* vt,
                     const swm_field* u, const swm_field* v);
/* massflux_colocated (massflux_colocated_mod.f90:19-29) */
int swm_op_massflux(swm_ctx* ctx, swm_field* hu, swm_field* hv,
                    const swm_field* h, const swm_field* ut,
                    const swm_field* vt);
/* KE_colocated (kinetic_energy/KE_colocated_mod.f90:17-48) */
int swm_op_ke(swm_ctx* ctx, swm_field* ke, const swm_field* u,
              const swm_field* v, const swm_field* ut, const swm_field* vt);
/* grad_ah_sbp_t%calc_grad incl. its covariant edge sync
 * (gradient/grad_ah_sbp_mod.f90:26-90) */
int swm_op_grad(swm_ctx* ctx, swm_field* gx, swm_field* gy,
                const swm_field* f);
/* div_ah_sbp_t%calc_div incl. its scalar sync (div_ah_sbp_mod.f90:24-98);
 * u, v contravariant */
int swm_op_div(swm_ctx* ctx, swm_field* div, const swm_field* u,
               const swm_field* v);
/* curl_div_based_t%calc_curl (curl/curl_div_based_mod.f90:26-66); u, v
 * covariant */
int swm_op_curl(swm_ctx* ctx, swm_field* curl, const swm_field* u,
                const swm_field* v);
/* coriolis_colocated%calc_coriolis_vec_inv (coriolis_colocated_mod.f90:61-103) */
int swm_op_coriolis(swm_ctx* ctx, swm_field* cor_u, swm_field* cor_v,
                    const swm_field* hu, const swm_field* hv,
                    const swm_field* h, const swm_field* curl);
/* C grid only: grad_perp_c_sbp21 / _sbp42 (grad_perp/grad_perp_c_sbp_mod.f90
 * :20-95) of a corner-mesh field w onto the u and v meshes, and the
 * transform2co of co2contra_c_sbp21_new / _sbp42_new (co2contra/
 * co2contra_Cgrid_mod.f90:135-203): covariant (u, v) from contravariant
 * (ut, vt), at the context's SBP order.  SWM_E_UNSUPPORTED on the Ah grid. */
int swm_op_grad_perp(swm_ctx* ctx, swm_field* gu, swm_field* gv,
                     const swm_field* w);
int swm_op_contra2co(swm_ctx* ctx, swm_field* u, swm_field* v,
                     const swm_field* ut, const swm_field* vt);
/* C grid only, on its cell-centre mesh (the A grid's points): the ECS_O
 * scalar halo (halo_t%get_halo_scalar for "ECS_O", equiang_cs/ecs_halo_mod.f90
 * :95-475 with the weights of ecs_halo_factory_mod.f90:164-196) and
 * gradient_a2_ecs (gradient/grad_a2_mod.f90:19-69: the central difference of
 * the cell values with that halo, covariant gx, gy at the centres).
 * swm_halo_ecs_o writes, synchronously, the extended tiles of halo width 1 or
 * 2 to host memory: 6 panels of (N+2hw) x (N+2hw) doubles, row-major, the
 * reference's 1-based (i, j) at row j + hw - 1, column i + hw - 1.
 * SWM_E_UNSUPPORTED on the Ah grid. */
int swm_op_grad_a2_ecs(swm_ctx* ctx, swm_field* gx, swm_field* gy,
                       const swm_field* f);
int swm_halo_ecs_o(swm_ctx* ctx, const swm_field* f, int halo_width,
                   double* ext);
/* The same for A-grid vectors (contravariant u, v on the cell centres): the
 * ecs_A_vec halo (halo_vec_t%get_halo_vector for "ecs_A_vec",
 * equiang_cs/ecs_halo_vec_a_mod.f90:34-158 with the maps of
 * ecs_halo_vec_a_factory_mod.f90:108-170; both extended tiles, laid out as
 * swm_halo_ecs_o's) and divergence_a2_ecs (divergence/div_a2_mod.f90:19-72:
 * the J-weighted central difference with that halo). */
int swm_op_div_a2_ecs(swm_ctx* ctx, swm_field* div, const swm_field* u,
                      const swm_field* v);
/* gradient_c2_ecs (gradient/grad_c2_ecs_mod.f90:33-51, 95-144): the C grid's
 * second-order gradient with the ECS_O halo; f on mesh p, gx on mesh u, gy on
 * mesh v.  C grid only. */
int swm_op_grad_c2_ecs(swm_ctx* ctx, swm_field* gx, swm_field* gy,
                       const swm_field* f);
/* C grid only, on its corner mesh (the Ah grid's nodes): the ECS_xy halo
 * (halo_t%get_halo_scalar for "ECS_xy", equiang_cs/ecs_halo_xy_mod.f90:38-217
 * with the weights of ecs_halo_factory_mod.f90:198-228; width 1..4; the
 * extended (N+1+2hw)^2 tiles to host memory as swm_halo_ecs_o writes them,
 * the panel's edge nodes synced) and laplace_ch_halo2 / laplace_ch_halo4
 * (laplace/laplace_ch_halo_mod.f90:15-179, laplace_factory_mod.f90:110-126:
 * with that halo of width 1 / 3, then the Ah scalar sync); order 2 or 4;
 * out may be in. */
int swm_halo_ecs_xy(swm_ctx* ctx, const swm_field* f, int halo_width,
                    double* ext);
int swm_laplace_ch(swm_ctx* ctx, swm_field* out, const swm_field* in, int order);
int swm_halo_ecs_a_vec(swm_ctx* ctx, const swm_field* u, const swm_field* v,
                       int halo_width, double* ext_u, double* ext_v);
/* halo_t%get_halo_scalar for "Ah_scalar_sync"
 * (halo/halo_Ah_scalar_sync_mod.f90:20-93) */
int swm_sync_scalar(swm_ctx* ctx, swm_field* f);
/* halo_vec_t%get_halo_vector for "ecs_Ah_vec_sync_covariant"
 * (equiang_cs/ecs_Ah_vec_sync_mod.f90:34-125) */
int swm_sync_vector_cov(swm_ctx* ctx, swm_field* gx, swm_field* gy);
/* quadrature_t%mass with the SBP_AhXX quadrature
 * (quadrature/abstract_quadrature_mod.f90:27-44, sbp_quadrature_mod.f90:21-40) */
int swm_quadrature_mass(swm_ctx* ctx, const swm_field* f, double* out);

/* ---------------------------------------------------------------------- */
/* Kernel timing for measurement (no reference counterpart): when enabled,  */
/* every fused-stage and cube-edge kernel launch is bracketed by CUDA       */
/* events on the context stream; swm_timing_read returns the summed time    */
/* [ms] and the number of launches of each kind since the last read.        */
/* ---------------------------------------------------------------------- */
int swm_timing_enable(swm_ctx* ctx, int on);
int swm_timing_read(swm_ctx* ctx, double* stage_ms, long* stage_launches,
                    double* edge_ms, long* edge_launches);

/* ---------------------------------------------------------------------- */
/* Tangent-linear and adjoint of the model (no counterpart in the           */
/* reference).  F is the model operator of swm_apply, Phi one RK4 step of   */
/* swm_rk4_step.  The adjoint is the exact transpose of the tangent-linear  */
/* model of the discrete operators (SBP stencils with their closures, the    */
/* cube-edge syncs, RK4) in the algebraic inner product of swm_dot.  The     */
/* tangent-linear calls need an FP64 context; the adjoint calls run in both  */
/* precisions (FP32 contexts: FP32 arithmetic, cotangents in the high part   */
/* of the state pair, low part cleared).  The first call allocates the       */
/* context's TL/AD workspace.  Arguments must be distinct states of the      */
/* context.                                                                 */
/* ---------------------------------------------------------------------- */
/* dk = F'(y) dx */
int swm_apply_tl(swm_ctx* ctx, const swm_state* y, const swm_state* dx,
                 swm_state* dk);
/* lx = F'(y)^T lk */
int swm_apply_ad(swm_ctx* ctx, const swm_state* y, const swm_state* lk,
                 swm_state* lx);
/* dx <- Phi'(x) dx */
int swm_rk4_tl(swm_ctx* ctx, const swm_state* x, swm_state* dx, double dt);
/* lx <- Phi'(x)^T lx (recomputes the stage states of x; CUDA graph) */
int swm_rk4_ad(swm_ctx* ctx, const swm_state* x, swm_state* lx, double dt);

/* Gradient through nsteps RK4 steps with binomial checkpointing: nsnap      */
/* stored states (x0 included) and recomputation by the revolve recursion.   */
typedef struct swm_adjoint swm_adjoint;
int  swm_adjoint_create(swm_ctx* ctx, int nsteps, int nsnap, double dt,
                        swm_adjoint** out);
void swm_adjoint_destroy(swm_adjoint* adj);
/* x_T = Phi^nsteps(x0), storing the first snapshots */
int  swm_adjoint_forward(swm_adjoint* adj, const swm_state* x0, swm_state* xT);
/* lambda: in dJ/dx_T, out dJ/dx0 (after swm_adjoint_forward) */
int  swm_adjoint_backward(swm_adjoint* adj, swm_state* lambda);
/* RK4 steps run by the last forward + backward, adjoint steps, and the
 * forward steps the plan needs in total */
int  swm_adjoint_counts(const swm_adjoint* adj, long* forward_steps,
                        long* adjoint_steps, long* planned_forward_steps);

/* States from/to DEVICE arrays in the host layout (framework tensors),      */
/* ordered on the context stream.                                           */
int swm_state_upload_device(swm_ctx* ctx, swm_state* s, const double* h,
                            const double* u, const double* v);
int swm_state_download_device(swm_ctx* ctx, const swm_state* s, double* h,
                              double* u, double* v);
/* SBP quadrature weight of every node (host layout), the weights of
 * swm_quadrature_mass: J hx^2 A_i A_j (sbp_quadrature_mod.f90:21-40). */
int swm_quadrature_weights(swm_ctx* ctx, double* w_host);

/* ---------------------------------------------------------------------- */
/* Ensembles (no counterpart in the reference, which runs one instance per  */
/* job): independent members, each with its own N, initial state and time   */
/* step, sharing SBP order, constants and precision.  Each member is a full */
/* context; an ensemble RK4 step is one CUDA graph with, per RK stage, one  */
/* stage-kernel launch over the work units of all members (persistent CTAs  */
/* in the FP32 form) and one edge-kernel launch.  Each member's arithmetic  */
/* is exactly that of swm_rk4_step on the member alone.                     */
/* ---------------------------------------------------------------------- */
typedef struct swm_ensemble swm_ensemble;

/* member_N[m], member_dt[m] for m < nmembers; base gives the rest. */
int  swm_ensemble_create(const swm_config* base, int nmembers,
                         const int* member_N, const double* member_dt,
                         swm_ensemble** out);
void swm_ensemble_destroy(swm_ensemble* ens);
const char* swm_ensemble_last_error(const swm_ensemble* ens);
int  swm_ensemble_size(const swm_ensemble* ens);
/* Member m's context and state (for single-instance calls on it; call
 * swm_ensemble_synchronize first). */
int  swm_ensemble_member(swm_ensemble* ens, int m, swm_ctx** ctx,
                         swm_state** state);
/* Host arrays in the layout of swm_state_upload/download (member's N). */
int  swm_ensemble_upload(swm_ensemble* ens, int m, const double* h,
                         const double* u, const double* v);
int  swm_ensemble_download(swm_ensemble* ens, int m, double* h, double* u,
                           double* v);
int  swm_ensemble_diagnostics(swm_ensemble* ens, int m, double out[7]);
/* nsteps RK4 steps of every member (asynchronous on the ensemble stream). */
int  swm_ensemble_step(swm_ensemble* ens, int nsteps);
int  swm_ensemble_synchronize(swm_ensemble* ens);
void* swm_ensemble_stream(swm_ensemble* ens);
/* Tile shape: rows per work unit (0: whole panel height) and persistent
 * CTAs of the stage kernel (0: one CTA per work unit). */
int  swm_ensemble_set_shape(swm_ensemble* ens, int seg_rows, int grid);
/* Consumer width of the members' FP32 stage kernel (64, 96, 128, 160 or 192;
 * bit-identical results); swm_ensemble_tune also searches it. */
int  swm_ensemble_set_width(swm_ensemble* ens, int cols);
int  swm_ensemble_get_width(const swm_ensemble* ens, int* cols);
int  swm_ensemble_get_shape(const swm_ensemble* ens, int* seg_rows, int* grid,
                            int* nunits);
/* Autotuner: times `steps` ensemble steps for each candidate tile shape,
 * keeps the fastest and restores the member states. */
int  swm_ensemble_tune(swm_ensemble* ens, int steps, int* seg_rows_out,
                       int* grid_out, double* ms_per_step_out);

/* ---------------------------------------------------------------------- */
/* Scalar cube-edge sync with static scratch (no counterpart in the        */
/* reference; same result as swm_sync_scalar).                             */
/*                                                                          */
/* For callers that must not have device memory allocated on their behalf: */
/* a host model that hands a fixed device budget to its own pool at        */
/* start-up, or one that cannot afford the device-wide synchronisation a   */
/* cudaMalloc/cudaFree brings.  The edge scratch is a fixed array in the   */
/* library's device image (reserved when the library's module loads), not  */
/* a buffer of the context; the call itself allocates nothing.             */
/*  - Limit: N <= SWM_SYNC_STATIC_MAX_N (scratch 6*4*4*(N+1) doubles,        */
/*    769 KiB at the limit); a larger N is rejected with SWM_E_INVALID.     */
/*  - The first call on each device looks up the scratch address on that   */
/*    device (cudaGetSymbolAddress); make that first call before any stream */
/*    capture begins.                                                        */
/*  - No scratch value has to start at zero: every slot the sync reads is   */
/*    written by the same call first.                                        */
/*  - All calls on one device share the scratch: calls that overlap in time */
/*    (different streams or contexts on the same device) race; calls on one */
/*    stream are ordered and safe.                                          */
/* ---------------------------------------------------------------------- */
#define SWM_SYNC_STATIC_MAX_N 1024
int swm_sync_scalar_static(swm_ctx* ctx, swm_field* f);

/* ---------------------------------------------------------------------- */
/* Lat-lon and paneled output                                             */
/* ---------------------------------------------------------------------- */
/* Interpolator of the Ah fields of a context to an Nlon x Nlat lat-lon grid
 * (lon = i*2pi/Nlon, lat = -pi/2 + j*pi/(Nlat-1)): create_latlon_regrid /
 * create_latlon_vector_regrid with scalar/vector grid type "Ah"
 * (regridders/regrid_factory_mod.f90:9-190, 195-299).  interp_type
 * "linear" or "cubic" (NULL: cubic, the outputers' choice);
 * components_type "covariant" or "contravariant" (NULL: covariant), the
 * meaning of the (u, v) it is given.  Outputs have Nlon*Nlat values,
 * longitude fastest; vectors come out as (east, north) components. */
int swm_latlon_create(swm_ctx* ctx, int nlon, int nlat, const char* interp_type,
                      const char* components_type, swm_latlon** out);
void swm_latlon_destroy(swm_latlon* r);
/* regrid_t%do_regrid (regrid_to_latlon_mod.f90:54-74) of an FP64 field */
int swm_latlon_regrid_field(swm_ctx* ctx, swm_latlon* r, const swm_field* f, double* out);
/* regrid_vec_t%do_regrid (regrid_to_latlon_mod.f90:76-124) of (u, v) */
int swm_latlon_regrid_vector(swm_ctx* ctx, swm_latlon* r, const swm_field* u, const swm_field* v,
                             double* uo, double* vo);
/* h and (u, v) of a state; any output may be NULL */
int swm_latlon_regrid_state(swm_ctx* ctx, swm_latlon* r, const swm_state* s, double* h, double* u,
                            double* v);
/* latlon_outputer_t%write and latlon_vec_outputer_t%write
 * (outputer/latlon_outputer_mod.f90:38-190): FP32 record rec_num (1-based)
 * of Nlon*Nlat values into direct-access files (the reference's h.dat,
 * u.dat, v.dat); a NULL or empty name skips that file. */
int swm_latlon_write(swm_ctx* ctx, swm_latlon* r, const swm_state* s, const char* h_file,
                     const char* u_file, const char* v_file, int rec_num);
/* master_paneled_outputer_t%write (outputer/master_paneled_outputer_mod.f90:
 * 24-77): FP32 record rec_num of 6*(N+1)^2 values (i fastest, then j, then
 * panel) of state component 0 (h), 1 (u) or 2 (v). */
int swm_paneled_write(swm_ctx* ctx, const swm_state* s, int component, const char* file, int rec_num);

/* ---------------------------------------------------------------------- */
/* Launch-shape tuning (no reference counterpart)                         */
/* ---------------------------------------------------------------------- */
/* The stage kernel's launch shape: the consumer width of the FP32 kernel
 * (64, 96, 128, 160 or 192 columns per CTA), the rows per work unit (0: enough
 * units for one wave of CTAs), the persistent grid (0: one CTA per unit) and
 * the box mode of the FP32 kernel's TMA loads: SWM_BOX_STRIP (the narrowest
 * box that covers every column strip, its width a kernel argument),
 * SWM_BOX_WIDEST (the width's widest box, a compile-time constant of the
 * kernel; needs a field pitch of at least that box) or SWM_BOX_AUTO (the
 * widest box where it fits and keeps the resident CTAs per SM).
 * The shape changes how the panels are split into work, not any node's
 * arithmetic (results are bit-identical).  The best shape depends on the
 * grid: swm_tune_stage times `steps` RK4 steps of dt per candidate on a copy
 * of s (s is not changed), keeps the fastest and returns it with its median
 * step time.  FP64 contexts have one width and ignore the box mode. */
#define SWM_BOX_AUTO 0
#define SWM_BOX_STRIP 1
#define SWM_BOX_WIDEST 2
int swm_tune_stage(swm_ctx* ctx, const swm_state* s, double dt, int steps, int* cols_out,
                   int* seg_rows_out, int* grid_out, int* box_out, double* ms_out);
int swm_get_stage_shape(swm_ctx* ctx, int* cols, int* seg_rows, int* grid, int* box, int* nunits);
int swm_set_stage_shape(swm_ctx* ctx, int cols, int seg_rows, int grid, int box);
/* The stage kernel's work split for a grid of N cells per panel edge and an
 * SBP order, with no device work (inspection and tests): consumer width
 * cols, the units of one wave target_units (seg_rows = 0) or seg_rows rows
 * per inner-strip unit.  Writes up to max_units units of 9 ints each (panel,
 * owned columns i0 i1, owned rows j0 j1, read columns cl0 cl1, read rows
 * rl0 rl1) to units_out and their count to *nunits; SWM_E_INVALID if the
 * split fails or max_units is too small. */
int swm_work_split(int N, int sbp_order, int cols, int target_units, int seg_rows, int* units_out,
                   int max_units, int* nunits);

/* ---------------------------------------------------------------------- */
/* Checkpoint / resume (no reference counterpart: the reference writes no   */
/* restart files)                                                          */
/* ---------------------------------------------------------------------- */
/* A state file holds a 64-byte header (magic "SWMSTATE", version 1, N, SBP
 * order, the writer's precision, the caller's model time) and the FP64
 * fields h, u, v in the reference layout (6*(N+1)^2 values each).  Loading
 * needs the same N; the precision may differ (FP32 pairs round-trip
 * exactly).  SWM_E_IO on file errors, SWM_E_INVALID on a foreign or
 * mismatched file. */
int swm_state_save(swm_ctx* ctx, const swm_state* s, const char* path, double time);
int swm_state_load(swm_ctx* ctx, swm_state* s, const char* path, double* time);

#ifdef __cplusplus
}
#endif
#endif
