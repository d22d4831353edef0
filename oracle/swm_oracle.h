/*
 * swm_oracle.h -- C interface of the FP64 CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is a plain C++ restatement of the
 * reference's shallow-water hot path (vvshashkin/cubedsphere_sbp_swm, Fortran).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it, and only as the checker or as the timed CPU baseline.  The product
 * path (cubedsphere_sbp_swm_gb300) never links, loads or calls it.
 *
 * Layout of every field passed through this interface: 6 panels, each panel
 * (N+1) x (N+1) FP64 nodes, i (alpha direction) fastest, then j, then panel:
 *     index(p, i, j) = p*(N+1)*(N+1) + j*(N+1) + i      (all 0-based)
 * which is the reference's per-tile array p(1:N+1, 1:N+1, 1) with one tile per
 * panel (parallel/partition_mod.f90:69-95), flattened panel after panel.
 *
 * Parity pins: orc_golden_* reproduce the reference's own known-answer test
 * src/test/test_diff_ops/test_diffops_mod.f90 (test_div 71-125, test_grad
 * 127-178, test_curl 466-522, test_co2contra 231-278, test_contra2co 279-324)
 * whose printed values are checked in at src/test/test_diff_ops/
 * reference_results.txt.
 */
#ifndef SWM_ORACLE_H
#define SWM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_domain orc_domain;

/* sbp_order: 21, 42, 43 or 63 (names d21/d42/d43/d63 of
 * differential_operators/sbp_operators/sbp_factory_mod.f90:38-179).
 * radius/omega/axis as config_metric_t (metric/config_metric_mod.f90:7-63);
 * the axis is normalised as config_metric_mod.f90:57 does. */
orc_domain* orc_create(int N, int sbp_order, double radius, double grav,
                       double omega, const double axis[3]);
void orc_destroy(orc_domain* d);
int  orc_npts(const orc_domain* d);          /* 6*(N+1)^2 */
void orc_set_threads(int nthreads);           /* OpenMP threads (CPU baseline) */
int  orc_get_threads(void);

/* Geometry export (mesh_factory_mod.f90:85-133, coriolis_factory_mod.f90:151-172). */
void orc_geometry(const orc_domain* d, double* J, double* Qi1, double* Qi2,
                  double* Qi3, double* f, double* rx, double* ry, double* rz);
/* Covariant basis a1,a2 and contravariant basis b1,b2 (3 comps each, xyz
 * interleaved per node: out[3*node + c]). */
void orc_bases(const orc_domain* d, double* a1, double* a2, double* b1,
               double* b2);
/* Edge-sync weights qb, qt, ql, qr (n each), covariant case
 * (equiang_cs/ecs_Ah_vec_sync_factory_mod.f90:97-144). */
void orc_sync_weights(const orc_domain* d, double* qb, double* qt, double* ql,
                      double* qr);

/* Single-field operators, each including its cube-edge sync. */
void orc_co2contra(const orc_domain* d, const double* u, const double* v,
                   double* ut, double* vt);
void orc_contra2co(const orc_domain* d, const double* ut, const double* vt,
                   double* u, double* v);
void orc_grad(const orc_domain* d, const double* f, double* gx, double* gy);
void orc_div(const orc_domain* d, const double* u, const double* v, double* div);
void orc_curl(const orc_domain* d, const double* u, const double* v, double* curl);
void orc_sync_scalar(const orc_domain* d, double* f);
void orc_sync_vector_cov(const orc_domain* d, double* gx, double* gy);
void orc_coriolis(const orc_domain* d, const double* hu, const double* hv,
                  const double* h, const double* curl, double* cor_u,
                  double* cor_v);

/* Model operator, RK4 and diagnostics.  hs (orography) may be NULL (zero). */
void orc_apply(const orc_domain* d, const double* hs, const double* h,
               const double* u, const double* v, double* th, double* tu,
               double* tv);
void orc_rk4(const orc_domain* d, const double* hs, double* h, double* u,
             double* v, double dt, int nsteps);
/* out[7] = hmin, hmax, mass, TE, KE, PE, Enstrophy (operator_swm_mod.f90:115-155) */
void orc_diagnostics(const orc_domain* d, const double* hs, const double* h,
                     const double* u, const double* v, double out[7]);
/* Hyperdiffusion (operator_swm_diff_mod.f90:25-46): narrow = 21, 42 or 63
 * picks laplace_ah_sbp21_narrow / _sbp42_narrow / _sbp63_narrow; coefficients as the
 * namelist's uv_diff_coeff / h_diff_coeff.  Return 0, or -1 for a bad order
 * or a grid too small for the closures. */
int orc_laplace(const orc_domain* d, int narrow, const double* f, double* out);
int orc_hordiff_scalar(const orc_domain* d, int narrow, double coeff, const double* f,
                       double* out);
int orc_hordiff_vec_xyz(const orc_domain* d, int narrow, double coeff, const double* u,
                        const double* v, double* ut, double* vt);
int orc_diffusion_apply(const orc_domain* d, int uv_narrow, double uv_coeff, int h_narrow,
                        double h_coeff, const double* h, const double* u, const double* v,
                        double* th, double* tu, double* tv);
/* explicit_Eul1 step (explicit_Eul1_mod.f90:20-30) of the diffusion operator */
int orc_diffusion_step(const orc_domain* d, int uv_narrow, double uv_coeff, int h_narrow,
                       double h_coeff, double* h, double* u, double* v, double dt);
/* Lat-lon regrid of Ah fields (regridders/regrid_factory_mod.f90,
 * regrid_to_latlon_mod.f90): width 2 linear, 4 cubic; Nlon*Nlat outputs,
 * longitude fastest, lat = -pi/2 .. pi/2. */
int orc_latlon_scalar(const orc_domain* d, int nlon, int nlat, int width, const double* f,
                      double* out);
int orc_latlon_vector(const orc_domain* d, int nlon, int nlat, int width, int contravariant,
                      const double* u, const double* v, double* uo, double* vo);
/* test_regrid_mod.f90 known-answer values on the Ah grid at N=32: kind 0
 * scalar, 1 covariant vector, 2 contravariant vector. */
int orc_golden_regrid(int kind, int width, double out[2]);
double orc_l2norm(const orc_domain* d, const double* f);   /* vec_math_mod.f90:50-90 */
double orc_mass(const orc_domain* d, const double* f);     /* SBP quadrature */

/* Analytic fields of the known-answer tests (test_fields/test_fields_mod.f90):
 * vector kinds 0 solid rotation (axis cycles with level), 1 cross-polar flow,
 * 2 gradient of x/y/z (cycles with level), 3 curl-free VSH; contravariant
 * selects b1/b2 components, else a1/a2.  Scalar kinds 10 x/y/z (cycles),
 * 11 cross-polar divergence, 12 cross-polar vorticity.  Returns 0 or -1. */
int orc_vector_test_field(const orc_domain* d, int kind, int level,
                          int contravariant, double* u, double* v);
int orc_scalar_test_field(const orc_domain* d, int kind, int level, double* f);

/* Known-answer tests at (N, nz=3, unit sphere); out receives the values
 * printed by the reference test (4 for div/curl, 2 for grad/co2contra). */
int orc_golden_div(int N, int sbp_order, double out[4]);
int orc_golden_grad(int N, int sbp_order, double out[2]);
int orc_golden_curl(int N, int sbp_order, double out[4]);
int orc_golden_co2contra(int N, double out[2]);
int orc_golden_contra2co(int N, double out[2]);
/* test_coriolis / test_KE of the colocated operators on the A grid */
int orc_golden_coriolis(int N, double out[2]);
int orc_golden_ke(int N, double out[4]);
/* SBP quadrature exactness (test_quadrature_mod.f90:18-80): returns the
 * largest |exact - numeric| over orders 0..max_order at N. */
double orc_golden_quadrature(int N, int sbp_order, int max_order);
/* RK4 amplification test (test_time_steping/test_ts_mod.f90:7-73). */
double orc_golden_rk4_iomega(void);

/* ---- C grid (swm_oracle_c.cpp): the &shallow_water_model_c operator family
 * (namelist_swm:80-102), sbp_order 21 or 42, one tile per panel.  Meshes:
 * 0 p (cell centres, N x N per panel), 1 u (x-faces, (N+1) x N), 2 v
 * (y-faces, N x (N+1)), 3 q (corners, (N+1) x (N+1)); dense FP64, i fastest,
 * then j, then panel.  h on p, covariant u on u, v on v, curl on q. */
typedef struct orcc_domain orcc_domain;
orcc_domain* orcc_create(int N, int sbp_order, double radius, double grav,
                         double omega, const double axis[3]);
void orcc_destroy(orcc_domain* d);
int  orcc_size(const orcc_domain* d, int mesh);   /* points of a mesh, 6 panels */
void orcc_points(const orcc_domain* d, int mesh, double* x, double* y, double* z);
void orcc_metric(const orcc_domain* d, int mesh, double* J, double* Qi1,
                 double* Qi2, double* Qi3, double* f);
void orcc_bases(const orcc_domain* d, int mesh, double* a1, double* a2,
                double* b1, double* b2);
void orcc_co2contra(const orcc_domain* d, const double* u, const double* v,
                    double* ut, double* vt);
void orcc_massflux(const orcc_domain* d, const double* h, const double* ut,
                   const double* vt, double* hu, double* hv);
void orcc_ke(const orcc_domain* d, const double* u, const double* v,
             const double* ut, const double* vt, double* ke);
void orcc_grad(const orcc_domain* d, const double* f, double* gx, double* gy);
void orcc_div(const orcc_domain* d, const double* hu, const double* hv, double* out);
void orcc_curl(const orcc_domain* d, const double* u, const double* v, double* out);
void orcc_coriolis(const orcc_domain* d, const double* hu, const double* hv,
                   const double* h, const double* curl, double* cor_u, double* cor_v);
void orcc_apply(const orcc_domain* d, const double* hs, const double* h,
                const double* u, const double* v, double* th, double* tu, double* tv);
void orcc_rk4(const orcc_domain* d, const double* hs, double* h, double* u,
              double* v, double dt, int nsteps);
/* grad_perp_c_sbp{21,42} of a corner field (u on mesh u, v on mesh v) and the
 * transform2co of co2contra_c_sbp{21,42}_new, at the domain's SBP order. */
void orcc_grad_perp(const orcc_domain* d, const double* w, double* gu, double* gv);
void orcc_contra2co(const orcc_domain* d, const double* ut, const double* vt,
                    double* u, double* v);
/* C-grid hyperdiffusion tendency with the 2/1 operators at any domain order:
 * parts 1 hordiff_c_biharm_div, 2 hordiff_c_biharm_curl, 3
 * hordiff_c_biharm_curl_div for (u, v); hordiff_scalar_C for h. */
void orcc_hordiff(const orcc_domain* d, int parts, double uv_coeff, double h_coeff,
                  const double* h, const double* u, const double* v,
                  double* th, double* tu, double* tv);
/* nsteps of the drivers' step: one RK4 step, then one explicit Euler step of
 * the hyperdiffusion. */
void orcc_model_step(const orcc_domain* d, const double* hs, double* h, double* u,
                     double* v, double dt, int nsteps, int parts, double uv_coeff,
                     double h_coeff);
/* The ECS_O scalar halo (create_halo_procedure "ECS_O") of a cell-centre
 * field, width 1 or 2: ext receives per panel the extended (N+2hw)^2 tile,
 * row-major; returns 0 or -1.  gradient_a2_ecs: its central-difference
 * gradient at the cell centres (the A grid's points). */
int orcc_ecs_o_halo(const orcc_domain* d, const double* f, int halo_width, double* ext);
void orcc_grad_a2_ecs(const orcc_domain* d, const double* f, double* gx, double* gy);
/* The ecs_A_vec halo of contravariant (u, v) at the cell centres (width 1 or
 * 2, the same layout as orcc_ecs_o_halo) and divergence_a2_ecs. */
int orcc_ecs_a_vec_halo(const orcc_domain* d, const double* u, const double* v, int halo_width,
                        double* eu, double* ev);
void orcc_div_a2_ecs(const orcc_domain* d, const double* u, const double* v, double* out);
/* gradient_c2_ecs: the ECS_O halo of width 1, then first differences of the
 * cell values onto the faces (gx on mesh u, gy on mesh v). */
void orcc_grad_c2_ecs(const orcc_domain* d, const double* f, double* gx, double* gy);
/* The ECS_xy halo of a corner (node) mesh field, width 1..4: per panel the
 * extended (N+1+2hw)^2 tile, row-major; returns 0 or -1.  laplace_ch_halo2 /
 * laplace_ch_halo4 (order 2 / 4) of a corner-mesh field, edge-synced. */
int orcc_ecs_xy_halo(const orcc_domain* d, const double* f, int halo_width, double* ext);
int orcc_laplace_ch(const orcc_domain* d, int order, const double* f, double* out);
double orcc_mass(const orcc_domain* d, int mesh, const double* f);
double orcc_l2norm(const orcc_domain* d, int mesh, const double* f);
/* Analytic test fields on the C meshes: vector kinds 0 solid rotation (axis
 * cycles with level), 1 cross-polar, 2 gradient of x/y/z, 3 curl-free VSH (u
 * on mesh u, v on mesh v); scalar kinds 10 x/y/z, 11 cross-polar divergence,
 * 12 cross-polar vorticity on the given mesh.  Return 0 or -1. */
int orcc_vector_test_field(const orcc_domain* d, int kind, int level,
                           int contravariant, double* u, double* v);
int orcc_scalar_test_field(const orcc_domain* d, int kind, int level, int mesh,
                           double* f);
/* Known-answer tests on the C grid at (N, nz=3, unit sphere): kind 0 div (4
 * values), 1 grad (2), 2 curl (4), 3 Coriolis (2), 4 KE (4), 5 co2contra (2),
 * 6 contra2co of co2contra_c_sbp*_new (2), 7 gradient_a2_ecs (2), 8
 * divergence_a2_ecs (4), 9 gradient_c2_ecs (2).
 * Returns 0, or -1 for an unknown kind / order. */
int orcc_golden(int kind, int N, int sbp_order, double* out);

#ifdef __cplusplus
}
#endif
#endif
