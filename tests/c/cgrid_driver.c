/*
 * cgrid_driver.c -- drives the C-grid family through the C-ABI
 * (include/swm_gpu.h) from plain C, as a Fortran driver configured with the
 * &shallow_water_model_c namelist would through the shim.
 *
 *   cgrid_driver N ORDER PRECISION DT NSTEPS IN OUT
 *
 * IN holds h (6 N N), u (6 N (N+1)) and v (6 (N+1) N) doubles: per panel the
 * reference tile p(1:nx, 1:ny, 1), i fastest.  The driver
 *  1. creates the context with the namelist's C-grid operator names and
 *     checks the staggering and the mesh shapes (swm_ctx_grid,
 *     swm_mesh_dims);
 *  2. runs NSTEPS RK4 steps through the abstract interfaces (operator%apply,
 *     stvec assign / update, rk4_mod.f90:20-42) and the same steps fused
 *     (swm_rk4_step) on a copy;
 *  3. computes the curl of the input velocity on a corner-mesh field and the
 *     SBP_C mass of the input h;
 *  4. checks three refusals: a mixed-order operator set, the diagnostics
 *     (an Ah-grid entry point) and an Ah-grid hyperdiffusion name;
 *  5. configures the namelist's hyperdiffusion (hordiff_c_biharm_curl_div
 *     and hordiff_scalar_C, coefficients 0.03) and runs NSTEPS of the
 *     drivers' step (RK4, then the explicit Euler diffusion step) on the
 *     input state.
 * OUT receives the generic state, the fused state, the curl field
 * (6 (N+1)^2), the mass and the state of step 5.  Exit status 0 on success,
 * 2 on an ABI error, 3 on a wrong shape or a refusal that did not happen.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "swm_gpu.h"

static swm_ctx* g_ctx = NULL;

static void check(int rc, const char* what) {
  if (rc != SWM_OK) {
    fprintf(stderr, "cgrid_driver: %s failed (%d): %s\n", what, rc, swm_last_error(g_ctx));
    exit(2);
  }
}

int main(int argc, char** argv) {
  if (argc != 8) {
    fprintf(stderr, "usage: cgrid_driver N ORDER PRECISION DT NSTEPS IN OUT\n");
    return 1;
  }
  const int N = atoi(argv[1]), order = atoi(argv[2]), prec = atoi(argv[3]);
  const double dt = atof(argv[4]);
  const int nsteps = atoi(argv[5]);
  char nm[8][64];
  snprintf(nm[0], 64, "divergence_c_sbp%d", order);
  snprintf(nm[1], 64, "gradient_c_sbp%d", order);
  snprintf(nm[2], 64, "curl_c_sbp%d", order);
  snprintf(nm[3], 64, "coriolis_Cgrid_sbp%d", order);
  snprintf(nm[4], 64, "KE_Cgrid_sbp%d", order);
  snprintf(nm[5], 64, "co2contra_c_sbp%d", order);
  snprintf(nm[6], 64, "massflux_c_sbp%d", order);
  snprintf(nm[7], 64, "SBP_C%d_quadrature", order);
  swm_config cfg = {N, order, 6.371e6, 9.80616, 7.292e-5, {0.0, 0.0, 1.0}, prec, 0};

  /* 4a. a mixed-order set is refused before any device work */
  {
    swm_ctx* bad = NULL;
    const char* other = order == 42 ? "curl_c_sbp21" : "curl_c_sbp42";
    if (swm_ctx_create_named(&cfg, nm[0], nm[1], other, nm[3], nm[4], nm[5], nm[6], nm[7], &bad) !=
        SWM_E_UNSUPPORTED) {
      fprintf(stderr, "cgrid_driver: a mixed-order operator set was accepted\n");
      return 3;
    }
  }
  /* 1. context and shapes */
  check(swm_ctx_create_named(&cfg, nm[0], nm[1], nm[2], nm[3], nm[4], nm[5], nm[6], nm[7], &g_ctx),
        "swm_ctx_create_named");
  if (swm_ctx_grid(g_ctx) != SWM_GRID_C) {
    fprintf(stderr, "cgrid_driver: the context is not on the C grid\n");
    return 3;
  }
  int nx[4], ny[4];
  for (int m = 0; m < 4; ++m) check(swm_mesh_dims(g_ctx, m, &nx[m], &ny[m]), "swm_mesh_dims");
  if (nx[SWM_MESH_P] != N || ny[SWM_MESH_P] != N || nx[SWM_MESH_U] != N + 1 || ny[SWM_MESH_U] != N ||
      nx[SWM_MESH_V] != N || ny[SWM_MESH_V] != N + 1 || nx[SWM_MESH_Q] != N + 1 || ny[SWM_MESH_Q] != N + 1) {
    fprintf(stderr, "cgrid_driver: unexpected mesh shapes\n");
    return 3;
  }
  const size_t np = (size_t)6 * N * N, nu = (size_t)6 * (N + 1) * N, nq = (size_t)6 * (N + 1) * (N + 1);
  const size_t ns = np + 2 * nu;
  double* in = malloc(ns * sizeof(double));
  double* out = malloc((3 * ns + nq + 1) * sizeof(double));
  FILE* f = fopen(argv[6], "rb");
  if (!f || fread(in, sizeof(double), ns, f) != ns) {
    fprintf(stderr, "cgrid_driver: cannot read %s\n", argv[6]);
    return 1;
  }
  fclose(f);
  const double *h = in, *u = in + np, *v = in + np + nu;

  swm_state *v0, *vf, *k1, *k2, *k3, *k4, *y;
  check(swm_state_create(g_ctx, &v0), "swm_state_create");
  swm_state** sim[] = {&vf, &k1, &k2, &k3, &k4, &y};
  for (int k = 0; k < 6; ++k) check(swm_state_create_similar(g_ctx, v0, sim[k]), "create_similar");
  check(swm_state_upload(g_ctx, v0, h, u, v), "swm_state_upload");
  check(swm_assign_s1v1(g_ctx, vf, 1.0, v0), "copy_to");

  /* 2. RK4 through the abstract interfaces, then the fused step */
  for (int s = 0; s < nsteps; ++s) {
    check(swm_apply(g_ctx, k1, v0), "apply");
    check(swm_assign_s1v1s2v2(g_ctx, y, 1.0, v0, 0.5 * dt, k1), "assign");
    check(swm_apply(g_ctx, k2, y), "apply");
    check(swm_assign_s1v1s2v2(g_ctx, y, 1.0, v0, 0.5 * dt, k2), "assign");
    check(swm_apply(g_ctx, k3, y), "apply");
    check(swm_assign_s1v1s2v2(g_ctx, y, 1.0, v0, dt, k3), "assign");
    check(swm_apply(g_ctx, k4, y), "apply");
    check(swm_update_s1v1s2v2(g_ctx, v0, dt / 6.0, k1, dt / 3.0, k2), "update");
    check(swm_update_s1v1s2v2(g_ctx, v0, dt / 3.0, k3, dt / 6.0, k4), "update");
  }
  check(swm_rk4_step(g_ctx, vf, dt, nsteps), "swm_rk4_step");
  check(swm_state_download(g_ctx, v0, out, out + np, out + np + nu), "download");
  check(swm_state_download(g_ctx, vf, out + ns, out + ns + np, out + ns + np + nu), "download");

  /* 3. single operators on mesh fields */
  swm_field *fu, *fv, *fc, *fh;
  check(swm_field_create_mesh(g_ctx, SWM_MESH_U, &fu), "field u");
  check(swm_field_create_mesh(g_ctx, SWM_MESH_V, &fv), "field v");
  check(swm_field_create_mesh(g_ctx, SWM_MESH_Q, &fc), "field q");
  check(swm_field_create_mesh(g_ctx, SWM_MESH_P, &fh), "field p");
  check(swm_field_upload(g_ctx, fu, u), "upload u");
  check(swm_field_upload(g_ctx, fv, v), "upload v");
  check(swm_field_upload(g_ctx, fh, h), "upload h");
  check(swm_op_curl(g_ctx, fc, fu, fv), "swm_op_curl");
  check(swm_field_download(g_ctx, fc, out + 2 * ns), "download curl");
  check(swm_quadrature_mass(g_ctx, fh, out + 2 * ns + nq), "swm_quadrature_mass");

  /* 4b. an Ah-grid entry point is refused on the C grid */
  {
    double d[7];
    if (swm_diagnostics(g_ctx, v0, d) != SWM_E_UNSUPPORTED) {
      fprintf(stderr, "cgrid_driver: swm_diagnostics was not refused on the C grid\n");
      return 3;
    }
  }
  /* 4c, 5. the hyperdiffusion of &shallow_water_model_c */
  if (swm_diffusion_set(g_ctx, "hordiff_vec_xyz_Ah_sbp_42_narrow", 0.03, "hordiff_scalar_C", 0.03) !=
      SWM_E_UNSUPPORTED) {
    fprintf(stderr, "cgrid_driver: an Ah-grid hyperdiffusion name was accepted\n");
    return 3;
  }
  check(swm_diffusion_set(g_ctx, "hordiff_c_biharm_curl_div", 0.03, "hordiff_scalar_C", 0.03),
        "swm_diffusion_set");
  check(swm_state_upload(g_ctx, y, h, u, v), "swm_state_upload");
  check(swm_model_step(g_ctx, y, dt, nsteps), "swm_model_step");
  double* md = out + 2 * ns + nq + 1;
  check(swm_state_download(g_ctx, y, md, md + np, md + np + nu), "download");

  swm_field_free(fu); swm_field_free(fv); swm_field_free(fc); swm_field_free(fh);
  swm_state_free(v0); swm_state_free(vf);
  for (int k = 1; k < 6; ++k) swm_state_free(*sim[k]);
  swm_ctx_destroy(g_ctx);

  f = fopen(argv[7], "wb");
  if (!f || fwrite(out, sizeof(double), 3 * ns + nq + 1, f) != 3 * ns + nq + 1) {
    fprintf(stderr, "cgrid_driver: cannot write %s\n", argv[7]);
    return 1;
  }
  fclose(f);
  free(in);
  free(out);
  return 0;
}
