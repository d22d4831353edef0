/*
 * abi_driver.c -- drives the C-ABI (include/swm_gpu.h) the way the Fortran
 * shim (fortran/swm_gpu_shim.f90) does, from plain C: no ctypes, no Python.
 *
 *   abi_driver N ORDER PRECISION DT NSTEPS IN OUT
 *
 * IN holds h, u, v (3 * 6*(N+1)^2 doubles, the reference's tile layout).
 * The driver
 *  1. creates the context with the namelist's operator names
 *     (create_swm_gpu_operator), and states with create / create_similar;
 *  2. runs NSTEPS RK4 steps through the abstract interfaces, as rk4_gpu_t's
 *     generic path does for any operator: operator%apply, y%assign(1, v0,
 *     c dt, k), v0%update(dt/6, k1, dt/3, k2), v0%update(dt/3, k3, dt/6, k4)
 *     (rk4_mod.f90:20-42);
 *  3. runs the same steps as rk4_gpu_t's fused path (swm_rk4_step) on a copy
 *     made by copy_to (create_similar + assign_s1v1);
 *  4. takes get_diagnostics, algebraic_norm2 and algebraic_dot;
 *  5. sets the TS2 scripts' hyperdiffusion and runs one explicit Euler step
 *     both ways: apply + update_s1v1 (explicit_Eul1_mod.f90:20-30) and the
 *     fused swm_diffusion_step;
 *  6. checks two error paths: a grid that is too small and an unknown
 *     operator name;
 *  7. moves the input through swm_state_upload_async / _download_async and
 *     checks the bytes against the synchronous upload / download.
 * OUT receives, in order: the generic RK4 state, the fused RK4 state (3
 * fields each), diagnostics[7], norm2, dot(v0, v0 fused), the generic and the
 * fused diffusion-step states.  Exit status 0 on success; on an ABI error it
 * prints the library's message and exits 2; 4 if the asynchronous transfers
 * disagree with the synchronous ones.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "swm_gpu.h"

static swm_ctx* g_ctx = NULL;

static void check(int rc, const char* what) {
  if (rc != SWM_OK) {
    fprintf(stderr, "abi_driver: %s failed (%d): %s\n", what, rc, swm_last_error(g_ctx));
    exit(2);
  }
}

static void download(swm_state* s, double* buf, size_t np, const char* what) {
  check(swm_state_download(g_ctx, s, buf, buf + np, buf + 2 * np), what);
}

int main(int argc, char** argv) {
  if (argc != 8) {
    fprintf(stderr, "usage: abi_driver N ORDER PRECISION DT NSTEPS IN OUT\n");
    return 1;
  }
  const int N = atoi(argv[1]), order = atoi(argv[2]), prec = atoi(argv[3]);
  const double dt = atof(argv[4]);
  const int nsteps = atoi(argv[5]);
  char div[64], grad[64], curl[64], quad[64];
  snprintf(div, sizeof div, "divergence_ah%d_sbp", order);
  snprintf(grad, sizeof grad, "gradient_ah%d_sbp_ecs", order);
  snprintf(curl, sizeof curl, "curl_divergence_ah%d_sbp", order);
  snprintf(quad, sizeof quad, "SBP_Ah%d_quadrature", order);

  swm_config cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.N = N;
  cfg.sbp_order = order;
  cfg.radius = 6.371e6;
  cfg.grav = 9.80616;
  cfg.omega = 7.292e-5;
  cfg.rotation_axis[2] = 1.0;
  cfg.precision = prec;
  cfg.device = 0;

  /* 6. error paths first (no context) */
  {
    swm_config bad = cfg;
    swm_ctx* c = NULL;
    bad.N = 4;
    if (swm_ctx_create(&bad, &c) != SWM_E_INVALID || strlen(swm_last_error(NULL)) == 0) {
      fprintf(stderr, "abi_driver: a too-small grid was not rejected\n");
      return 3;
    }
    if (swm_ctx_create_named(&cfg, "divergence_ah42_nonsense", grad, curl, "coriolis_colocated",
                             "KE_colocated", "co2contra_colocated", "massflux_colocated", quad,
                             &c) != SWM_E_UNSUPPORTED) {
      fprintf(stderr, "abi_driver: an unknown operator name was not rejected\n");
      return 3;
    }
  }

  /* 1. context and states */
  check(swm_ctx_create_named(&cfg, div, grad, curl, "coriolis_colocated", "KE_colocated",
                             "co2contra_colocated", "massflux_colocated", quad, &g_ctx),
        "swm_ctx_create_named");
  const size_t np = swm_ctx_npts(g_ctx);
  double* in = malloc(3 * np * sizeof(double));
  double* buf = malloc(3 * np * sizeof(double));
  FILE* f = fopen(argv[6], "rb");
  if (!f || fread(in, sizeof(double), 3 * np, f) != 3 * np) {
    fprintf(stderr, "abi_driver: cannot read %s\n", argv[6]);
    return 1;
  }
  fclose(f);
  FILE* out = fopen(argv[7], "wb");
  if (!out) return 1;

  swm_state *v0, *k1, *k2, *k3, *k4, *y, *vf, *d1, *d2, *tend;
  check(swm_state_create(g_ctx, &v0), "swm_state_create");
  check(swm_state_create_similar(g_ctx, v0, &k1), "create_similar");
  check(swm_state_create_similar(g_ctx, v0, &k2), "create_similar");
  check(swm_state_create_similar(g_ctx, v0, &k3), "create_similar");
  check(swm_state_create_similar(g_ctx, v0, &k4), "create_similar");
  check(swm_state_create_similar(g_ctx, v0, &y), "create_similar");
  check(swm_state_create_similar(g_ctx, v0, &vf), "create_similar");
  check(swm_state_create_similar(g_ctx, v0, &d1), "create_similar");
  check(swm_state_create_similar(g_ctx, v0, &d2), "create_similar");
  check(swm_state_create_similar(g_ctx, v0, &tend), "create_similar");
  check(swm_state_upload(g_ctx, v0, in, in + np, in + 2 * np), "swm_state_upload");

  /* 7. asynchronous round trip against the synchronous one */
  {
    double* a = malloc(3 * np * sizeof(double));
    check(swm_state_upload_async(g_ctx, y, in, in + np, in + 2 * np), "swm_state_upload_async");
    check(swm_state_download_async(g_ctx, y, a, a + np, a + 2 * np), "swm_state_download_async");
    check(swm_assign_s1(g_ctx, y, 0.0), "assign");   /* after the call: does not reach a */
    check(swm_ctx_synchronize(g_ctx), "synchronize");
    download(v0, buf, np, "download");
    if (memcmp(a, buf, 3 * np * sizeof(double)) != 0) {
      fprintf(stderr, "abi_driver: asynchronous transfers differ from the synchronous ones\n");
      return 4;
    }
    free(a);
  }
  check(swm_assign_s1v1(g_ctx, vf, 1.0, v0), "copy_to");
  check(swm_assign_s1v1(g_ctx, d1, 1.0, v0), "copy_to");
  check(swm_assign_s1v1(g_ctx, d2, 1.0, v0), "copy_to");

  /* 2. RK4 through the abstract interfaces */
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
  /* 3. the fused step */
  check(swm_rk4_step(g_ctx, vf, dt, nsteps), "swm_rk4_step");

  download(v0, buf, np, "download");
  fwrite(buf, sizeof(double), 3 * np, out);
  download(vf, buf, np, "download");
  fwrite(buf, sizeof(double), 3 * np, out);

  /* 4. diagnostics and the algebra's reductions */
  double diag[7], nrm, dot;
  check(swm_diagnostics(g_ctx, v0, diag), "swm_diagnostics");
  check(swm_norm2(g_ctx, v0, &nrm), "swm_norm2");
  check(swm_dot(g_ctx, v0, vf, &dot), "swm_dot");
  fwrite(diag, sizeof(double), 7, out);
  fwrite(&nrm, sizeof(double), 1, out);
  fwrite(&dot, sizeof(double), 1, out);

  /* 5. one explicit Euler step of the hyperdiffusion, both ways */
  char huv[64], hh[64];
  const int narrow = order == 63 ? 63 : 42;
  snprintf(huv, sizeof huv, "hordiff_vec_xyz_Ah_sbp_%d_narrow", narrow);
  snprintf(hh, sizeof hh, "hordiff_scalar_Ah_sbp_%d_narrow", narrow);
  check(swm_diffusion_set(g_ctx, huv, 0.03, hh, 0.01), "swm_diffusion_set");
  check(swm_apply_diffusion(g_ctx, tend, d1), "swm_apply_diffusion");
  check(swm_update_s1v1(g_ctx, d1, dt, tend), "update_s1v1");
  check(swm_diffusion_step(g_ctx, d2, dt, 1), "swm_diffusion_step");
  download(d1, buf, np, "download");
  fwrite(buf, sizeof(double), 3 * np, out);
  download(d2, buf, np, "download");
  fwrite(buf, sizeof(double), 3 * np, out);
  fclose(out);

  swm_state* all[] = {v0, k1, k2, k3, k4, y, vf, d1, d2, tend};
  for (size_t i = 0; i < sizeof all / sizeof all[0]; ++i) swm_state_free(all[i]);
  check(swm_ctx_synchronize(g_ctx), "synchronize");
  swm_ctx_destroy(g_ctx);
  free(in);
  free(buf);
  return 0;
}
