/*
 * A host program in plain C over include/gmcore_gpu.h, standing in for the
 * GMCORE Fortran driver (src/drivers/gmcore_driver.F90 -> gmcore_run,
 * src/dynamics/gmcore_mod.F90:97-144): it keeps its own state arrays in the
 * reference's layout -- column-major, with longitude and latitude halos --
 * hands them to the library through gmc_view, runs the prologue and N steps,
 * reads the state back into the same halo'd arrays and calls diagnose.  The
 * time loop is that of a driver coupled through its host arrays: the arrays
 * are registered (gmc_host_register) and each step is one gmc_step_io
 * exchange that sets the state from them and reads it back into them.
 *
 *   step_driver KIND NLON NLAT NLEV DT SCHEME NTRACER PRECISION NSTEPS SEED OUT
 *
 * KIND 1: shallow water (u_lon, v_lat, gz, gzs); 2: baroclinic (u_lon, v_lat,
 * pt, phs, gzs and NTRACER tracers).  OUT receives, as float64, the interior
 * of each prognostic field in (i, j, k) order, then the tracers, then the
 * eight diagnose values.  Exit status 0 on success, else the failing call's
 * status with its message on stderr.
 */
#define _POSIX_C_SOURCE 200112L /* posix_memalign */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gmcore_gpu.h"

#define HX 3 /* longitude halo of the driver's arrays */
#define HY 2 /* latitude halo */

typedef struct {
  double *data;
  size_t bytes; /* whole pages, so that each array registers on its own */
  int lb[3], ub[3];
} Arr;

static Arr arr_new(int ni, int nj, int nk) {
  Arr a;
  a.lb[0] = 1 - HX; a.ub[0] = ni + HX;
  a.lb[1] = 1 - HY; a.ub[1] = nj + HY;
  a.lb[2] = 1;      a.ub[2] = nk;
  size_t n = (size_t)(a.ub[0] - a.lb[0] + 1) * (a.ub[1] - a.lb[1] + 1) * nk;
  a.bytes = (n * sizeof(double) + 4095) / 4096 * 4096;
  void *p = NULL;
  if (posix_memalign(&p, 4096, a.bytes) != 0) exit(7);
  a.data = (double *)p;
  for (size_t t = 0; t < n; ++t) a.data[t] = -9.99e33; /* halo fill: must never be read */
  return a;
}

static double *at(Arr *a, int i, int j, int k) {
  long n0 = a->ub[0] - a->lb[0] + 1, n1 = a->ub[1] - a->lb[1] + 1;
  return a->data + (i - a->lb[0]) + n0 * ((j - a->lb[1]) + n1 * (long)(k - a->lb[2]));
}

static gmc_view view_of(Arr *a) {
  gmc_view v;
  v.data = a->data;
  memcpy(v.lb, a->lb, sizeof v.lb);
  memcpy(v.ub, a->ub, sizeof v.ub);
  return v;
}

/* interior of a C-ordered [k][j][i] array into the halo'd array and back */
static void fill(Arr *a, const double *src, int ni, int nj, int nk) {
  for (int k = 1; k <= nk; ++k)
    for (int j = 1; j <= nj; ++j)
      for (int i = 1; i <= ni; ++i) *at(a, i, j, k) = src[((size_t)(k - 1) * nj + (j - 1)) * ni + (i - 1)];
}

static void dump(FILE *f, Arr *a, int ni, int nj, int nk) {
  for (int k = 1; k <= nk; ++k)
    for (int j = 1; j <= nj; ++j) fwrite(at(a, 1, j, k), sizeof(double), (size_t)ni, f);
}

static int check(gmc_ctx *ctx, int rc, const char *what) {
  if (rc != GMC_OK) {
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, ctx ? gmc_last_error(ctx) : "");
    exit(rc < 0 ? -rc : rc);
  }
  return rc;
}

int main(int argc, char **argv) {
  if (argc != 12) {
    fprintf(stderr, "usage: %s KIND NLON NLAT NLEV DT SCHEME NTRACER PRECISION NSTEPS SEED OUT\n", argv[0]);
    return 2;
  }
  const int kind = atoi(argv[1]), nlon = atoi(argv[2]), nlat = atoi(argv[3]), nlev = atoi(argv[4]);
  const double dt = atof(argv[5]);
  const int scheme = atoi(argv[6]), ntr = atoi(argv[7]), prec = atoi(argv[8]), nsteps = atoi(argv[9]);
  const unsigned long long seed = strtoull(argv[10], NULL, 10);
  const int bc = kind == 2;

  gmc_config cfg;
  gmc_config_default(&cfg);
  cfg.nlon = nlon; cfg.nlat = nlat; cfg.nlev = nlev;
  cfg.baroclinic = bc;
  cfg.dt_dyn = dt;
  cfg.time_scheme = scheme;
  cfg.precision = prec;
  cfg.ntracer = bc ? ntr : 0;
  if (bc) {
    cfg.vert_coord_template = nlev;
    cfg.max_wave_speed = 400.0;
  }

  /* the seeded initial state, interior-only, C order */
  const size_t nf = (size_t)nlon * nlat * nlev, nh = (size_t)nlon * (nlat - 1) * nlev, n2 = (size_t)nlon * nlat;
  double *u = calloc(nf, 8), *v = calloc(nh, 8), *gzs = calloc(n2, 8);
  double *third = calloc(bc ? nf : n2, 8), *phs = bc ? calloc(n2, 8) : NULL;
  double *q = (bc && ntr > 0) ? calloc((size_t)ntr * nf, 8) : NULL;
  check(NULL, gmc_make_ic(&cfg, kind, seed, 1.0, u, v, third, phs, gzs, q), "gmc_make_ic");

  Arr A_u = arr_new(nlon, nlat, nlev), A_v = arr_new(nlon, nlat - 1, nlev), A_gzs = arr_new(nlon, nlat, 1);
  Arr A_t = arr_new(nlon, nlat, bc ? nlev : 1), A_phs = arr_new(nlon, nlat, 1);
  fill(&A_u, u, nlon, nlat, nlev);
  fill(&A_v, v, nlon, nlat - 1, nlev);
  fill(&A_gzs, gzs, nlon, nlat, 1);
  fill(&A_t, third, nlon, nlat, bc ? nlev : 1);
  if (bc) fill(&A_phs, phs, nlon, nlat, 1);

  gmc_ctx *ctx = NULL;
  int rc = gmc_create(&cfg, &ctx);
  if (rc != GMC_OK) check(ctx, rc, "gmc_create");

  gmc_view vu = view_of(&A_u), vv = view_of(&A_v), vz = view_of(&A_gzs), vt = view_of(&A_t), vp = view_of(&A_phs);
  check(ctx, gmc_set_field(ctx, 0, "u_lon", &vu), "gmc_set_field u_lon");
  check(ctx, gmc_set_field(ctx, 0, "v_lat", &vv), "gmc_set_field v_lat");
  check(ctx, gmc_set_field(ctx, 0, "gzs", &vz), "gmc_set_field gzs");
  check(ctx, gmc_set_field(ctx, 0, bc ? "pt" : "gz", &vt), "gmc_set_field pt|gz");
  if (bc) check(ctx, gmc_set_field(ctx, 0, "phs", &vp), "gmc_set_field phs");
  Arr *A_q = NULL;
  if (bc && ntr > 0) {
    A_q = malloc(sizeof(Arr) * ntr);
    for (int l = 0; l < ntr; ++l) {
      A_q[l] = arr_new(nlon, nlat, nlev);
      fill(&A_q[l], q + (size_t)l * nf, nlon, nlat, nlev);
      gmc_view vq = view_of(&A_q[l]);
      check(ctx, gmc_set_tracer(ctx, 0, l, &vq), "gmc_set_tracer");
    }
  }

  /* a wrong call is refused with a status, not an abort */
  if (gmc_step(ctx, -1) != GMC_EINVAL) {
    fprintf(stderr, "gmc_step(-1) was not refused\n");
    return 3;
  }

  check(ctx, gmc_prepare(ctx), "gmc_prepare");
  /* the driver's time loop: one exchange per step through the registered arrays */
  gmc_io io[16];
  int nio = 0;
  const char *names[4] = {"u_lon", "v_lat", bc ? "pt" : "gz", "phs"};
  Arr *arrs[4] = {&A_u, &A_v, &A_t, &A_phs};
  for (int f = 0; f < (bc ? 4 : 3); ++f) {
    check(ctx, gmc_host_register(arrs[f]->data, arrs[f]->bytes), "gmc_host_register");
    io[nio].name = names[f];
    io[nio].tracer = -1;
    io[nio].view = view_of(arrs[f]);
    ++nio;
  }
  for (int l = 0; bc && l < ntr; ++l) {
    check(ctx, gmc_host_register(A_q[l].data, A_q[l].bytes), "gmc_host_register");
    io[nio].name = NULL;
    io[nio].tracer = l;
    io[nio].view = view_of(&A_q[l]);
    ++nio;
  }
  for (int s = 0; s < nsteps; ++s) check(ctx, gmc_step_io(ctx, 0, io, nio, 1, io, nio), "gmc_step_io");
  int64_t ts = -1;
  check(ctx, gmc_time_step(ctx, &ts), "gmc_time_step");
  if (ts != nsteps) {
    fprintf(stderr, "time step %lld after %d steps\n", (long long)ts, nsteps);
    return 4;
  }

  check(ctx, gmc_get_field(ctx, 0, "u_lon", &vu), "gmc_get_field u_lon");
  check(ctx, gmc_get_field(ctx, 0, "v_lat", &vv), "gmc_get_field v_lat");
  check(ctx, gmc_get_field(ctx, 0, bc ? "pt" : "gz", &vt), "gmc_get_field pt|gz");
  if (bc) check(ctx, gmc_get_field(ctx, 0, "phs", &vp), "gmc_get_field phs");
  for (int l = 0; bc && l < ntr; ++l) {
    gmc_view vq = view_of(&A_q[l]);
    check(ctx, gmc_get_tracer(ctx, 0, l, &vq), "gmc_get_tracer");
  }
  /* the halos the library must not touch */
  if (*at(&A_u, 1 - HX, 1 - HY, 1) != -9.99e33 || *at(&A_u, nlon + HX, nlat + HY, nlev) != -9.99e33) {
    fprintf(stderr, "a halo point of u_lon was written\n");
    return 5;
  }
  gmc_diag d;
  check(ctx, gmc_diagnose(ctx, 0, &d), "gmc_diagnose");
  for (int f = 0; f < (bc ? 4 : 3); ++f) check(ctx, gmc_host_unregister(arrs[f]->data), "gmc_host_unregister");
  for (int l = 0; bc && l < ntr; ++l) check(ctx, gmc_host_unregister(A_q[l].data), "gmc_host_unregister");

  FILE *f = fopen(argv[11], "wb");
  if (!f) {
    perror(argv[11]);
    return 6;
  }
  dump(f, &A_u, nlon, nlat, nlev);
  dump(f, &A_v, nlon, nlat - 1, nlev);
  dump(f, &A_t, nlon, nlat, bc ? nlev : 1);
  if (bc) dump(f, &A_phs, nlon, nlat, 1);
  for (int l = 0; bc && l < ntr; ++l) dump(f, &A_q[l], nlon, nlat, nlev);
  const double dv[8] = {d.tm, d.te, d.te_ke, d.te_ie, d.te_pe, d.tav, d.tpe, d.tpt};
  fwrite(dv, sizeof(double), 8, f);
  fclose(f);
  /* history (in the background, overlapping one more exchange-free call) and
   * restart files of the final state: OUT.h0.nc, OUT.r0.nc */
  char path[4096];
  const double elapsed = dt * nsteps;
  gmc_file_opts fo = {"hours", "2000-01-01 00:00:00", NULL, "1 days", 1};
  snprintf(path, sizeof path, "%s.h0.nc", argv[11]);
  check(ctx, gmc_history_write(ctx, 0, path, elapsed, 0, &fo), "gmc_history_write");
  check(ctx, gmc_output_wait(ctx), "gmc_output_wait");
  fo.background = 0;
  snprintf(path, sizeof path, "%s.r0.nc", argv[11]);
  check(ctx, gmc_restart_write(ctx, 0, path, elapsed, &fo), "gmc_restart_write");
  gmc_destroy(ctx);
  printf("step_driver ok: %d steps\n", nsteps);
  return 0;
}
