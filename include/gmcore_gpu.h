/*
 * gmcore_gpu.h -- C ABI of the GB300 dynamics step for the GMCORE
 * latitude-longitude C-grid model.
 *
 * The library replaces one call of the reference model:
 *
 *   time_integrate(dt_dyn, blocks)      src/dynamics/gmcore_mod.F90:577-591
 *
 * together with the run prologue that prepares the first step
 * (src/dynamics/gmcore_mod.F90:97-135) and the conservation monitor
 * `diagnose` (src/dynamics/gmcore_mod.F90:213-341).  A Fortran host keeps
 * its namelist, initial conditions, output and restart code and calls these
 * functions through iso_c_binding (module gmcore_gpu_mod in
 * include/gmcore_gpu_mod.F90 binds every entry point).
 *
 * Conventions
 *  - Every function returns an int status: GMC_OK (0) or a negative code.
 *    A message for the last failure is available from gmc_last_error().
 *    The library never aborts the process (the reference stops through
 *    log_error / MPI_ABORT instead).  Kernels record errors in a device
 *    error word; gmc_prepare and gmc_step return the first error raised in
 *    launch order (the one at which the reference would have stopped) after
 *    all requested steps ran.
 *  - Host arrays are described by gmc_view: a base pointer plus Fortran
 *    lower/upper bounds per dimension, column-major (i fastest), so a
 *    Fortran array with halos can be passed as c_loc(a) with lbound/ubound.
 *    Only interior points are read or written; halos are left untouched.
 *  - The caller owns host memory; the library keeps no host pointer except
 *    the ranges the caller registers with gmc_host_register.
 *    The library owns device memory; model state stays resident in HBM
 *    between calls.
 *  - One host thread per context at a time.  All calls are synchronous, but
 *    for history and restart files written in the background
 *    (gmc_file_opts.background, gmc_output_wait).
 */
#ifndef GMCORE_GPU_H
#define GMCORE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GMC_OK           0
#define GMC_EINVAL      -1   /* malformed argument or unsupported option      */
#define GMC_ECFL        -2   /* |cflx| > lon halo width or |cfly| > 1 or cflz out of range
                                (adv_batch_mod.F90:284-287, 331-333, 538-601) */
#define GMC_ENONMONO    -3   /* pressure levels not monotonic (operators_mod.F90:493-500) */
#define GMC_ENEGTRACER  -4   /* negative tracer not fixable (adv_mod.F90:251-253, 290-292) */
#define GMC_ENAN        -5   /* non-finite value in the prognostic state (surface
                                pressure, potential temperature or gz, winds) */
/* -6 is not used: no kernel of the library waits on another */
#define GMC_ECUDA       -7   /* CUDA runtime error                           */
#define GMC_ENOMEM      -8   /* device allocation failed                     */
#define GMC_ESTATE      -9   /* call out of order (e.g. step before prepare) */
#define GMC_EIO        -10   /* a history or restart file could not be written or read */

/* ---- option enums (namelist strings of src/utils/namelist_mod.F90) ------ */
#define GMC_TIME_EULER    0  /* time_scheme = 'euler'  */
#define GMC_TIME_PC2      1  /* time_scheme = 'pc2'    */
#define GMC_TIME_WRFRK3   2  /* time_scheme = 'wrfrk3' */

#define GMC_PV_MIDPOINT   0  /* pv_scheme = 'midpoint' */
#define GMC_PV_UPWIND     1  /* pv_scheme = 'upwind'   */
#define GMC_PV_TVD        2  /* pv_scheme = 'tvd'      */

#define GMC_TVD_NONE      0  /* tvd_limiter_type = 'none'     */
#define GMC_TVD_VAN_LEER  1  /* tvd_limiter_type = 'van_leer' */
#define GMC_TVD_MC        2  /* tvd_limiter_type = 'mc'       */

#define GMC_FLUX_PPM      0  /* ffsl_flux_type = 'ppm'      */
#define GMC_FLUX_VAN_LEER 1  /* ffsl_flux_type = 'van_leer' */

#define GMC_LIMITER_NONE  0  /* limiter_type = 'none'  */
#define GMC_LIMITER_MONO  1  /* limiter_type = 'mono'  */
#define GMC_LIMITER_PD    2  /* limiter_type = 'pd'    */

#define GMC_VCOORD_NONE       0   /* shallow water                           */
#define GMC_VCOORD_TEST_L26  26   /* hybrid_coord_test_l26 (hybrid_coord_test_mod.F90:78)  */
#define GMC_VCOORD_WRF_L32   32   /* hybrid_coord_wrf_l32  (hybrid_coord_test_mod.F90:565) */
#define GMC_VCOORD_WRF_L64   64   /* hybrid_coord_wrf_l64  (hybrid_coord_test_mod.F90:734) */

#define GMC_FORCING_NONE         0  /* test_case without forcing                   */
#define GMC_FORCING_HELD_SUAREZ  1  /* test_case = 'held_suarez' (test_forcing_mod.F90:24-25) */

#define GMC_PREC_FP64     0  /* FP64 everywhere                               */
#define GMC_PREC_MIXED    1  /* FP32 bulk stencils/advection, FP64 pole rings,
                                column sweeps, integrals and filter weights   */

/* ---- configuration: the namelist fields the step depends on ------------- */
typedef struct gmc_config {
  int32_t nlon, nlat, nlev;        /* num_lon, num_lat (both pole rows), num_lev  */
  int32_t baroclinic;              /* 0: shallow water (nlev must be 1)          */
  int32_t time_scheme;             /* GMC_TIME_*                                 */
  double  dt_dyn;                  /* s                                          */
  double  dt_adv;                  /* s; <= 0 means dt_dyn                       */
  int32_t ke_scheme;               /* 1 or 2                                     */
  double  ke_cell_wgt;
  int32_t pv_scheme;               /* GMC_PV_*                                   */
  int32_t upwind_order_pv;         /* 1 or 3                                     */
  double  upwind_wgt_pv;
  int32_t pv_pole_stokes;          /* logical                                    */
  int32_t coriolis_scheme;         /* 1 or 2                                     */
  int32_t ffsl_flux_type;          /* GMC_FLUX_*                                 */
  int32_t limiter_type;            /* GMC_LIMITER_*                              */
  int32_t use_div_damp;            /* divergence damping after each step         */
  int32_t div_damp_order;          /* 2 or 4                                     */
  double  div_damp_coef2;          /* namelist div_damp_coef2                    */
  int32_t vert_coord_template;     /* GMC_VCOORD_*                               */
  double  ptop;                    /* Pa (namelist ptop)                         */
  double  hybrid_coord_p0;         /* Pa                                         */
  double  max_wave_speed, max_cfl; /* polar filter                               */
  double  filter_coef_a, filter_coef_b, filter_coef_c, filter_coef_d, filter_coef_e;
  int32_t lon_halo_width;          /* namelist minimum; widened by the filter    */
  int32_t ntracer;                 /* tracers of one FFSL batch (0: none)        */
  int32_t precision;               /* GMC_PREC_*                                 */
  int32_t n_members;               /* ensemble members sharing this grid         */
  double  radius, omega, g, Rd, cpd, p0;   /* const_mod.F90:51-85 ('earth')     */
  int32_t tvd_limiter_type;        /* GMC_TVD_* (pv_scheme = tvd)                */
  double  div_damp_coef4;          /* namelist div_damp_coef4 (order 4)          */
  int32_t forcing;                 /* GMC_FORCING_*: test forcing applied after the
                                      integrator, before damping (gmcore_mod.F90:586) */
  int32_t use_smag_damp;           /* namelist use_smag_damp (damp_mod.F90:59-61) */
  double  smag_damp_coef;          /* namelist smag_damp_coef                    */
} gmc_config;

/* Diagnostics of gmcore_mod.F90:213-341 (FP64, compensated sums). */
typedef struct gmc_diag {
  double tm, te, te_ke, te_ie, te_pe, tav, tpe, tpt;
} gmc_diag;

/* Host array view: data(i,j,k) = data[(i-lb0) + n0*((j-lb1) + n1*(k-lb2))],
 * n0 = ub0-lb0+1, n1 = ub1-lb1+1.  2-D fields use lb[2] = ub[2] = 1. */
typedef struct gmc_view {
  double *data;
  int32_t lb[3];
  int32_t ub[3];
} gmc_view;

typedef struct gmc_ctx gmc_ctx;

/* Fill cfg with the reference defaults (namelist_mod.F90:10-113, earth). */
void gmc_config_default(gmc_config *cfg);

/* Build mesh metrics, vertical coordinate, polar filters and device state.
 * Replaces gmcore_init's block set-up (gmcore_mod.F90:45-95). */
int gmc_create(const gmc_config *cfg, gmc_ctx **out);

/* Longitude halo width the reference would use for this configuration
 * (process_mod.F90:208-213): max(namelist width, (big-filter taps - 1)/2). */
int gmc_lon_halo_width(const gmc_ctx *ctx, int32_t *out);

/* Set one prognostic field of one member, interior points only.  Before
 * gmc_prepare this defines the initial state; afterwards it overwrites the
 * current state in place (e.g. a host that keeps its Fortran arrays and
 * hands them to every step), keeping the filtered copies and the tracer
 * batch of the previous step as the reference's state(old) would.
 * Names: "u_lon" (i=1..nlon half lon, j=1..nlat, k=1..nlev),
 *        "v_lat" (i=1..nlon, j=1..nlat-1, k=1..nlev),
 *        "pt"    (baroclinic) or "gz" (shallow water), full cells,
 *        "phs"   (baroclinic, 2-D), "gzs" (static surface geopotential, 2-D),
 *        "q"     (tracer t: pass k-range 1..nlev, tracer index via gmc_set_tracer).
 * Mirrors the assignments a set_ic routine makes (e.g.
 * tests/swm/steady_geostrophic_flow_test_mod.F90:20-67). */
int gmc_set_field(gmc_ctx *ctx, int32_t member, const char *name, const gmc_view *v);
int gmc_set_tracer(gmc_ctx *ctx, int32_t member, int32_t tracer, const gmc_view *v);

/* Run prologue: filters of u, v, phs|gz, mass-batch set-up, all-pass
 * operators_prepare (gmcore_mod.F90:97-135). */
int gmc_prepare(gmc_ctx *ctx);

/* Advance nsteps dynamics steps: time_integrate x nsteps, including tracer
 * advection (adv_run) and the old/new swap of time_advance.  Returns after
 * the device error word was checked. */
int gmc_step(gmc_ctx *ctx, int32_t nsteps);

/* Copy a field of the current (old) state to the host, interior only.
 * Names: those of gmc_set_field plus "u_f", "v_f", "phs_f", "gz_f", "m",
 * "t", "pv", "ke". */
int gmc_get_field(gmc_ctx *ctx, int32_t member, const char *name, const gmc_view *v);
int gmc_get_tracer(gmc_ctx *ctx, int32_t member, int32_t tracer, const gmc_view *v);

/* One exchange of a coupled step: the inputs set (as gmc_set_field /
 * gmc_set_tracer), nsteps steps (as gmc_step), the outputs read back (as
 * gmc_get_field / gmc_get_tracer), with the same results, status and error
 * word as those calls in that order.  An item names a field (name) or, with
 * name NULL, a tracer (tracer).  Where the host arrays lie in registered
 * ranges (gmc_host_register) with one row pitch, the transfers overlap the
 * step: tracer inputs move while the first step's dynamics run, and field
 * outputs while the last step's tracer advection runs (one-member contexts
 * with tracers); the rest move before and after the step.  No reference
 * counterpart: the field exchange a driver coupled through host arrays makes
 * around time_integrate (gmcore_mod.F90:138-139). */
typedef struct gmc_io {
  const char *name;   /* field name, or NULL for a tracer        */
  int32_t tracer;     /* tracer index when name is NULL           */
  gmc_view view;
} gmc_io;
int gmc_step_io(gmc_ctx *ctx, int32_t member, const gmc_io *in, int32_t n_in, int32_t nsteps, const gmc_io *out,
                int32_t n_out);

/* Global integrals of the current state (gmcore_mod.F90:213-341). */
int gmc_diagnose(gmc_ctx *ctx, int32_t member, gmc_diag *out);

/* Number of steps taken since gmc_prepare. */
int gmc_time_step(const gmc_ctx *ctx, int64_t *out);

/* ---- history and restart files --------------------------------------------
 * netCDF classic files (64-bit offset format, readable by any netCDF reader)
 * with the reference's dimensions (time, lon, lat, ilon, ilat, lev, ilev),
 * variable names, long names and units.  netCDF lists dimensions slowest
 * first, so the reference's u(ilon, lat, lev, time) is stored as
 * u(time, lev, lat, ilon): the library's own [k][j][i] order.
 *   restart (r0): time_step_size, u, v, phs, pt (baroclinic) or u, v, gz
 *     (shallow water), gzs, and the tracers  (restart_mod.F90:54-151; the
 *     reference's restart holds no tracers)
 *   history (h0): tm, te, tpe, te_ke, te_ie, te_pe, zs, phs, u, v, pt, t, z,
 *     ph, vor, div and the tracers (hydrostatic, history_mod.F90:194-240,
 *     519-580); tm, te, tpe, u, v, z, pv, div, zs (shallow water, :125-150,
 *     398-444).  t, z, ph, vor and div are diagnosed in FP64 on the device
 *     from the state (calc_ph, calc_t, calc_gz_lev, calc_vor, calc_div). */
typedef struct gmc_file_opts {
  const char *time_units;        /* "days", "hours", "minutes", "seconds"; NULL: "hours" */
  const char *start_time;        /* origin of the time axis; NULL: "2000-01-01 00:00:00" */
  const char *tracer_names;      /* comma-separated tracer variable names; NULL: q1, q2, ... */
  const char *restart_interval;  /* restart file attribute restart_interval; NULL: none  */
  int32_t background;            /* nonzero: gmc_history_write / gmc_restart_write copy the
                                    member's fields on the device (in stream order after the
                                    steps so far) and return; a host thread moves and writes
                                    them while the caller steps on; gmc_output_wait ends it */
} gmc_file_opts;

/* Host arrays of a restart (FP64, dense interior [k][j][i]): u_lon, v_lat,
 * pt, phs (baroclinic) or gz (shallow water), gzs, and q with the ntracer
 * tracers one after the other.  Unused pointers may be NULL; on reading, a
 * NULL destination is skipped. */
typedef struct gmc_restart_arrays {
  double *u_lon, *v_lat, *pt, *phs, *gz, *gzs, *q;
} gmc_restart_arrays;

/* Restart file of a member's state at elapsed_seconds since the start. */
int gmc_restart_write(gmc_ctx *ctx, int32_t member, const char *path, double elapsed_seconds,
                      const gmc_file_opts *opts);
/* Sets a member's state from the first record of a restart file (then
 * gmc_prepare, as restart_read precedes the run's operators_prepare) and
 * returns its time.  Tracers the file lacks are left as they are. */
int gmc_restart_read(gmc_ctx *ctx, int32_t member, const char *path, const gmc_file_opts *opts,
                     double *elapsed_seconds);
/* History record of a member's state: a new file, or with append != 0 one
 * more record of the history file at path (created when absent). */
int gmc_history_write(gmc_ctx *ctx, int32_t member, const char *path, double elapsed_seconds, int32_t append,
                      const gmc_file_opts *opts);
/* Waits for the context's background file write (gmc_file_opts.background)
 * and returns its status; GMC_OK when none is in flight.  Every file call and
 * gmc_destroy wait for it first; a failed background write is reported by the
 * next of them. */
int gmc_output_wait(gmc_ctx *ctx);
/* The same restart files from and into host arrays, without a context or a
 * GPU.  errbuf (may be NULL) receives the message of a failure. */
int gmc_restart_write_host(const gmc_config *cfg, const char *path, double elapsed_seconds, const gmc_file_opts *opts,
                           const gmc_restart_arrays *a, char *errbuf, int32_t errlen);
int gmc_restart_read_host(const gmc_config *cfg, const char *path, const gmc_file_opts *opts,
                          double *elapsed_seconds, const gmc_restart_arrays *a, char *errbuf, int32_t errlen);

/* ---- operator entry points -----------------------------------------------
 * Device pointers, interior layout [k][j][i] (i fastest), in the context's
 * precision (double for GMC_PREC_FP64, float for GMC_PREC_MIXED).  Half-
 * latitude fields have nlat-1 rows. */
typedef struct gmc_ffsl_fields {
  const void *q;                  /* advected field (cells)                       */
  const void *u, *v;              /* advecting winds (lon edges, lat edges)       */
  const void *mfx, *mfy;          /* mass fluxes of the outer operator            */
  const void *cflx, *cfly;        /* Courant numbers (lon edges, lat edges)       */
  const void *divx, *divy;        /* axis divergences (cells)                     */
  void *qmfx, *qmfy;              /* out: fluxes on lon / lat edges               */
} gmc_ffsl_fields;

/* Horizontal FFSL flux of one field (inner advective operators, intermediate
 * qx/qy, outer flux-form operators), the reference's adv_calc_tracer_hflx_cell
 * plugin (adv_mod.F90:109, ffsl_calc_tracer_hflx_cell ffsl_mod.F90:318-413).
 * Its two scratch fields are allocated from the device pool for the call. */
int gmc_ffsl_hflx(gmc_ctx *ctx, const gmc_ffsl_fields *f, double dt);

/* gmc_ffsl_hflx without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory at the
 * moment of the call -- a host model that reserved all device memory for its
 * own pool at start-up (so a cudaMalloc would fail), or a time-critical loop
 * where an allocation would synchronise the device or take an unbounded
 * time.  Its two scratch fields (the intermediates qx, qy) live in one fixed
 * 32 MiB device array compiled into the library (every GPU that loads the
 * library keeps it until the process exits), so it accepts grids with
 * 2 x nlon x nlat x nlev x sizeof(value) <= 32 MiB and returns GMC_EINVAL
 * beyond that.  The call runs on the context's stream, waits for it and
 * reads the device error word, like gmc_ffsl_hflx.  The first call on a
 * device looks up the array's device address.  All calls share the one
 * array: nothing in it needs to start at zero, and calls whose kernels
 * overlap on the GPU (two contexts on different host threads at the same
 * time) race on it.  Results equal gmc_ffsl_hflx's. */
int gmc_ffsl_hflx_noalloc(gmc_ctx *ctx, const gmc_ffsl_fields *f, double dt);

/* Tangent-linear and adjoint of nsteps model steps (the differentiation
 * path for variational data assimilation; the reference, a forward-only model, has no
 * counterpart: its closest interface is time_integrate,
 * gmcore_mod.F90:577-591, whose derivative these are).  Both start from the
 * prepared state (call right after gmc_prepare) and leave the model at step
 * nsteps, like gmc_step(nsteps).  The three views are, in order, u_lon,
 * v_lat and gz (interior bounds as for gmc_set_field).  Available for the
 * FP64 shallow-water model with one member, pv_pole_stokes on and no
 * divergence damping (GMC_EINVAL otherwise).
 *   gmc_tlm_step: dx_n = M'(x_0) dx_0, with the run prologue's filters
 *                 applied to dx_0.
 *   gmc_adjoint:  lambda_0 = M'(x_0)^T lambda_n; the step start states are
 *                 recomputed from checkpoints stored every ckpt_every steps.
 * For J(x_n), lambda_n = dJ/dx_n gives lambda_0 = dJ/dx_0. */
int gmc_tlm_step(gmc_ctx *ctx, int32_t nsteps, const gmc_view dx0[3], const gmc_view dxn[3]);
int gmc_adjoint(gmc_ctx *ctx, int32_t nsteps, int32_t ckpt_every, const gmc_view lambda_n[3],
                const gmc_view lambda_0[3]);

/* CUDA graphs for gmc_step (on by default): each distinct launch sequence
 * of a step (slot roles, tracer cadence) is captured once and replayed.
 * Results are identical either way; profiling (gmc_set_profiling) launches
 * kernels directly.  No counterpart in the reference (a host-side launch
 * mechanism). */
int gmc_set_graphs(gmc_ctx *ctx, int32_t on);

/* Page-lock and map a caller-owned host range (cudaHostRegister, mapped).
 * gmc_set_field / gmc_get_field / gmc_set_tracer / gmc_get_tracer of a view
 * whose interior rows lie inside one registered range skip the host-side
 * staging: a device kernel gathers or scatters the rows over the host link
 * and converts FP64 <-> the form's type on the GPU (same values as the staged
 * path).  The library keeps the range until gmc_host_unregister(ptr) with the
 * same ptr; the caller keeps the memory alive until then.  Ranges may not
 * overlap.  No reference counterpart: a transfer option of the same calls.
 * Returns GMC_EINVAL (null, empty or overlapping range; unknown ptr) or
 * GMC_ECUDA (registration refused). */
int gmc_host_register(void *ptr, size_t bytes);
int gmc_host_unregister(void *ptr);

/* Timing of the last gmc_step call (or of the steps of the last gmc_step_io
 * call, with its tracer outputs): device time between CUDA events recorded on
 * the context's stream around the whole call, and the number of kernels it
 * launched.  An ensemble context (n_members > 1) times its
 * launch layouts on its first steps and keeps the fastest: layout 0 launches
 * each member's kernels separately over up to 8 streams; layout G > 0 runs G
 * groups of members, each group one member-batched launch per operator on its
 * own stream.  All layouts give identical results. */
typedef struct gmc_stats {
  double step_ms;           /* device time of the last gmc_step, all steps  */
  int64_t steps;            /* steps in that call                            */
  int64_t kernel_launches;  /* kernels launched by that call                 */
  int32_t member_layout;    /* launch layout in use (see above)              */
  int32_t layout_tuned;     /* 1 once the layout is chosen                   */
} gmc_stats;
int gmc_get_stats(const gmc_ctx *ctx, gmc_stats *out);

/* Launch layout of an ensemble context (see gmc_stats): -1 times the
 * candidates on the next steps and keeps the fastest (the default), 0 or
 * G = 1, 2, 4, 8 (at most n_members) fixes it.  Results do not depend on the
 * layout.  GMC_EINVAL for a layout this context cannot run.  No reference
 * counterpart (a launch option). */
int gmc_set_member_layout(gmc_ctx *ctx, int32_t layout);

/* Per-kernel device timing: when enabled, every kernel launch is bracketed
 * by CUDA events on the context stream and its duration accumulated under
 * the kernel's name.  gmc_kernel_profile returns entry `index` (GMC_EINVAL
 * past the last one). */
int gmc_set_profiling(gmc_ctx *ctx, int32_t on);
int gmc_kernel_profile(const gmc_ctx *ctx, int32_t index, char *name, size_t name_len, double *total_ms,
                       int64_t *launches);

const char *gmc_last_error(const gmc_ctx *ctx);
void gmc_destroy(gmc_ctx *ctx);

/* ---- host-side set-up helpers (no device work) -------------------------
 * A host without the reference's Fortran initialisation can obtain the same
 * 1-D metrics and seeded synthetic initial states from these. */

/* 1-D mesh metric by name ("full_lat", "half_lat", "area_cell", "area_lon",
 * "area_lat", "area_vtx", "le_lon", "de_lon", "le_lat", "de_lat",
 * "full_f", "half_f", "full_cos_lat", "half_cos_lat", "area_subcell1", ...)
 * of mesh_mod.F90:134-447; n must equal the metric's length. */
int gmc_mesh_metric(const gmc_config *cfg, const char *name, double *out, size_t n);

/* Polar-filter tap counts per latitude row: which = 0 big, 1 small1,
 * 2 small2; lat = 0 full latitudes (nlat), 1 half latitudes (nlat-1). */
int gmc_filter_taps(const gmc_config *cfg, int32_t which, int32_t lat, int32_t *out, size_t n);

/* Seeded synthetic initial state of a benchmark configuration.
 *  kind 1: shallow water, 8000 m + degree<=8 harmonics, Gaussian hill,
 *          geostrophic winds (u, v, gz, gzs filled; phs, pt, q ignored);
 *  kind 2: dry baroclinic, 300 K + N(0, noise_k) noise, 35 m/s jet,
 *          Gaussian-blob tracers (u, v, pt, phs, gzs, q filled).
 * Arrays are interior-only, C order [k][j][i] (Fortran (i,j,k)); q is
 * [tracer][k][j][i].  A NULL pointer skips that field. */
int gmc_make_ic(const gmc_config *cfg, int32_t kind, uint64_t seed, double noise_k,
                double *u_lon, double *v_lat, double *pt_or_gz, double *phs,
                double *gzs, double *q);

/* Measured FP64 fused multiply-add throughput of the current device, in
 * TFLOP/s: independent FMA chains over every SM, timed with CUDA events (no
 * clock or other setting of the GPU is changed).  No reference counterpart:
 * it is the peak against which the FP64 form's kernels are placed. */
int gmc_fp64_fma_peak(double *tflops);
/* The same for FP32 fused multiply-adds: the peak against which the mixed
 * form's arithmetic per step is placed. */
int gmc_fp32_fma_peak(double *tflops);

#ifdef __cplusplus
}
#endif

#endif /* GMCORE_GPU_H */
