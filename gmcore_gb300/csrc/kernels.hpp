// Host-visible launchers of the device kernels and the pointer bundles they
// operate on.  R is the storage/arithmetic type of the bulk 3-D fields
// (double for the FP64 form, float for the mixed form); the FP64-only pieces
// (surface pressure, column sweeps, pole rings, diagnostics) are double.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace gmc {

// Fields of one state slot (one of the reference's state(1:3)).
template <class R>
struct Slot {
  R *u_lon, *v_lat, *u_f, *v_f;     // wind on its edges and filtered wind
  R *pt;                             // baroclinic potential temperature
  R *gz, *gz_f;                      // shallow-water geopotential
  double *phs, *phs_f;               // surface pressure (baroclinic)
  R *mfx_lon, *mfy_lat;              // mass fluxes of the last forward pass on this slot
  R *pv, *pv_lon, *pv_lat;           // potential vorticity and its edge values
  double *we_lev;                    // vertical mass flux on half levels
  const double *gzs;                 // surface geopotential (static, shared by the slots)
};

// Work arrays of one member that live only within a pass.
template <class R>
struct Work {
  R *u_lat, *v_lon, *ke;
  R *cflx, *cfly, *cflz, *divx, *divy;
  R *qmfx, *qmfy, *qx, *qy, *ptf_lon, *ptf_lat;
  R *du, *dv, *dpt, *dgz;
  double *dphs, *ph_exn_lev, *gz_lev;
  const double *gzs;
};

// FFSL advection inputs of one batch (adv_batch_type, adv_batch_mod.F90:19-57).
template <class R>
struct BatchView {
  const R *u, *v;              // advecting winds
  const R *mfx, *mfy;          // mass fluxes (outer operator)
  const R *cflx, *cfly, *divx, *divy, *cflz;
  const R *we;                 // vertical mass flux (R copy for tracers)
  const double *we_d;          // or FP64 (mass batch)
  const R *m_lev;
};

struct Launch {
  cudaStream_t stream;
  int threads;   // block size for row kernels
};

// ---- dynamics (dyn.cu) ----------------------------------------------------
template <class R> void launch_mass_flux(const DGrid &g, const Launch &L, const Slot<R> &s);
template <class R> void launch_tangent_winds(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w);
template <class R> void launch_kinetic_energy(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w);
template <class R> void launch_pv(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w);
template <class R> void launch_pv_edges(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w);
// CFL numbers and axis divergences of a batch (adv_batch_accum_uv_cell).
template <class R> void launch_batch_cfl(const DGrid &g, const Launch &L, const R *u, const R *v, R *cflx, R *cfly, R *divx, R *divy, double dt);
template <class R> void launch_column_mass(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w, double dt);
template <class R> void launch_momentum_tend(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w);
template <class R> void launch_swm_dgz(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w);
template <class R> void launch_update_phs(const DGrid &g, const Launch &L, const Slot<R> &o, const Slot<R> &n, const Work<R> &w, double dt);
template <class R> void launch_update_pt(const DGrid &g, const Launch &L, const Slot<R> &o, const Slot<R> &n, const Work<R> &w, double dt);
template <class R> void launch_update_gz(const DGrid &g, const Launch &L, const Slot<R> &o, const Slot<R> &n, const Work<R> &w, double dt);
template <class R> void launch_column_backward(const DGrid &g, const Launch &L, const Slot<R> &n, const Work<R> &w);
template <class R> void launch_update_uv(const DGrid &g, const Launch &L, const Slot<R> &o, const Slot<R> &n, const Work<R> &w, double dt);
template <class R> void launch_filter_prologue(const DGrid &g, const Launch &L, const Slot<R> &s);
template <class R> void launch_diagnose(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w, double *partial, double *out);

// ---- advection (adv.cu) ---------------------------------------------------
// Horizontal FFSL flux of q (ffsl_calc_tracer_hflx_cell): inner advective
// operators, intermediate qx/qy, outer flux-form operators into (fx, fy).
template <class R> void launch_ffsl_hflx(const DGrid &g, const Launch &L, const BatchView<R> &b, const R *q, R *qmfx, R *qmfy, R *qx, R *qy, R *fx, R *fy, double dt);
// Potential-temperature tendency: flux divergence of (ptf_lon, ptf_lat) with
// pole rings plus the vertical FFSL flux with ghost levels (calc_grad_ptf).
template <class R> void launch_pt_tendency(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w);

}  // namespace gmc
