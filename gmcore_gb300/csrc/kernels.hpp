// Host-visible launchers of the device kernels and the pointer bundles they
// operate on.  R is the storage/arithmetic type of the bulk 3-D fields
// (double for the FP64 form, float for the mixed form); the FP64-only pieces
// (surface pressure, column sweeps, pole rings, diagnostics) are double.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "common.cuh"

namespace gmc {

// Fields of one state slot (one of the reference's state(1:3)).
template <class R>
struct Slot {
  R *u_lon, *v_lat, *u_f, *v_f;     // wind on its edges and filtered wind
  R *pt;                             // baroclinic potential temperature
  R *gz, *gz_f;                      // shallow-water geopotential
  double *phs, *phs_f;               // surface pressure (baroclinic)
  float *psr;                        // FP32 form: phs_f - ptop in FP32 (null in the FP64 form)
  R *mfx_lon, *mfy_lat;              // mass fluxes of the last forward pass on this slot
  R *pv, *pv_lon, *pv_lat;           // potential vorticity and its edge values
  R *we_lev;                         // vertical mass flux on half levels
  const double *gzs;                 // surface geopotential (static, shared by the slots)
  __host__ __device__ SurfP<R> surf() const { return SurfP<R>{phs_f, psr}; }
};

// Work arrays of one member that live only within a pass.
template <class R>
struct Work {
  R *u_lat, *v_lon, *ke;
  R *cflx, *cfly, *cflz, *divx, *divy;
  R *qmfx, *qmfy, *qx, *qy, *ptf_lon, *ptf_lat;
  R *du, *dv, *dpt, *dgz;
  double *dphs, *ph_exn_lev, *gz_lev;
  // FP32 form views of the same memory: Exner pressure minus the reference
  // column's (pea) and geopotential as a (hi, lo) FP32 pair (gzhl).
  float *pea;
  float2 *gzhl;
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

// Opt a kernel in to more than 48 KB of dynamic shared memory when a launch
// needs it (wide rows, tall columns).
template <class Kern>
inline void allow_smem(Kern k, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

struct Launch {
  cudaStream_t stream;
  int threads;       // block size for row kernels
  int members = 1;   // ensemble members of one launch (grid z; member-batched kernels)
};

// Launch f(std::true_type) when the launch covers several members (the
// member-batched kernel variant, which moves its pointers by the member's
// offset) and f(std::false_type) otherwise (the single-member variant, whose
// pointers stay in the parameter bank).
template <class F>
inline void mb_launch(const Launch &L, F &&f) {
  if (L.members > 1) f(std::true_type{});
  else f(std::false_type{});
}

// Member-batched launches: blockIdx.z selects the ensemble member.  The
// members' arena blocks are carved identically one after the other, so every
// member-owned pointer of member m is member 0's plus m * g.mstride bytes.
__device__ __forceinline__ size_t member_offset(const DGrid &g) { return (size_t)blockIdx.z * g.mstride; }
template <class T>
__device__ __forceinline__ T *mshift(T *p, size_t mo) {
  return p ? reinterpret_cast<T *>(reinterpret_cast<uintptr_t>(p) + mo) : p;
}
template <class R>
__device__ __forceinline__ void to_member(const DGrid &g, Slot<R> &s) {
  const size_t mo = member_offset(g);
  s.u_lon = mshift(s.u_lon, mo); s.v_lat = mshift(s.v_lat, mo); s.u_f = mshift(s.u_f, mo); s.v_f = mshift(s.v_f, mo);
  s.pt = mshift(s.pt, mo); s.gz = mshift(s.gz, mo); s.gz_f = mshift(s.gz_f, mo);
  s.phs = mshift(s.phs, mo); s.phs_f = mshift(s.phs_f, mo); s.psr = mshift(s.psr, mo);
  s.mfx_lon = mshift(s.mfx_lon, mo); s.mfy_lat = mshift(s.mfy_lat, mo);
  s.pv = mshift(s.pv, mo); s.pv_lon = mshift(s.pv_lon, mo); s.pv_lat = mshift(s.pv_lat, mo);
  s.we_lev = mshift(s.we_lev, mo); s.gzs = mshift(s.gzs, mo);
}
template <class R>
__device__ __forceinline__ void to_member(const DGrid &g, Work<R> &w) {
  const size_t mo = member_offset(g);
  w.u_lat = mshift(w.u_lat, mo); w.v_lon = mshift(w.v_lon, mo); w.ke = mshift(w.ke, mo);
  w.cflx = mshift(w.cflx, mo); w.cfly = mshift(w.cfly, mo); w.cflz = mshift(w.cflz, mo);
  w.divx = mshift(w.divx, mo); w.divy = mshift(w.divy, mo);
  w.qmfx = mshift(w.qmfx, mo); w.qmfy = mshift(w.qmfy, mo); w.qx = mshift(w.qx, mo); w.qy = mshift(w.qy, mo);
  w.ptf_lon = mshift(w.ptf_lon, mo); w.ptf_lat = mshift(w.ptf_lat, mo);
  w.du = mshift(w.du, mo); w.dv = mshift(w.dv, mo); w.dpt = mshift(w.dpt, mo); w.dgz = mshift(w.dgz, mo);
  w.dphs = mshift(w.dphs, mo); w.ph_exn_lev = mshift(w.ph_exn_lev, mo); w.gz_lev = mshift(w.gz_lev, mo);
  w.pea = mshift(w.pea, mo); w.gzhl = mshift(w.gzhl, mo); w.gzs = mshift(w.gzs, mo);
}

// ---- dynamics (dyn.cu) ----------------------------------------------------
template <class R> void launch_mass_flux(const DGrid &g, const Launch &L, const Slot<R> &s);
template <class R> void launch_tangent_winds(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w);
template <class R> void launch_kinetic_energy(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w);
template <class R> void launch_pv(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w);
template <class R> void launch_pv_edges(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w, double dt);
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
// FP32 form: psr = phs_f - ptop of a slot (no-op in the FP64 form).
template <class R> void launch_surface_rel(const DGrid &g, const Launch &L, const Slot<R> &s);
// non-finite or non-monotonic columns of a slot's filtered surface pressure (ERR_NAN, ERR_NONMONO)
template <class R> void launch_check_columns(const DGrid &g, const Launch &L, const Slot<R> &s);
template <class R> void launch_diagnose(const DGrid &g, const Launch &L, const Slot<R> &s, double *partial, double *out);
// FP64 history diagnostics of a slot (out.cu): ph, t, z at full levels
// (baroclinic; z = gz / g in shallow water, ph and t unused), div at cells,
// vor at vertices; dense [k][j][i] device arrays.
template <class R> void launch_output_diag(const DGrid &g, cudaStream_t st, const Slot<R> &s, double *ph, double *t,
                                           double *z, double *div, double *vor);

// Divergence damping of order 2 or 4 (div_damp_run, div_damp_mod.F90:89-139);
// div and div2 are scratch cell fields.
template <class R> void launch_div_damp(const DGrid &g, const Launch &L, const Slot<R> &n, R *div, R *div2);
template <class R> void launch_held_suarez(const DGrid &g, const Launch &L, const Slot<R> &n, double dt);
template <class R> void launch_smag_damp(const DGrid &g, const Launch &L, const Slot<R> &n, R *st, R *ss, R *du, R *dv,
                                         double dt);

// ---- advection (adv.cu) ---------------------------------------------------
// Horizontal FFSL flux of q (ffsl_calc_tracer_hflx_cell): inner advective
// operators, intermediate qx/qy, outer flux-form operators into (fx, fy).
template <class R> void launch_ffsl_hflx(const DGrid &g, const Launch &L, const BatchView<R> &b, const R *q, R *qx, R *qy, R *fx, R *fy, double dt);
// the three FFSL kernels of launch_ffsl_hflx separately (profiled as three groups)
template <class R> void launch_ffsl_inner_y(const DGrid &g, const Launch &L, const BatchView<R> &b, const R *q, R *qy, double dt);
template <class R> void launch_ffsl_x2(const DGrid &g, const Launch &L, const BatchView<R> &b, const R *q, const R *qy, R *qx, R *fx, double dt);
template <class R> void launch_hflx_y(const DGrid &g, const Launch &L, const BatchView<R> &b, const R *qx, R *fy);
// Potential-temperature tendency: flux divergence of (ptf_lon, ptf_lat) with
// pole rings plus the vertical FFSL flux with ghost levels (calc_grad_ptf).
template <class R> void launch_pt_tendency(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w);

// Tracer batch (adv_run, adv_mod.F90:152-312).
template <class R>
struct TracerBatch {
  R *u, *v, *mfx, *mfy;            // accumulated winds and mass fluxes
  R *we, *m_lev;                   // accumulated vertical mass flux and half-level mass
  R *cflx, *cfly, *divx, *divy, *cflz;
  double *old_phs_f;               // surface pressure whose layer masses are old_m
  float *old_psr;                  // its FP32 form (null in the FP64 form)
  __host__ __device__ SurfP<R> old_surf() const { return SurfP<R>{old_phs_f, old_psr}; }
};
// Accumulation of one field: mode 0 copy, 1 add, 2 average with divisor.
template <class T> void launch_accum(const Launch &L, T *dst, const T *src, size_t n, int mode, double divisor);
// accumulation entries of one launch (copy / add / average, as launch_accum)
template <class T>
struct AccumEntry {
  T *dst;
  const T *src;   // null: a zero sample
  size_t n;
  int mode;
  double divisor;
};
template <class T>
struct AccumSet {
  AccumEntry<T> e[6];
  int count;
};
template <class T> void launch_accum_multi(const Launch &L, const AccumSet<T> &set);
// Half-level mass of a slot (calc_m, operators_mod.F90:505-525) into a
// level field, or zero it when src_phs_f is null.
template <class R> void launch_half_level_mass(const DGrid &g, const Launch &L, const SurfP<R> &sp, R *m_lev, int mode, double divisor);
// Vertical Courant numbers of a batch (adv_batch_accum_we_lev RK4 part).
template <class R> void launch_batch_cflz(const DGrid &g, const Launch &L, const R *we, const R *m_lev, R *cflz, double dt);
// Horizontal tracer update with pole rings, division by the new mass and the
// zonal negative fixer (adv_mod.F90:183-258).
template <class R> void launch_tracer_horizontal(const DGrid &g, const Launch &L, const R *q_old, R *q_new, const R *fx, const R *fy, const SurfP<R> &old_sp, const SurfP<R> &sp, double dt_adv);
// Vertical FFSL update with the vertical fixer (adv_mod.F90:259-297).
template <class R> void launch_tracer_vertical(const DGrid &g, const Launch &L, R *q, const R *cflz, const R *we, const SurfP<R> &sp, double dt_adv);
// Three passes of the order-2 zonal smoother (lon_damp_on_cell, adv_mod.F90:298-302).
template <class R> void launch_tracer_lon_damp(const DGrid &g, const Launch &L, R *q);

// ---- tangent-linear and adjoint of the shallow-water step (tlad.cu, FP64) ----
// TL of forward_prepare at the star state s (values w from forward_prepare):
// tangents of mfx, mfy, pv, pv_lon, pv_lat into t, of u_lat, v_lon, ke into tw.
void tl_forward_prepare(const DGrid &g, const Launch &L, const Slot<double> &s, const Work<double> &w,
                        const Slot<double> &t, const Work<double> &tw);
// TL of the shallow-water momentum tendencies into tw.du, tw.dv.
void tl_momentum(const DGrid &g, const Launch &L, const Slot<double> &s, const Slot<double> &t, const Work<double> &tw);
// AD of the updates of a stage: consumes (and clears) the adjoint of the new
// slot an, adds to the old slot ao, sets aw.du, aw.dv, aw.dgz, and clears
// the nzero values at zero (the adjoint work the forward pass accumulates into).
void ad_update(const DGrid &g, const Launch &L, const Slot<double> &ao, const Slot<double> &an, const Work<double> &aw,
               double *zero, size_t nzero, double dt);
// AD of the forward pass at the star state s: from aw.du, aw.dv, aw.dgz into
// the star adjoint a (u_f, v_f, gz; work adjoints mfx, mfy, pv, pv_lon, pv_lat
// in a must start at zero, as must aw.u_lat, aw.v_lon, aw.ke).
void ad_forward(const DGrid &g, const Launch &L, const Slot<double> &s, const Work<double> &w, const Slot<double> &a,
                const Work<double> &aw);
// AD of the run-prologue filters: u += big^T u_f, v += big^T v_f, gz += big^T gz_f.
void ad_prologue(const DGrid &g, const Launch &L, const Slot<double> &a);

}  // namespace gmc
