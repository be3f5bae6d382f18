// Device-side common definitions for the GB300 GMCORE step.
//
// Layout in HBM: every field is stored without halos, level-major,
// [k][j][i] with i (longitude) fastest and a row pitch of nlon elements.
// Full-latitude fields have nlat rows (both pole rows included), half-latitude
// fields nlat-1 rows, half-level fields nlev+1 levels.  Halo points of the
// reference arrays are produced by index arithmetic instead of copies:
//   - longitude: periodic wrap;
//   - latitude beyond a pole: the row on the other side of the pole, rotated
//     by nlon/2 for interior columns, which is what the single-rank
//     fill_halo writes (src/utils/parallel_mod.F90:529-563);
//   - level ghost values of potential temperature and tracers: the linear
//     extrapolation / copy the reference stores in its level halo
//     (operators_mod.F90:1085-1090, adv_mod.F90:260-265), recomputed on load.
// Indices in kernels are the reference's 1-based Fortran indices.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gmcore_gpu.h"

namespace gmc {

// Error word bits set by kernels (read by the host after a step).
enum : unsigned {
  ERR_CFLX = 1u, ERR_CFLY = 2u, ERR_CFLZ = 4u, ERR_NONMONO = 8u, ERR_NEGTRACER = 16u, ERR_NAN = 32u,
};

struct FilterDev {
  const int *ntaps_full;   // [nlat], row j at [j-1]
  const int *ntaps_half;   // [nhalf]
  const int *off_full;     // weight offsets
  const int *off_half;
  const double *wgt;
  const float *wgt_f;      // FP32 copy for rows accumulated in FP32
  int max_taps;
};

// FP32 copies of the row tables (same indexing), read by the FP32 form so
// that no FP64 arithmetic or conversion runs in its kernels.
struct RowF {
  const float *area_cell, *area_subcell1, *area_subcell2;
  const float *area_lon, *area_lon_west, *area_lon_east, *area_lon_north, *area_lon_south;
  const float *area_lat, *area_lat_west, *area_lat_east, *area_lat_north, *area_lat_south;
  const float *area_vtx, *de_lon, *le_lon, *de_lat, *le_lat, *full_f, *half_f;
  const float *ftw1, *ftw2, *htw1, *htw2, *full_cos_lat, *half_lat, *half_cos_lat, *full_sin_lat;
};

// Grid constants and 1-D metric tables (device pointers).  Row tables are
// indexed [j + 1] for j = -1 .. n+2 (j = 0 and j = n+1 hold the reference's
// halo values), level tables [k - 1].
struct DGrid {
  int nlon, nlat, nhalf, nlev, hx, half;
  int baroclinic;
  double radius, g, Rd, cpd, p0, kappa, p0h, ptop, dlon;
  int ke_scheme;
  double ke_cell_wgt;
  int pv_scheme, upwind_order_pv, pv_pole_stokes, coriolis_scheme, limiter;
  double upwind_wgt_pv;
  // FP32 copies of scalar constants read by the FP32 form (no per-thread
  // FP64 -> FP32 conversion on the FP64 pipe)
  float ke_cell_wgt_f, upwind_wgt_pv_f, kappa_f, Rd_f, g_f;
  const double *area_cell, *area_subcell1, *area_subcell2;
  const double *area_lon, *area_lon_west, *area_lon_east, *area_lon_north, *area_lon_south;
  const double *area_lat, *area_lat_west, *area_lat_east, *area_lat_north, *area_lat_south;
  const double *area_vtx, *de_lon, *le_lon, *de_lat, *le_lat, *full_f, *half_f;
  const double *ftw1, *ftw2, *htw1, *htw2, *full_cos_lat, *half_lat, *half_cos_lat, *full_sin_lat;
  RowF f;
  int flux_type;        // GMC_FLUX_*
  int tvd_limiter;      // GMC_TVD_* (pv_scheme = tvd)
  int div_damp_order;   // 2 or 4
  // FP32 form of the y departure: offsets radius (half_lat(l) - half_lat(j)) / de_lat(j)
  // for l = j-1 .. j+2 at [(j-1)*4 + l-j+1] (0 outside 1..nhalf)
  const float *cfl_yoff;
  const double *hyai, *hybi, *half_lev, *half_dlev, *full_dlev;   // [k-1]
  const float *dmA, *dmB;                                          // FP32 layer-mass coefficients [k-1]
  int f_layer_mass;                                                // 1: the form's layer mass is dmA + dmB psr (FP32)
  int tangent_inline;   // 1: the FP32 edge PV and pole PV form the tangential winds themselves (no u_lat/v_lon fields)
  int forcing;                  // GMC_FORCING_*
  double smag_coef;             // smag_damp_coef
  const double *full_lev;       // eta at full levels [k-1]
  const float *ph_lev_a;        // FP32 hyai(k) (p0 - ptop) + ptop [k-1]: ph_lev = a + hybi psr
  const float *half_lev_f, *half_dlev_f, *full_dlev_f;             // FP32 copies of the eta tables
  const float *hybi_f;                                             // FP32 copy of hybi [k-1]
  const float *full_dlev_rf;                                       // FP32 1 / full_dlev [k-1]
  // FP32 column sweep about a reference column with surface pressure ps_ref
  // (pressures p_ref on half levels, ph_ref on full levels):
  //   pr_c[k-1]    = hybi(k) / p_ref(k)              k = 1..nlev+1
  //   pe_ref[k-1]  = p_ref(k)^kappa                  k = 1..nlev+1
  //   dpe_ref[k-1] = p_ref(k+1)^kappa - p_ref(k)^kappa   k = 1..nlev
  //   cf[k-1]      = (hybi(k) + hybi(k+1)) / 2 / ph_ref(k)
  //   tf_ref[k-1]  = (ph_ref(k) / p0)^kappa
  //   dlnp_ref[k-1] = ln(p_ref(k+1) / p_ref(k))
  const float *pr_c, *pe_ref, *dpe_ref, *cf, *tf_ref, *dlnp_ref;
  double ps_ref;
  const double *lon_damp_full;                                     // [j-1]
  const double *div_c_lon, *div_c_lat;                             // [(k-1)*n + j-1]
  FilterDev big, small1, small2;
  unsigned *err;                                                   // device error words [2] (raise_err)
  size_t mstride;                                                  // bytes between ensemble members' fields
};

// Raise an error from a kernel: err[0] collects every bit raised, err[1]
// keeps the first one (kernels run in the step's launch order, so that is the
// error the reference, which stops at its first log_error, would report).
__device__ __forceinline__ void raise_err(const DGrid &g, unsigned bit) {
  atomicOr(g.err, bit);
  atomicCAS(g.err + 1, 0u, bit);
}

#define ROW(t, j) ((t)[(j) + 1])

// Row table `name` at row j in the arithmetic type R of the form.
template <class R>
struct RowSel;
template <>
struct RowSel<double> {
  static __device__ __forceinline__ const double *pick(const double *d, const float *) { return d; }
};
template <>
struct RowSel<float> {
  static __device__ __forceinline__ const float *pick(const double *, const float *f) { return f; }
};
#define ROWR(R, name, j) (RowSel<R>::pick(g.name, g.f.name)[(j) + 1])
// Scalar constant `name` of DGrid in the form's type (name_f in FP32).
template <class R>
struct ScalarSel;
template <>
struct ScalarSel<double> {
  static __device__ __forceinline__ double pick(double d, float) { return d; }
};
template <>
struct ScalarSel<float> {
  static __device__ __forceinline__ float pick(double, float f) { return f; }
};
#define SCALR(R, name) (ScalarSel<R>::pick(g.name, g.name##_f))

// Surface pressure as the layer-mass formula of each form reads it: the FP64
// form takes phs_f, the FP32 form psr = phs_f - ptop rounded once to FP32.
template <class R>
struct SurfP;
template <>
struct SurfP<double> {
  const double *phs_f;
  const float *psr;
  __device__ __forceinline__ double at(size_t o) const { return phs_f[o]; }
};
template <>
struct SurfP<float> {
  const double *phs_f;
  const float *psr;
  __device__ __forceinline__ float at(size_t o) const { return psr[o]; }
};

// Launch bounds of the row and column kernels (blocks of at most 256
// threads). Their FP32 forms are bound by memory latency: each is capped at
// the register count that keeps NB blocks resident per SM without spilling
// (8 blocks = 2048 threads at 32 registers, 6 at 40, 4 at 64), which measured
// faster than forms with fewer resident warps and more loads in flight per
// thread. The FP64 forms are capped at 128 registers.
#define GMC_BOUNDS(R, NB) __launch_bounds__(256, sizeof(R) == 4 ? NB : 2)
#define GMC_BOUNDS_F(NB) __launch_bounds__(256, NB)
// The member-batched variant of a kernel (MB) keeps its member offset in
// registers: one resident block fewer per SM (a few more registers) there.
#define GMC_BOUNDS_MB(R, NB, MB) __launch_bounds__(256, sizeof(R) == 4 ? ((MB) ? (NB) - 2 : (NB)) : 2)
#define GMC_BOUNDS_FMB(NB, NB_MB, MB) __launch_bounds__(256, (MB) ? (NB_MB) : (NB))

__device__ __forceinline__ int wrap(int i, int n) { return i < 1 ? i + n : (i > n ? i - n : i); }

// Offset of (i, j, k) in a [k][j][i] field; 32-bit arithmetic (grids are
// validated to (nlev+1) * nlat * nlon < 2^31).
__device__ __forceinline__ size_t ix3(int nrow, int nlon, int i, int j, int k) {
  return (size_t)(((unsigned)(k - 1) * (unsigned)nrow + (unsigned)(j - 1)) * (unsigned)nlon + (unsigned)(i - 1));
}

// Read a full-latitude field at any (i, j) the reference's stencils touch.
template <class T>
__device__ __forceinline__ T rd_full(const T *a, const DGrid &g, int i, int j, int k) {
  if (j < 1 || j > g.nlat) {
    bool lon_halo = i < 1 || i > g.nlon;
    if (lon_halo) {
      j = j < 1 ? j + 3 : j - 3;   // halo columns keep the unrotated rows
    } else {
      j = j < 1 ? 2 - j : 2 * g.nlat - j;
      i += g.half;
    }
  }
  return a[ix3(g.nlat, g.nlon, wrap(i, g.nlon), j, k)];
}

// Same for half-latitude fields.
template <class T>
__device__ __forceinline__ T rd_half(const T *a, const DGrid &g, int i, int j, int k) {
  if (j < 1 || j > g.nhalf) {
    bool lon_halo = i < 1 || i > g.nlon;
    if (lon_halo) {
      j = j < 1 ? j + 2 : j - 2;
    } else {
      j = j < 1 ? 1 - j : 2 * g.nhalf + 1 - j;
      i += g.half;
    }
  }
  return a[ix3(g.nhalf, g.nlon, wrap(i, g.nlon), j, k)];
}

// Fixed-order block sum (deterministic for a given blockDim).  All threads
// receive the result.
__device__ __forceinline__ double block_sum(double v, double *smem) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (l == 0) smem[w] = v;
  __syncthreads();
  double s = 0;
  for (int t = 0; t < nw; ++t) s += smem[t];
  __syncthreads();
  return s;
}

// Sum of f(i) over a latitude ring i = 1..nlon by one block.
template <class F>
__device__ __forceinline__ double ring_sum(int nlon, double *smem, F f) {
  double s = 0;
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) s += f(i);
  return block_sum(s, smem);
}

__device__ __forceinline__ double fsign(double a, double b) { return copysign(fabs(a), b); }
__device__ __forceinline__ float fsign(float a, float b) { return copysignf(fabsf(a), b); }

}  // namespace gmc
