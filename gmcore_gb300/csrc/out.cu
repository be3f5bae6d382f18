// FP64 diagnostics of a state for history files: hydrostatic pressure,
// temperature and height at full levels, divergence at cells and relative
// vorticity at vertices, from the slot's prognostic and filtered fields
// (the reference writes state%ph, t, gz / g, div and vor, history_mod.F90:519-580).
// Both forms compute them in FP64 from the values the slot holds, so the
// output of the mixed form is the FP64 diagnosis of its FP32 state.
#include <cuda_runtime.h>

#include <type_traits>

#include "kernels.hpp"
#include "stencil.cuh"

namespace gmc {

namespace {

constexpr int kOutThreads = 128;
constexpr int kMaxLev = 65;   // largest level count a grid is validated for (+1 half level)

// One column per thread: ph, t (calc_ph, calc_t: operators_mod.F90:136-190,
// formula_mod.F90:24-31) and z = gz / g with gz the mean of the half-level
// geopotentials of calc_gz_lev (operators_mod.F90:433-469); each half level
// sums its layers from itself down to the surface, in that order.
template <class R>
__global__ void __launch_bounds__(kOutThreads) k_out_column(DGrid g, const R *__restrict__ pt,
                                                           const double *__restrict__ phs_f,
                                                           const double *__restrict__ gzs, double *__restrict__ ph,
                                                           double *__restrict__ t, double *__restrict__ z) {
  const size_t H = (size_t)g.nlat * g.nlon;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= H) return;
  const int nlev = g.nlev;
  double pl[kMaxLev + 1], dz[kMaxLev];
  const double ps = phs_f[c];
  for (int k = 1; k <= nlev + 1; ++k) pl[k - 1] = ph_lev(g, k, ps);
  for (int k = 1; k <= nlev; ++k) {
    const size_t o = (size_t)(k - 1) * H + c;
    const double p = 0.5 * (pl[k - 1] + pl[k]);
    const double tk = (double)pt[o] * pow(p / g.p0, g.kappa);
    ph[o] = p;
    t[o] = tk;
    dz[k - 1] = g.Rd * tk * log(pl[k] / pl[k - 1]);
  }
  const double s = gzs[c];
  double above = s;   // gz_lev(nlev + 1) = gzs
  for (int k = nlev; k >= 1; --k) {
    double acc = 0;
    for (int l = k; l <= nlev; ++l) acc = acc + dz[l - 1];
    const double here = s + acc;   // gz_lev(k)
    z[(size_t)(k - 1) * H + c] = 0.5 * (here + above) / g.g;
    above = here;
  }
}

// Shallow water: z = gz / g.
template <class R>
__global__ void k_out_swm_z(DGrid g, const R *__restrict__ gz, double *__restrict__ z) {
  const size_t H = (size_t)g.nlat * g.nlon;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < H; c += (size_t)gridDim.x * blockDim.x)
    z[c] = (double)gz[c] / g.g;
}

// Divergence of the filtered wind at cells (calc_div, operators_mod.F90:356-410):
// one block per (row, level); the pole rows from the ring sums of v.
template <class R>
__global__ void __launch_bounds__(kOutThreads) k_out_div(DGrid g, const R *__restrict__ u, const R *__restrict__ v,
                                                        double *__restrict__ div) {
  __shared__ double red[kOutThreads / 32];
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlon = g.nlon, nlat = g.nlat, nhalf = g.nhalf;
  const size_t fo = (size_t)ix3(nlat, nlon, 1, j, k);
  if (j == 1 || j == nlat) {
    const size_t ho = (size_t)ix3(nhalf, nlon, 1, j == 1 ? 1 : nhalf, k);
    const double sgn = j == 1 ? 1.0 : -1.0;
    const double r = ring_sum(nlon, red, [&](int i) { return sgn * (double)v[ho + i - 1]; });
    const double p = r * ROW(g.le_lat, j == 1 ? 1 : nhalf) / nlon / ROW(g.area_cell, j);
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) div[fo + i] = p;
    return;
  }
  const size_t hn = (size_t)ix3(nhalf, nlon, 1, j, k), hs = hn - nlon;
  const double lel = ROW(g.le_lon, j), ln = ROW(g.le_lat, j), ls = ROW(g.le_lat, j - 1), ac = ROW(g.area_cell, j);
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    const int iw = i == 0 ? nlon - 1 : i - 1;
    div[fo + i] = (((double)u[fo + i] * lel - (double)u[fo + iw] * lel) +
                   ((double)v[hn + i] * ln - (double)v[hs + i] * ls)) / ac;
  }
}

// Layer mass at cell (i0, row j) of level k: ph_lev(k+1) - ph_lev(k)
// (baroclinic) or (gz - gzs) / g (calc_m, operators_mod.F90:471-531).
template <class R>
__device__ __forceinline__ double out_mass(const DGrid &g, const Slot<R> &s, int i0, int j, int k) {
  const size_t c = (size_t)(j - 1) * g.nlon + i0;
  if (g.baroclinic) return Mass<double>::layer(g, k, s.phs_f[c]);
  return ((double)s.gz[c] - s.gzs[c]) / g.g;
}

// Relative vorticity of the filtered wind at vertices (calc_vor,
// operators_mod.F90:612-680): one block per (half row, level).  With
// pv_pole_stokes the two polar half rows hold the circulation along the ring
// of the tangential wind u_lat = mfx_lat / m_lat (calc_mf, :585-597) over the
// polar cap.
template <class R>
__global__ void __launch_bounds__(kOutThreads) k_out_vor(DGrid g, Slot<R> s, double *__restrict__ vor) {
  __shared__ double red[kOutThreads / 32];
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlon = g.nlon, nlat = g.nlat, nhalf = g.nhalf;
  const size_t ho = (size_t)ix3(nhalf, nlon, 1, j, k);
  if (g.pv_pole_stokes && (j == 1 || j == nhalf)) {
    // u_lat of half row j from the zonal mass fluxes m_lon u_f of full rows j
    // and j+1 (zero on the pole rows, where the reference forms none)
    auto mfx = [&](int i0, int jj) -> double {
      if (jj == 1 || jj == nlat) return 0.0;
      const int ie = i0 + 1 == nlon ? 0 : i0 + 1;
      const double ml = (out_mass(g, s, i0, jj, k) + out_mass(g, s, ie, jj, k)) * 0.5;
      return ml * (double)s.u_f[(size_t)ix3(nlat, nlon, 1, jj, k) + i0];
    };
    const double w1 = ROW(g.htw1, j), w2 = ROW(g.htw2, j);
    const double sgn = j == 1 ? -1.0 : 1.0;
    const double r = ring_sum(nlon, red, [&](int i) {
      const int i0 = i - 1, iw = i0 == 0 ? nlon - 1 : i0 - 1;
      const double mf = w1 * (mfx(iw, j) + mfx(i0, j)) + w2 * (mfx(iw, j + 1) + mfx(i0, j + 1));
      const double ml = (out_mass(g, s, i0, j, k) + out_mass(g, s, i0, j + 1, k)) * 0.5;
      return sgn * (mf / ml) * ROW(g.le_lat, j);
    });
    const double p = r / nlon / ROW(g.area_cell, j == 1 ? 1 : nhalf + 1);
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) vor[ho + i] = p;
    return;
  }
  const size_t fs = (size_t)ix3(nlat, nlon, 1, j, k), fn = fs + nlon;
  const double dls = ROW(g.de_lon, j), dln = ROW(g.de_lon, j + 1), dla = ROW(g.de_lat, j), av = ROW(g.area_vtx, j);
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    const int ie = i + 1 == nlon ? 0 : i + 1;
    vor[ho + i] = ((double)s.u_f[fs + i] * dls - (double)s.u_f[fn + i] * dln + (double)s.v_f[ho + ie] * dla -
                   (double)s.v_f[ho + i] * dla) / av;
  }
}

}  // namespace

template <class R>
void launch_output_diag(const DGrid &g, cudaStream_t st, const Slot<R> &s, double *ph, double *t, double *z,
                        double *div, double *vor) {
  const size_t H = (size_t)g.nlat * g.nlon;
  if (g.baroclinic)
    k_out_column<R><<<(unsigned)((H + kOutThreads - 1) / kOutThreads), kOutThreads, 0, st>>>(g, s.pt, s.phs_f, s.gzs,
                                                                                             ph, t, z);
  else
    k_out_swm_z<R><<<(unsigned)((H + kOutThreads - 1) / kOutThreads), kOutThreads, 0, st>>>(g, s.gz, z);
  k_out_div<R><<<dim3(g.nlat, g.nlev), kOutThreads, 0, st>>>(g, s.u_f, s.v_f, div);
  k_out_vor<R><<<dim3(g.nhalf, g.nlev), kOutThreads, 0, st>>>(g, s, vor);
}

template void launch_output_diag<double>(const DGrid &, cudaStream_t, const Slot<double> &, double *, double *,
                                         double *, double *, double *);
template void launch_output_diag<float>(const DGrid &, cudaStream_t, const Slot<float> &, double *, double *,
                                        double *, double *, double *);

}  // namespace gmc
