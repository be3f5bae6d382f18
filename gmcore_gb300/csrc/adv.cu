// Flux-form semi-Lagrangian (FFSL) advection kernels (Lin-Rood with PPM
// sub-grid reconstruction) for potential temperature with the dynamic mass
// batch and for the tracer batch.
//
// The PPM coefficients of the upwind cell are reconstructed where a face
// flux needs them instead of being stored as six work fields
// (ffsl_mod.F90:813-826 keeps qlx/dqx/q6x/qly/dqy/q6y in HBM); the
// integer-Courant part sums whole cells along the row in the reference's
// order.
#include <cuda_runtime.h>

#include "kernels.hpp"
#include "stencil.cuh"

namespace gmc {

namespace {

// One horizontal pass of hflx_ppm_cell (ffsl_mod.F90:778-881): x fluxes on
// full-latitude rows without the poles, y fluxes on half-latitude rows.
//   u, v  : advecting velocities (or mass fluxes for the outer operator)
//   mx    : field reconstructed along x;  my : field reconstructed along y.
template <class R>
__global__ void k_hflx(DGrid g, const R *u, const R *v, const R *cflx, const R *cfly, const R *mx, const R *my,
                       R *fx, R *fy) {
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon, lim = g.limiter;
  if (j != 1 && j != nlat) {
    auto X = [&](int l) { return mx[ix3(nlat, nlon, wrap(l, nlon), j, k)]; };
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      const size_t o = ix3(nlat, nlon, i, j, k);
      const R c = cflx[o];
      R flux;
      if (!(fabs(c) <= (R)g.hx)) {   // |cflx| beyond the reach the reference allows: error, no flux
        atomicOr(g.err, ERR_CFLX);
        fx[o] = 0;
        continue;
      }
      const int ci = (int)c;
      const R cf = c - (R)ci;
      if (c > 0) {
        const int iu = i - ci;
        R sum = 0;
        for (int l = i + 1 - ci; l <= i; ++l) sum = sum + X(l);
        R fl, df, f6;
        ppm(lim, X(iu - 2), X(iu - 1), X(iu), X(iu + 1), X(iu + 2), fl, df, f6);
        flux = u[o] * ppm_tail(sum, fl, df, f6, (R)1 - cf, (R)1) / c;
      } else if (c < 0) {
        const int iu = i - ci + 1;
        R sum = 0;
        for (int l = i + 1; l <= i - ci; ++l) sum = sum + X(l);
        R fl, df, f6;
        ppm(lim, X(iu - 2), X(iu - 1), X(iu), X(iu + 1), X(iu + 2), fl, df, f6);
        flux = -u[o] * ppm_tail(sum, fl, df, f6, (R)0, -cf) / c;
      } else {
        flux = 0;
      }
      fx[o] = flux;
    }
  }
  if (j <= nhalf) {
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      auto Y = [&](int jj) { return rd_full(my, g, i, jj, k); };
      const size_t o = ix3(nhalf, nlon, i, j, k);
      const R c = cfly[o];
      R flux;
      if (!(fabs(c) <= (R)1)) {
        atomicOr(g.err, ERR_CFLY);
        fy[o] = 0;
        continue;
      }
      if (c > 0) {
        const int ju = j;
        R fl, df, f6;
        ppm(lim, Y(ju - 2), Y(ju - 1), Y(ju), Y(ju + 1), Y(ju + 2), fl, df, f6);
        flux = v[o] * ppm_tail((R)0, fl, df, f6, (R)1 - c, (R)1) / c;
      } else if (c < 0) {
        const int ju = j + 1;
        R fl, df, f6;
        ppm(lim, Y(ju - 2), Y(ju - 1), Y(ju), Y(ju + 1), Y(ju + 2), fl, df, f6);
        flux = -v[o] * ppm_tail((R)0, fl, df, f6, (R)0, -c) / c;
      } else {
        flux = 0;
      }
      fy[o] = flux;
    }
  }
}

// Intermediate advective-form values qx, qy (ffsl_mod.F90:353-406).
template <class R>
__global__ void k_qxqy(DGrid g, const R *q, const R *qmfx, const R *qmfy, const R *divx, const R *divy, R *qx, R *qy,
                       double dt) {
  __shared__ double red[32];
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  const R hdt = (R)dt;
  if (j == 1 || j == nlat) {
    const int jv = j == 1 ? 1 : nhalf;
    double p = ring_sum(nlon, red, [&](int i) { return (double)qmfy[ix3(nhalf, nlon, i, jv, k)]; });
    p = p * ROW(g.le_lat, jv) / nlon / ROW(g.area_cell, j);
    const R pole = (R)p;
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      const size_t o = ix3(nlat, nlon, i, j, k);
      const R qv = q[o];
      qx[o] = qv;
      if (j == 1)
        qy[o] = qv - (R)0.5 * (pole - divy[o] * qv) * hdt;
      else
        qy[o] = qv + (R)0.5 * (pole - divy[o] * qv) * hdt;
    }
    return;
  }
  const R lel = (R)ROW(g.le_lon, j), ac = (R)ROW(g.area_cell, j), la0 = (R)ROW(g.le_lat, j), la1 = (R)ROW(g.le_lat, j - 1);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const size_t o = ix3(nlat, nlon, i, j, k);
    const R qv = q[o];
    R fxe = qmfx[o], fxw = qmfx[ix3(nlat, nlon, wrap(i - 1, nlon), j, k)];
    qx[o] = qv - (R)0.5 * ((fxe - fxw) * lel / ac - divx[o] * qv) * hdt;
    R fyn = qmfy[ix3(nhalf, nlon, i, j, k)], fys = qmfy[ix3(nhalf, nlon, i, j - 1, k)];
    qy[o] = qv - (R)0.5 * ((fyn * la0 - fys * la1) / ac - divy[o] * qv) * hdt;
  }
}

// Vertical FFSL flux at interface k of a column (vflx_ppm_cell,
// ffsl_mod.F90:905-938).  col[] holds the column with two ghost levels on
// each side at col[k + 1] for k = -1 .. nlev+2; PPM coefficients of levels
// outside 1..nlev are zero, as in the reference's level halo.
template <class R>
__device__ __forceinline__ R vflx_at(const DGrid &g, const R *col, int k, R c, R w) {
  const int nlev = g.nlev, lim = g.limiter;
  auto C = [&](int kk) { return col[min(max(kk, -1), nlev + 2) + 1]; };
  if (!(fabs(c) <= (R)nlev)) {
    atomicOr(g.err, ERR_CFLZ);
    return 0;
  }
  const int ci = (int)c;
  const R cf = c - (R)ci;
  auto coef = [&](int ku, R &fl, R &df, R &f6) {
    if (ku < 1 || ku > nlev) { fl = df = f6 = 0; return; }
    ppm(lim, C(ku - 2), C(ku - 1), C(ku), C(ku + 1), C(ku + 2), fl, df, f6);
  };
  if (c > 0) {
    const int ku = k - ci - 1;
    R sum = 0;
    for (int l = k - ci; l <= k - 1; ++l) sum = sum + C(l);
    R fl, df, f6;
    coef(ku, fl, df, f6);
    return w * ppm_tail(sum, fl, df, f6, (R)1 - cf, (R)1) / c;
  }
  if (c < 0) {
    const int ku = k - ci;
    R sum = 0;
    for (int l = k; l <= k - ci - 1; ++l) sum = sum + C(l);
    R fl, df, f6;
    coef(ku, fl, df, f6);
    return -w * ppm_tail(sum, fl, df, f6, (R)0, -cf) / c;
  }
  return 0;
}

// calc_grad_ptf tail (operators_mod.F90:1034-1098) with the tendency
// assembly dpt = -(dptf/dlon + dptf/dlat + dptf/dlev) (gmcore_mod.F90:491-495).
template <class R>
__global__ void k_pt_tendency(DGrid g, Slot<R> s, Work<R> w) {
  extern __shared__ double sh[];
  double *red = sh, *ring = sh + 32;
  const int j = blockIdx.y + 1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon, nlev = g.nlev;
  const bool pole = j == 1 || j == nlat;
  if (pole) {
    const int jv = j == 1 ? 1 : nhalf;
    const double sgn = j == 1 ? 1.0 : -1.0;
    for (int k = 1; k <= nlev; ++k) {
      double p = ring_sum(nlon, red, [&](int ii) { return sgn * (double)w.ptf_lat[ix3(nhalf, nlon, ii, jv, k)]; });
      if (threadIdx.x == 0) ring[k - 1] = p * ROW(g.le_lat, jv) / nlon / ROW(g.area_cell, j);
    }
    __syncthreads();
  }
  if (i > nlon) return;
  R col[70];
  for (int k = 1; k <= nlev; ++k) col[k + 1] = s.pt[ix3(nlat, nlon, i, j, k)];
  col[1] = (R)2 * col[2] - col[3];                       // k = 0
  col[0] = (R)2 * col[1] - col[2];                       // k = -1
  col[nlev + 2] = (R)2 * col[nlev + 1] - col[nlev];      // k = nlev+1
  col[nlev + 3] = (R)2 * col[nlev + 2] - col[nlev + 1];  // k = nlev+2
  const R lel = (R)ROW(g.le_lon, j), ac = (R)ROW(g.area_cell, j), la0 = (R)ROW(g.le_lat, j), la1 = (R)ROW(g.le_lat, j - 1);
  const int im = wrap(i - 1, nlon);
  R f_top = 0;   // ptf_lev(1) = 0
  for (int k = 1; k <= nlev; ++k) {
    const size_t o = ix3(nlat, nlon, i, j, k);
    R f_bot = 0;
    if (k + 1 <= nlev) {
      const size_t ol = ix3(nlat, nlon, i, j, k + 1);
      f_bot = vflx_at<R>(g, col, k + 1, w.cflz[ol], (R)s.we_lev[ol]);
    }
    R dlon, dlat;
    if (pole) {
      dlon = 0;
      dlat = (R)ring[k - 1];
    } else {
      dlon = (w.ptf_lon[o] - w.ptf_lon[ix3(nlat, nlon, im, j, k)]) * lel / ac;
      dlat = (w.ptf_lat[ix3(nhalf, nlon, i, j, k)] * la0 - w.ptf_lat[ix3(nhalf, nlon, i, j - 1, k)] * la1) / ac;
    }
    R dlev = f_bot - f_top;
    w.dpt[o] = -dlon - dlat - dlev;
    f_top = f_bot;
  }
}

}  // namespace

template <class R>
void launch_ffsl_hflx(const DGrid &g, const Launch &L, const BatchView<R> &b, const R *q, R *qmfx, R *qmfy, R *qx, R *qy,
                      R *fx, R *fy, double dt) {
  dim3 grid(g.nlat, g.nlev);
  k_hflx<R><<<grid, L.threads, 0, L.stream>>>(g, b.u, b.v, b.cflx, b.cfly, q, q, qmfx, qmfy);
  k_qxqy<R><<<grid, L.threads, 0, L.stream>>>(g, q, qmfx, qmfy, b.divx, b.divy, qx, qy, dt);
  k_hflx<R><<<grid, L.threads, 0, L.stream>>>(g, b.mfx, b.mfy, b.cflx, b.cfly, qy, qx, fx, fy);
}

template <class R>
void launch_pt_tendency(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w) {
  const int bt = 64;
  size_t smem = (32 + g.nlev + 2) * sizeof(double);
  k_pt_tendency<R><<<dim3((g.nlon + bt - 1) / bt, g.nlat), bt, smem, L.stream>>>(g, s, w);
}

template void launch_ffsl_hflx<double>(const DGrid &, const Launch &, const BatchView<double> &, const double *, double *,
                                       double *, double *, double *, double *, double *, double);
template void launch_ffsl_hflx<float>(const DGrid &, const Launch &, const BatchView<float> &, const float *, float *,
                                      float *, float *, float *, float *, float *, double);
template void launch_pt_tendency<double>(const DGrid &, const Launch &, const Slot<double> &, const Work<double> &);
template void launch_pt_tendency<float>(const DGrid &, const Launch &, const Slot<float> &, const Work<float> &);

}  // namespace gmc
