// Tangent-linear (TL) and adjoint (AD) kernels of the shallow-water dynamics
// step in FP64: one kernel of each kind per nonlinear forward kernel.  The
// forward kernels that are linear in their inputs (k_swm_dgz, k_update_gz,
// k_update_uv, k_filter_copy) serve as their own tangent-linear operators;
// their adjoints are here.
//
// The linearisation point of a stage is the star state S and the quantities
// forward_prepare derives from it (mfx, mfy, u_lat, v_lon, ke, pv, pv_lon,
// pv_lat), recomputed by the forward kernels before the stage's TL or AD
// kernels run.  AD kernels scatter: each thread takes one output point, forms
// its local partial derivatives and adds them to the input adjoints, with
// atomicAdd where neighbouring outputs share an input.  Index maps (longitude
// wrap, pole halo rows) are the forward kernels' own.
//
// Reference operators differentiated: calc_mf (operators_mod.F90:545-610),
// calc_ke ke_scheme 1 (:234-282), calc_vor/calc_pv (:612-703),
// interp_pv_midpoint/upwind (:705-795, upwind_mod.F90:27-39), calc_coriolis
// (:846-906), calc_grad_ke (:908-937), the shallow-water dgz (gmcore_mod.F90:520-524),
// update_state (time_schemes_mod.F90:120-242), pgf_swm (pgf_swm_mod.F90:18-46)
// and the polar filters (filter_mod.F90:25-163).
#include <cuda_runtime.h>

#include "kernels.hpp"
#include "stencil.cuh"

namespace gmc {

namespace {

__device__ __forceinline__ double mcell(const DGrid &g, const double *gz, const double *gzs, int i, int j) {
  i = wrap(i, g.nlon);
  const size_t o = (size_t)(j - 1) * g.nlon + (i - 1);
  return (gz[o] - gzs[o]) / g.g;
}
__device__ __forceinline__ size_t off_full(const DGrid &g, int i, int j) { return ix3(g.nlat, g.nlon, wrap(i, g.nlon), j, 1); }
__device__ __forceinline__ size_t off_hlat(const DGrid &g, int i, int j) { return ix3(g.nhalf, g.nlon, wrap(i, g.nlon), j, 1); }
// offset that rd_half reads for (i, j) (pole halo rows included)
__device__ __forceinline__ size_t off_half_halo(const DGrid &g, int i, int j) {
  if (j < 1 || j > g.nhalf) {
    bool lon_halo = i < 1 || i > g.nlon;
    if (lon_halo) {
      j = j < 1 ? j + 2 : j - 2;
    } else {
      j = j < 1 ? 1 - j : 2 * g.nhalf + 1 - j;
      i += g.half;
    }
  }
  return ix3(g.nhalf, g.nlon, wrap(i, g.nlon), j, 1);
}
__device__ __forceinline__ void aadd(double *p, double v) { atomicAdd(p, v); }

// ---------------------------------------------------------------------------
// calc_mf: mfx = m_lon u_f, mfy = m_lat v_f, m = (gz - gzs) / g
// ---------------------------------------------------------------------------
__global__ void k_tl_mass_flux(DGrid g, Slot<double> s, Slot<double> t) {
  const int j = blockIdx.x + 1;
  const double ig = 1.0 / g.g;
  for (int i = 1 + threadIdx.x; i <= g.nlon; i += blockDim.x) {
    if (j == 1 || j == g.nlat) {
      t.mfx_lon[off_full(g, i, j)] = 0;
    } else {
      const size_t o = off_full(g, i, j);
      const double m_lon = (mcell(g, s.gz, s.gzs, i, j) + mcell(g, s.gz, s.gzs, i + 1, j)) * 0.5;
      const double dm_lon = (t.gz[off_full(g, i, j)] + t.gz[off_full(g, i + 1, j)]) * ig * 0.5;
      t.mfx_lon[o] = dm_lon * s.u_f[o] + m_lon * t.u_f[o];
    }
    if (j <= g.nhalf) {
      const size_t o = off_hlat(g, i, j);
      const double m_lat = (mcell(g, s.gz, s.gzs, i, j) + mcell(g, s.gz, s.gzs, i, j + 1)) * 0.5;
      const double dm_lat = (t.gz[off_full(g, i, j)] + t.gz[off_full(g, i, j + 1)]) * ig * 0.5;
      t.mfy_lat[o] = dm_lat * s.v_f[o] + m_lat * t.v_f[o];
    }
  }
}
__global__ void k_ad_mass_flux(DGrid g, Slot<double> s, Slot<double> a) {
  const int j = blockIdx.x + 1;
  const double ig = 1.0 / g.g;
  for (int i = 1 + threadIdx.x; i <= g.nlon; i += blockDim.x) {
    if (j != 1 && j != g.nlat) {
      const size_t o = off_full(g, i, j);
      const double fb = a.mfx_lon[o];
      const double m_lon = (mcell(g, s.gz, s.gzs, i, j) + mcell(g, s.gz, s.gzs, i + 1, j)) * 0.5;
      a.u_f[o] += m_lon * fb;
      const double mb = 0.5 * s.u_f[o] * fb * ig;
      aadd(&a.gz[off_full(g, i, j)], mb);
      aadd(&a.gz[off_full(g, i + 1, j)], mb);
    }
    if (j <= g.nhalf) {
      const size_t o = off_hlat(g, i, j);
      const double fb = a.mfy_lat[o];
      const double m_lat = (mcell(g, s.gz, s.gzs, i, j) + mcell(g, s.gz, s.gzs, i, j + 1)) * 0.5;
      a.v_f[o] += m_lat * fb;
      const double mb = 0.5 * s.v_f[o] * fb * ig;
      aadd(&a.gz[off_full(g, i, j)], mb);
      aadd(&a.gz[off_full(g, i, j + 1)], mb);
    }
  }
}

// ---------------------------------------------------------------------------
// tangential winds: u_lat = mfx_lat / m_lat, v_lon = mfy_lon / m_lon
// ---------------------------------------------------------------------------
__global__ void k_tl_tangent(DGrid g, Slot<double> s, Work<double> w, Slot<double> t, Work<double> tw) {
  const int j = blockIdx.x + 1;
  const double ig = 1.0 / g.g;
  if (j <= g.nhalf) {
    const double w1 = ROW(g.htw1, j), w2 = ROW(g.htw2, j);
    for (int i = 1 + threadIdx.x; i <= g.nlon; i += blockDim.x) {
      const double dmfx = w1 * (t.mfx_lon[off_full(g, i - 1, j)] + t.mfx_lon[off_full(g, i, j)]) +
                          w2 * (t.mfx_lon[off_full(g, i - 1, j + 1)] + t.mfx_lon[off_full(g, i, j + 1)]);
      const double m_lat = (mcell(g, s.gz, s.gzs, i, j) + mcell(g, s.gz, s.gzs, i, j + 1)) * 0.5;
      const double dm_lat = (t.gz[off_full(g, i, j)] + t.gz[off_full(g, i, j + 1)]) * ig * 0.5;
      const size_t o = off_hlat(g, i, j);
      tw.u_lat[o] = (dmfx - w.u_lat[o] * dm_lat) / m_lat;
    }
  }
  for (int i = 1 + threadIdx.x; i <= g.nlon; i += blockDim.x) {
    const size_t o = off_full(g, i, j);
    if (j == 1 || j == g.nlat) {
      tw.v_lon[o] = 0;
      continue;
    }
    const double w1 = ROW(g.ftw1, j), w2 = ROW(g.ftw2, j);
    const double dmfy = w1 * (t.mfy_lat[off_hlat(g, i, j - 1)] + t.mfy_lat[off_hlat(g, i + 1, j - 1)]) +
                        w2 * (t.mfy_lat[off_hlat(g, i, j)] + t.mfy_lat[off_hlat(g, i + 1, j)]);
    const double m_lon = (mcell(g, s.gz, s.gzs, i, j) + mcell(g, s.gz, s.gzs, i + 1, j)) * 0.5;
    const double dm_lon = (t.gz[off_full(g, i, j)] + t.gz[off_full(g, i + 1, j)]) * ig * 0.5;
    tw.v_lon[o] = (dmfy - w.v_lon[o] * dm_lon) / m_lon;
  }
}
__global__ void k_ad_tangent(DGrid g, Slot<double> s, Work<double> w, Slot<double> a, Work<double> aw) {
  const int j = blockIdx.x + 1;
  const double ig = 1.0 / g.g;
  if (j <= g.nhalf) {
    const double w1 = ROW(g.htw1, j), w2 = ROW(g.htw2, j);
    for (int i = 1 + threadIdx.x; i <= g.nlon; i += blockDim.x) {
      const size_t o = off_hlat(g, i, j);
      const double ub = aw.u_lat[o];
      const double m_lat = (mcell(g, s.gz, s.gzs, i, j) + mcell(g, s.gz, s.gzs, i, j + 1)) * 0.5;
      const double qb = ub / m_lat;
      aadd(&a.mfx_lon[off_full(g, i - 1, j)], w1 * qb);
      aadd(&a.mfx_lon[off_full(g, i, j)], w1 * qb);
      aadd(&a.mfx_lon[off_full(g, i - 1, j + 1)], w2 * qb);
      aadd(&a.mfx_lon[off_full(g, i, j + 1)], w2 * qb);
      const double mb = -w.u_lat[o] * qb * 0.5 * ig;
      aadd(&a.gz[off_full(g, i, j)], mb);
      aadd(&a.gz[off_full(g, i, j + 1)], mb);
    }
  }
  if (j == 1 || j == g.nlat) return;
  const double w1 = ROW(g.ftw1, j), w2 = ROW(g.ftw2, j);
  for (int i = 1 + threadIdx.x; i <= g.nlon; i += blockDim.x) {
    const size_t o = off_full(g, i, j);
    const double vb = aw.v_lon[o];
    const double m_lon = (mcell(g, s.gz, s.gzs, i, j) + mcell(g, s.gz, s.gzs, i + 1, j)) * 0.5;
    const double qb = vb / m_lon;
    aadd(&a.mfy_lat[off_hlat(g, i, j - 1)], w1 * qb);
    aadd(&a.mfy_lat[off_hlat(g, i + 1, j - 1)], w1 * qb);
    aadd(&a.mfy_lat[off_hlat(g, i, j)], w2 * qb);
    aadd(&a.mfy_lat[off_hlat(g, i + 1, j)], w2 * qb);
    const double mb = -w.v_lon[o] * qb * 0.5 * ig;
    aadd(&a.gz[off_full(g, i, j)], mb);
    aadd(&a.gz[off_full(g, i + 1, j)], mb);
  }
}

// ---------------------------------------------------------------------------
// calc_ke, ke_scheme 1 (the shallow-water setting); pole rows: ring mean of v^2
// ---------------------------------------------------------------------------
__global__ void k_tl_ke(DGrid g, Slot<double> s, Slot<double> t, Work<double> tw) {
  __shared__ double red[32];
  const int j = blockIdx.x + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  if (j == 1 || j == nlat) {
    const int jv = j == 1 ? 1 : nhalf;
    double p = ring_sum(nlon, red, [&](int i) { return 2.0 * s.v_f[off_hlat(g, i, jv)] * t.v_f[off_hlat(g, i, jv)]; });
    p = p / nlon;
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) tw.ke[off_full(g, i, j)] = p;
    return;
  }
  const double alw = ROW(g.area_lon_west, j), ale = ROW(g.area_lon_east, j);
  const double aln = ROW(g.area_lat_north, j - 1), als = ROW(g.area_lat_south, j), ac = ROW(g.area_cell, j);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const size_t uw = off_full(g, i - 1, j), ue = off_full(g, i, j), vs = off_hlat(g, i, j - 1), vn = off_hlat(g, i, j);
    tw.ke[off_full(g, i, j)] = 2.0 * (alw * s.u_f[uw] * t.u_f[uw] + ale * s.u_f[ue] * t.u_f[ue] +
                                      aln * s.v_f[vs] * t.v_f[vs] + als * s.v_f[vn] * t.v_f[vn]) / ac;
  }
}
__device__ __forceinline__ void ad_ke_body(DGrid g, Slot<double> s, Slot<double> a, Work<double> aw, int j) {
  __shared__ double red[32];
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  if (j == 1 || j == nlat) {
    const int jv = j == 1 ? 1 : nhalf;
    const double r = ring_sum(nlon, red, [&](int i) { return aw.ke[off_full(g, i, j)]; }) / nlon;
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      const size_t o = off_hlat(g, i, jv);
      aadd(&a.v_f[o], 2.0 * s.v_f[o] * r);
    }
    return;
  }
  const double alw = ROW(g.area_lon_west, j), ale = ROW(g.area_lon_east, j);
  const double aln = ROW(g.area_lat_north, j - 1), als = ROW(g.area_lat_south, j), ac = ROW(g.area_cell, j);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const double kb = 2.0 * aw.ke[off_full(g, i, j)] / ac;
    const size_t uw = off_full(g, i - 1, j), ue = off_full(g, i, j), vs = off_hlat(g, i, j - 1), vn = off_hlat(g, i, j);
    aadd(&a.u_f[uw], alw * s.u_f[uw] * kb);
    aadd(&a.u_f[ue], ale * s.u_f[ue] * kb);
    aadd(&a.v_f[vs], aln * s.v_f[vs] * kb);
    aadd(&a.v_f[vn], als * s.v_f[vn] * kb);
  }
}

// ---------------------------------------------------------------------------
// calc_vor + calc_pv: pv = (vor + f) / m_vtx; Stokes pole vertices from u_lat
// ---------------------------------------------------------------------------
__global__ void k_tl_pv(DGrid g, Slot<double> s, Slot<double> t, Work<double> tw) {
  __shared__ double red[32];
  const int j = blockIdx.x + 1;
  const int nhalf = g.nhalf, nlon = g.nlon;
  const double ig = 1.0 / g.g;
  const bool pole = g.pv_pole_stokes && (j == 1 || j == nhalf);
  double dpole = 0;
  if (pole) {
    const double le = ROW(g.le_lat, j), sgn = j == 1 ? -1.0 : 1.0;
    dpole = ring_sum(nlon, red, [&](int i) { return sgn * tw.u_lat[off_hlat(g, i, j)] * le; });
    dpole = dpole / nlon / ROW(g.area_cell, j == 1 ? 1 : nhalf + 1);
  }
  const double dl0 = ROW(g.de_lon, j), dl1 = ROW(g.de_lon, j + 1), dt = ROW(g.de_lat, j), av = ROW(g.area_vtx, j);
  const double as2 = ROW(g.area_subcell2, j), as1 = ROW(g.area_subcell1, j + 1);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    double dvor;
    if (pole)
      dvor = dpole;
    else
      dvor = (t.u_f[off_full(g, i, j)] * dl0 - t.u_f[off_full(g, i, j + 1)] * dl1 + t.v_f[off_hlat(g, i + 1, j)] * dt -
              t.v_f[off_hlat(g, i, j)] * dt) / av;
    const double m_vtx = ((mcell(g, s.gz, s.gzs, i, j) + mcell(g, s.gz, s.gzs, i + 1, j)) * as2 +
                          (mcell(g, s.gz, s.gzs, i, j + 1) + mcell(g, s.gz, s.gzs, i + 1, j + 1)) * as1) / av;
    const double dm_vtx = ((t.gz[off_full(g, i, j)] + t.gz[off_full(g, i + 1, j)]) * as2 +
                           (t.gz[off_full(g, i, j + 1)] + t.gz[off_full(g, i + 1, j + 1)]) * as1) * ig / av;
    const size_t o = off_hlat(g, i, j);
    t.pv[o] = (dvor - s.pv[o] * dm_vtx) / m_vtx;
  }
}
__device__ __forceinline__ void ad_pv_body(DGrid g, Slot<double> s, Slot<double> a, Work<double> aw, int j) {
  __shared__ double red[32];
  const int nhalf = g.nhalf, nlon = g.nlon;
  const double ig = 1.0 / g.g;
  const bool pole = g.pv_pole_stokes && (j == 1 || j == nhalf);
  const double dl0 = ROW(g.de_lon, j), dl1 = ROW(g.de_lon, j + 1), dt = ROW(g.de_lat, j), av = ROW(g.area_vtx, j);
  const double as2 = ROW(g.area_subcell2, j), as1 = ROW(g.area_subcell1, j + 1);
  double vsum = 0;   // pole: sum of vor adjoints over the ring
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const size_t o = off_hlat(g, i, j);
    const double m_vtx = ((mcell(g, s.gz, s.gzs, i, j) + mcell(g, s.gz, s.gzs, i + 1, j)) * as2 +
                          (mcell(g, s.gz, s.gzs, i, j + 1) + mcell(g, s.gz, s.gzs, i + 1, j + 1)) * as1) / av;
    const double pb = a.pv[o];
    const double vb = pb / m_vtx;
    const double mb = -s.pv[o] * vb * ig / av;   // adjoint of m_vtx times d m_vtx / d gz
    aadd(&a.gz[off_full(g, i, j)], mb * as2);
    aadd(&a.gz[off_full(g, i + 1, j)], mb * as2);
    aadd(&a.gz[off_full(g, i, j + 1)], mb * as1);
    aadd(&a.gz[off_full(g, i + 1, j + 1)], mb * as1);
    if (pole) {
      vsum += vb;
    } else {
      aadd(&a.u_f[off_full(g, i, j)], vb * dl0 / av);
      aadd(&a.u_f[off_full(g, i, j + 1)], -vb * dl1 / av);
      aadd(&a.v_f[off_hlat(g, i + 1, j)], vb * dt / av);
      aadd(&a.v_f[off_hlat(g, i, j)], -vb * dt / av);
    }
  }
  if (pole) {
    const double r = block_sum(vsum, red);
    const double le = ROW(g.le_lat, j), sgn = j == 1 ? -1.0 : 1.0;
    const double c = r * sgn * le / nlon / ROW(g.area_cell, j == 1 ? 1 : nhalf + 1);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) aadd(&aw.u_lat[off_hlat(g, i, j)], c);
  }
}

// ---------------------------------------------------------------------------
// interp_pv (midpoint; upwind order 1 or 3 blended by b = |vt| / (|V| + eps))
// ---------------------------------------------------------------------------
// d upwind / d f_q for q = 0..3 (order 3) or 0..1 (order 1)
__device__ __forceinline__ void upwind_coef(int order, double dir, double wgt, double c[4]) {
  if (order == 3) {
    const double c31 = 7.0 / 12.0, c32 = -1.0 / 12.0, c33 = 1.0 / 12.0;
    const double wd = c33 * wgt * dir;
    c[0] = c32 - wd;
    c[1] = c31 + 3.0 * wd;
    c[2] = c31 - 3.0 * wd;
    c[3] = c32 + wd;
  } else {
    c[0] = 0.5 + 0.5 * wgt * dir;
    c[1] = 0.5 - 0.5 * wgt * dir;
    c[2] = c[3] = 0;
  }
}
// b(un, vt) and its partial derivatives
__device__ __forceinline__ void blend_b(double un, double vt, double &b, double &db_dun, double &db_dvt) {
  const double eps = 2.220446049250313e-16;
  const double s2 = un * un + vt * vt, sq = sqrt(s2), D = sq + eps;
  b = fabs(vt) / D;
  const double dir = fsign(1.0, vt);
  const double dsq_dun = sq > 0 ? un / sq : 0.0, dsq_dvt = sq > 0 ? vt / sq : 0.0;
  db_dun = -b * dsq_dun / D;
  db_dvt = (dir - b * dsq_dvt) / D;
}

__global__ void k_tl_pv_edges(DGrid g, Slot<double> s, Work<double> w, Slot<double> t, Work<double> tw) {
  const int j = blockIdx.x + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon, ord = g.upwind_order_pv;
  const double wgt = g.upwind_wgt_pv;
  auto P = [&](int i, int jj) { return rd_half(s.pv, g, i, jj, 1); };
  auto dP = [&](int i, int jj) { return rd_half(t.pv, g, i, jj, 1); };
  if (j == 1 || j == nlat) {
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) t.pv_lon[off_full(g, i, j)] = 0;
  } else {
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      const size_t o = off_full(g, i, j);
      const double dmid = dP(i, j - 1) + dP(i, j);
      if (g.pv_scheme == GMC_PV_MIDPOINT) {
        t.pv_lon[o] = 0.5 * dmid;
        continue;
      }
      const double mid = P(i, j - 1) + P(i, j);
      const double un = s.u_f[o], vt = w.v_lon[o];
      double b, bu, bv;
      blend_b(un, vt, b, bu, bv);
      const double dir = fsign(1.0, vt);
      double c[4];
      upwind_coef(ord, dir, wgt, c);
      double up, dup;
      if (ord == 3) {
        up = upwind3(dir, wgt, P(i, j - 2), P(i, j - 1), P(i, j), P(i, j + 1));
        dup = c[0] * dP(i, j - 2) + c[1] * dP(i, j - 1) + c[2] * dP(i, j) + c[3] * dP(i, j + 1);
      } else {
        up = upwind1(dir, wgt, P(i, j - 1), P(i, j));
        dup = c[0] * dP(i, j - 1) + c[1] * dP(i, j);
      }
      const double db = bu * t.u_f[o] + bv * tw.v_lon[o];
      t.pv_lon[o] = db * (up - 0.5 * mid) + b * dup + (1.0 - b) * 0.5 * dmid;
    }
  }
  if (j > nhalf) return;
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const size_t o = off_hlat(g, i, j);
    const double dmid = dP(i - 1, j) + dP(i, j);
    if (g.pv_scheme == GMC_PV_MIDPOINT) {
      t.pv_lat[o] = 0.5 * dmid;
      continue;
    }
    const double mid = P(i - 1, j) + P(i, j);
    const double ut = w.u_lat[o], vn = s.v_f[o];
    double b, bt, bn;
    blend_b(vn, ut, b, bn, bt);   // b = |ut| / (|V| + eps): ut plays the tangential role
    const double dir = fsign(1.0, ut);
    double c[4];
    upwind_coef(ord, dir, wgt, c);
    double up, dup;
    if (ord == 3) {
      up = upwind3(dir, wgt, P(i - 2, j), P(i - 1, j), P(i, j), P(i + 1, j));
      dup = c[0] * dP(i - 2, j) + c[1] * dP(i - 1, j) + c[2] * dP(i, j) + c[3] * dP(i + 1, j);
    } else {
      up = upwind1(dir, wgt, P(i - 1, j), P(i, j));
      dup = c[0] * dP(i - 1, j) + c[1] * dP(i, j);
    }
    const double db = bt * tw.u_lat[o] + bn * t.v_f[o];
    t.pv_lat[o] = db * (up - 0.5 * mid) + b * dup + (1.0 - b) * 0.5 * dmid;
  }
}
__global__ void k_ad_pv_edges(DGrid g, Slot<double> s, Work<double> w, Slot<double> a, Work<double> aw) {
  const int j = blockIdx.x + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon, ord = g.upwind_order_pv;
  const double wgt = g.upwind_wgt_pv;
  auto P = [&](int i, int jj) { return rd_half(s.pv, g, i, jj, 1); };
  auto addP = [&](int i, int jj, double v) { aadd(&a.pv[off_half_halo(g, i, jj)], v); };
  if (j != 1 && j != nlat) {
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      const size_t o = off_full(g, i, j);
      const double yb = a.pv_lon[o];
      if (g.pv_scheme == GMC_PV_MIDPOINT) {
        addP(i, j - 1, 0.5 * yb);
        addP(i, j, 0.5 * yb);
        continue;
      }
      const double mid = P(i, j - 1) + P(i, j);
      const double un = s.u_f[o], vt = w.v_lon[o];
      double b, bu, bv;
      blend_b(un, vt, b, bu, bv);
      const double dir = fsign(1.0, vt);
      double c[4];
      upwind_coef(ord, dir, wgt, c);
      const double up = ord == 3 ? upwind3(dir, wgt, P(i, j - 2), P(i, j - 1), P(i, j), P(i, j + 1))
                                 : upwind1(dir, wgt, P(i, j - 1), P(i, j));
      const double bb = (up - 0.5 * mid) * yb, ub = b * yb, mb = (1.0 - b) * 0.5 * yb;
      if (ord == 3) {
        addP(i, j - 2, c[0] * ub);
        addP(i, j - 1, c[1] * ub + mb);
        addP(i, j, c[2] * ub + mb);
        addP(i, j + 1, c[3] * ub);
      } else {
        addP(i, j - 1, c[0] * ub + mb);
        addP(i, j, c[1] * ub + mb);
      }
      aadd(&a.u_f[o], bu * bb);
      aadd(&aw.v_lon[o], bv * bb);
    }
  }
  if (j > nhalf) return;
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const size_t o = off_hlat(g, i, j);
    const double yb = a.pv_lat[o];
    if (g.pv_scheme == GMC_PV_MIDPOINT) {
      addP(i - 1, j, 0.5 * yb);
      addP(i, j, 0.5 * yb);
      continue;
    }
    const double mid = P(i - 1, j) + P(i, j);
    const double ut = w.u_lat[o], vn = s.v_f[o];
    double b, bt, bn;
    blend_b(vn, ut, b, bn, bt);
    const double dir = fsign(1.0, ut);
    double c[4];
    upwind_coef(ord, dir, wgt, c);
    const double up = ord == 3 ? upwind3(dir, wgt, P(i - 2, j), P(i - 1, j), P(i, j), P(i + 1, j))
                               : upwind1(dir, wgt, P(i - 1, j), P(i, j));
    const double bb = (up - 0.5 * mid) * yb, ub = b * yb, mb = (1.0 - b) * 0.5 * yb;
    if (ord == 3) {
      addP(i - 2, j, c[0] * ub);
      addP(i - 1, j, c[1] * ub + mb);
      addP(i, j, c[2] * ub + mb);
      addP(i + 1, j, c[3] * ub);
    } else {
      addP(i - 1, j, c[0] * ub + mb);
      addP(i, j, c[1] * ub + mb);
    }
    aadd(&aw.u_lat[o], bt * bb);
    aadd(&a.v_f[o], bn * bb);
  }
}

// ---------------------------------------------------------------------------
// momentum tendencies of the shallow-water forward pass: Coriolis + grad KE
// ---------------------------------------------------------------------------
__global__ void k_tl_momentum(DGrid g, Slot<double> s, Slot<double> t, Work<double> tw) {
  const int j = blockIdx.x + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  auto MFX = [&](const double *f, int i, int jj) { return f[off_full(g, i, jj)]; };
  auto MFY = [&](const double *f, int i, int jj) { return f[off_hlat(g, i, jj)]; };
  if (j != 1 && j != nlat) {
    const double t1 = ROW(g.ftw1, j), t2 = ROW(g.ftw2, j), de = ROW(g.de_lon, j);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      const size_t o = off_full(g, i, j);
      const double pl = s.pv_lon[o], dpl = t.pv_lon[o];
      double dq;
      if (g.coriolis_scheme == 1) {
        auto term = [&](int ii, int jj) {
          return MFY(t.mfy_lat, ii, jj) * (pl + MFY(s.pv_lat, ii, jj)) + MFY(s.mfy_lat, ii, jj) * (dpl + MFY(t.pv_lat, ii, jj));
        };
        dq = (t1 * (term(i, j - 1) + term(i + 1, j - 1)) + t2 * (term(i, j) + term(i + 1, j))) * 0.5;
      } else {
        const double mf = t1 * (MFY(s.mfy_lat, i, j - 1) + MFY(s.mfy_lat, i + 1, j - 1)) + t2 * (MFY(s.mfy_lat, i, j) + MFY(s.mfy_lat, i + 1, j));
        const double dmf = t1 * (MFY(t.mfy_lat, i, j - 1) + MFY(t.mfy_lat, i + 1, j - 1)) + t2 * (MFY(t.mfy_lat, i, j) + MFY(t.mfy_lat, i + 1, j));
        dq = dmf * pl + mf * dpl;
      }
      tw.du[o] = dq - (tw.ke[off_full(g, i + 1, j)] - tw.ke[o]) / de;
    }
  }
  if (j > nhalf) return;
  const double t1 = ROW(g.htw1, j), t2 = ROW(g.htw2, j), de = ROW(g.de_lat, j);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const size_t o = off_hlat(g, i, j);
    const double pl = s.pv_lat[o], dpl = t.pv_lat[o];
    double dq;
    if (g.coriolis_scheme == 1) {
      auto term = [&](int ii, int jj) {
        return MFX(t.mfx_lon, ii, jj) * (pl + MFX(s.pv_lon, ii, jj)) + MFX(s.mfx_lon, ii, jj) * (dpl + MFX(t.pv_lon, ii, jj));
      };
      dq = (t1 * (term(i - 1, j) + term(i, j)) + t2 * (term(i - 1, j + 1) + term(i, j + 1))) * 0.5;
    } else {
      const double mf = t1 * (MFX(s.mfx_lon, i - 1, j) + MFX(s.mfx_lon, i, j)) + t2 * (MFX(s.mfx_lon, i - 1, j + 1) + MFX(s.mfx_lon, i, j + 1));
      const double dmf = t1 * (MFX(t.mfx_lon, i - 1, j) + MFX(t.mfx_lon, i, j)) + t2 * (MFX(t.mfx_lon, i - 1, j + 1) + MFX(t.mfx_lon, i, j + 1));
      dq = dmf * pl + mf * dpl;
    }
    tw.dv[o] = -dq - (tw.ke[off_full(g, i, j + 1)] - tw.ke[off_full(g, i, j)]) / de;
  }
}
__device__ __forceinline__ void ad_momentum_body(DGrid g, Slot<double> s, Slot<double> a, Work<double> aw, int j) {
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  if (j != 1 && j != nlat) {
    const double t1 = ROW(g.ftw1, j), t2 = ROW(g.ftw2, j), de = ROW(g.de_lon, j);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      const size_t o = off_full(g, i, j);
      const double qb = aw.du[o];
      aadd(&aw.ke[off_full(g, i + 1, j)], -qb / de);
      aadd(&aw.ke[o], qb / de);
      const double pl = s.pv_lon[o];
      if (g.coriolis_scheme == 1) {
        double plb = 0;
        auto term = [&](int ii, int jj, double c) {
          const size_t oh = off_hlat(g, ii, jj);
          aadd(&a.mfy_lat[oh], c * (pl + s.pv_lat[oh]));
          aadd(&a.pv_lat[oh], c * s.mfy_lat[oh]);
          plb += c * s.mfy_lat[oh];
        };
        term(i, j - 1, 0.5 * t1 * qb);
        term(i + 1, j - 1, 0.5 * t1 * qb);
        term(i, j, 0.5 * t2 * qb);
        term(i + 1, j, 0.5 * t2 * qb);
        aadd(&a.pv_lon[o], plb);
      } else {
        const double mf = t1 * (s.mfy_lat[off_hlat(g, i, j - 1)] + s.mfy_lat[off_hlat(g, i + 1, j - 1)]) +
                          t2 * (s.mfy_lat[off_hlat(g, i, j)] + s.mfy_lat[off_hlat(g, i + 1, j)]);
        aadd(&a.pv_lon[o], mf * qb);
        aadd(&a.mfy_lat[off_hlat(g, i, j - 1)], t1 * pl * qb);
        aadd(&a.mfy_lat[off_hlat(g, i + 1, j - 1)], t1 * pl * qb);
        aadd(&a.mfy_lat[off_hlat(g, i, j)], t2 * pl * qb);
        aadd(&a.mfy_lat[off_hlat(g, i + 1, j)], t2 * pl * qb);
      }
    }
  }
  if (j > nhalf) return;
  const double t1 = ROW(g.htw1, j), t2 = ROW(g.htw2, j), de = ROW(g.de_lat, j);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const size_t o = off_hlat(g, i, j);
    const double vb = aw.dv[o];
    aadd(&aw.ke[off_full(g, i, j + 1)], -vb / de);
    aadd(&aw.ke[off_full(g, i, j)], vb / de);
    const double qb = -vb;   // dv = -qhu - dkedlat
    const double pl = s.pv_lat[o];
    if (g.coriolis_scheme == 1) {
      double plb = 0;
      auto term = [&](int ii, int jj, double c) {
        const size_t of = off_full(g, ii, jj);
        aadd(&a.mfx_lon[of], c * (pl + s.pv_lon[of]));
        aadd(&a.pv_lon[of], c * s.mfx_lon[of]);
        plb += c * s.mfx_lon[of];
      };
      term(i - 1, j, 0.5 * t1 * qb);
      term(i, j, 0.5 * t1 * qb);
      term(i - 1, j + 1, 0.5 * t2 * qb);
      term(i, j + 1, 0.5 * t2 * qb);
      aadd(&a.pv_lat[o], plb);
    } else {
      const double mf = t1 * (s.mfx_lon[off_full(g, i - 1, j)] + s.mfx_lon[off_full(g, i, j)]) +
                        t2 * (s.mfx_lon[off_full(g, i - 1, j + 1)] + s.mfx_lon[off_full(g, i, j + 1)]);
      aadd(&a.pv_lat[o], mf * qb);
      aadd(&a.mfx_lon[off_full(g, i - 1, j)], t1 * pl * qb);
      aadd(&a.mfx_lon[off_full(g, i, j)], t1 * pl * qb);
      aadd(&a.mfx_lon[off_full(g, i - 1, j + 1)], t2 * pl * qb);
      aadd(&a.mfx_lon[off_full(g, i, j + 1)], t2 * pl * qb);
    }
  }
}

// ---------------------------------------------------------------------------
// adjoint of the shallow-water dgz = -(dmf/dlon + dmf/dlat) g with pole rings
// ---------------------------------------------------------------------------
__device__ __forceinline__ void ad_dgz_body(DGrid g, Slot<double> a, Work<double> aw, int j) {
  __shared__ double red[32];
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  if (j == 1 || j == nlat) {
    const int jv = j == 1 ? 1 : nhalf;
    const double sgn = j == 1 ? 1.0 : -1.0;
    const double r = ring_sum(nlon, red, [&](int i) { return aw.dgz[off_full(g, i, j)]; });
    const double c = -r * g.g * sgn * ROW(g.le_lat, jv) / nlon / ROW(g.area_cell, j);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) aadd(&a.mfy_lat[off_hlat(g, i, jv)], c);
    return;
  }
  const double lel = ROW(g.le_lon, j), ac = ROW(g.area_cell, j), la0 = ROW(g.le_lat, j), la1 = ROW(g.le_lat, j - 1);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const double b = -aw.dgz[off_full(g, i, j)] * g.g;   // adjoint of (dlon + dlat)
    aadd(&a.mfx_lon[off_full(g, i, j)], b * lel / ac);
    aadd(&a.mfx_lon[off_full(g, i - 1, j)], -b * lel / ac);
    aadd(&a.mfy_lat[off_hlat(g, i, j)], b * la0 / ac);
    aadd(&a.mfy_lat[off_hlat(g, i, j - 1)], -b * la1 / ac);
  }
}

// ---------------------------------------------------------------------------
// transposed polar filter of one row held in shared memory: y^T = F^T y,
// (F^T y)(l) = sum_t w_t y(l + hn - t)  (reversed taps of the forward filter)
// ---------------------------------------------------------------------------
__device__ bool filter_row_t(const FilterDev &f, bool full_lat, int j, int nlon, double *row, double *ext) {
  const int n = full_lat ? f.ntaps_full[j - 1] : f.ntaps_half[j - 1];
  if (n <= 1) return false;
  const int hn = (n - 1) / 2;
  const double *w = f.wgt + (full_lat ? f.off_full[j - 1] : f.off_half[j - 1]);
  __syncthreads();
  for (int t = threadIdx.x; t < nlon + 2 * hn; t += blockDim.x) {
    int i = t - hn + 1;
    i = i < 1 ? i + nlon : (i > nlon ? i - nlon : i);
    ext[t] = row[i - 1];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    double s = 0;
    for (int t = 0; t < n; ++t) s = s + w[n - 1 - t] * ext[i + t];
    row[i] = s;
  }
  __syncthreads();
  return true;
}

// update_gz adjoint: t = gz_o + dt dgz; gz_f = big(t); gz = small1(t).
// Also clears the new slot's u/v adjoints (consumed by k_ad_uv) and the
// adjoint work range [zero, zero + nzero) the forward-pass adjoint
// accumulates into.
__global__ void k_ad_update_gz(DGrid g, Slot<double> ao, Slot<double> an, Work<double> aw, double dt, double *zero,
                               size_t nzero) {
  extern __shared__ double sh[];
  const int j = blockIdx.x + 1, nlon = g.nlon;
  double *r1 = sh, *r2 = sh + nlon, *ext = r2 + nlon;
  const size_t c0 = (size_t)(j - 1) * nlon;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nzero; t += (size_t)gridDim.x * blockDim.x) zero[t] = 0;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    an.u_lon[c0 + i] = 0;
    an.u_f[c0 + i] = 0;
    if (j <= g.nhalf) {
      an.v_lat[c0 + i] = 0;
      an.v_f[c0 + i] = 0;
    }
  }
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    r1[i] = an.gz_f[c0 + i];
    r2[i] = an.gz[c0 + i];
  }
  filter_row_t(g.big, true, j, nlon, r1, ext);
  filter_row_t(g.small1, true, j, nlon, r2, ext);
  __syncthreads();
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    const double tb = r1[i] + r2[i];
    ao.gz[c0 + i] += tb;
    aw.dgz[c0 + i] = dt * tb;
    an.gz_f[c0 + i] = 0;
    an.gz[c0 + i] = 0;
  }
}

// update_uv adjoint.  Forward rows: t = old + dt (tend - pgf) with
// pgf = d gz_f / d edge; u = t, u_f = big(u) (pole rows of u untouched);
// v(1) = 0.4 t(1) + 0.6 t(2), v(nhalf) = 0.4 t(nhalf) + 0.6 t(nhalf-1), other
// rows v = t; v_f = big(v).  A block takes one u row or one v row; the v rows
// next to the pole rows also form the pole rows' adjoint (their blend
// partner).  The new slot's u/v adjoints are read here and cleared later by
// k_ad_update_gz.
__device__ void ad_v_post(const DGrid &g, const Slot<double> &an, int j, double *row, double *ext) {
  // row <- adjoint of the blended v row j: v_n_bar + big^T(v_f_n_bar)
  const size_t c0 = (size_t)(j - 1) * g.nlon;
  __syncthreads();
  for (int i = threadIdx.x; i < g.nlon; i += blockDim.x) row[i] = an.v_f[c0 + i];
  filter_row_t(g.big, false, j, g.nlon, row, ext);
  __syncthreads();
  for (int i = threadIdx.x; i < g.nlon; i += blockDim.x) row[i] += an.v_lat[c0 + i];
  __syncthreads();
}
__global__ void k_ad_uv(DGrid g, Slot<double> ao, Slot<double> an, Work<double> aw, double dt) {
  extern __shared__ double sh[];
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  double *row = sh, *row2 = sh + nlon, *ext = row2 + nlon;
  if ((int)blockIdx.x < nlat) {
    const int j = blockIdx.x + 1;
    if (j == 1 || j == nlat) return;   // pole rows of u are not updated: their adjoint ends here
    const size_t c0 = (size_t)(j - 1) * nlon;
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) row[i] = an.u_f[c0 + i];
    filter_row_t(g.big, true, j, nlon, row, ext);
    __syncthreads();
    const double de = ROW(g.de_lon, j);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      const size_t o = off_full(g, i, j);
      const double tb = row[i - 1] + an.u_lon[o];
      ao.u_lon[o] += tb;
      aw.du[o] = dt * tb;
      const double pb = -dt * tb / de;   // pgf = (gz_f(i+1) - gz_f(i)) / de
      aadd(&an.gz_f[off_full(g, i + 1, j)], pb);
      aadd(&an.gz_f[o], -pb);
    }
    return;
  }
  const int j = blockIdx.x - nlat + 1;
  const double wgt = 0.6;
  ad_v_post(g, an, j, row, ext);
  const bool with_s = j == 2, with_n = j == nhalf - 1;   // partner of a pole row
  if (with_s || with_n) ad_v_post(g, an, with_s ? 1 : nhalf, row2, ext);
  const double de = ROW(g.de_lat, j);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const size_t o = off_hlat(g, i, j);
    double tb = (j == 1 || j == nhalf) ? (1.0 - wgt) * row[i - 1] : row[i - 1];
    if (with_s || with_n) tb += wgt * row2[i - 1];
    ao.v_lat[o] += tb;
    aw.dv[o] = dt * tb;
    const double pb = -dt * tb / de;   // pgf = (gz_f(i, j+1) - gz_f(i, j)) / de
    aadd(&an.gz_f[off_full(g, i, j + 1)], pb);
    aadd(&an.gz_f[off_full(g, i, j)], -pb);
  }
}

// adjoint of the prologue filters u_f = big(u), v_f = big(v), gz_f = big(gz)
__global__ void k_ad_prologue(DGrid g, Slot<double> a) {
  extern __shared__ double sh[];
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  double *row = sh, *ext = sh + nlon;
  const int which = blockIdx.y;   // 0 u, 1 v, 2 gz
  const int j = blockIdx.x + 1;
  if (which == 1 && j > nhalf) return;
  double *src = which == 0 ? a.u_f : which == 1 ? a.v_f : a.gz_f;
  double *dst = which == 0 ? a.u_lon : which == 1 ? a.v_lat : a.gz;
  const size_t c0 = (size_t)(j - 1) * nlon;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) row[i] = src[c0 + i];
  filter_row_t(g.big, which != 1, j, nlon, row, ext);
  __syncthreads();
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    dst[c0 + i] += row[i];
    src[c0 + i] = 0;
  }
}

// fused launches of the adjoint forward pass (one block per full row)
__global__ void k_ad_dgz_momentum(DGrid g, Slot<double> s, Slot<double> a, Work<double> aw) {
  const int j = blockIdx.x + 1;
  ad_dgz_body(g, a, aw, j);
  ad_momentum_body(g, s, a, aw, j);
}
__global__ void k_ad_pv_ke(DGrid g, Slot<double> s, Slot<double> a, Work<double> aw) {
  const int j = blockIdx.x + 1;
  if (j <= g.nhalf) ad_pv_body(g, s, a, aw, j);
  ad_ke_body(g, s, a, aw, j);
}

inline size_t row_smem(const DGrid &g, int rows) {
  int hmax = (g.big.max_taps - 1) / 2;
  return (size_t)(rows * g.nlon + g.nlon + 2 * hmax + 8) * sizeof(double);
}

}  // namespace

void tl_forward_prepare(const DGrid &g, const Launch &L, const Slot<double> &s, const Work<double> &w,
                        const Slot<double> &t, const Work<double> &tw) {
  k_tl_mass_flux<<<g.nlat, L.threads, 0, L.stream>>>(g, s, t);
  k_tl_tangent<<<g.nlat, L.threads, 0, L.stream>>>(g, s, w, t, tw);
  k_tl_ke<<<g.nlat, L.threads, 0, L.stream>>>(g, s, t, tw);
  k_tl_pv<<<g.nhalf, L.threads, 0, L.stream>>>(g, s, t, tw);
  k_tl_pv_edges<<<g.nlat, L.threads, 0, L.stream>>>(g, s, w, t, tw);
}
void tl_momentum(const DGrid &g, const Launch &L, const Slot<double> &s, const Slot<double> &t, const Work<double> &tw) {
  k_tl_momentum<<<g.nlat, L.threads, 0, L.stream>>>(g, s, t, tw);
}
void ad_update(const DGrid &g, const Launch &L, const Slot<double> &ao, const Slot<double> &an, const Work<double> &aw,
               double *zero, size_t nzero, double dt) {
  allow_smem(k_ad_uv, row_smem(g, 2));
  allow_smem(k_ad_update_gz, row_smem(g, 2));
  k_ad_uv<<<g.nlat + g.nhalf, L.threads, row_smem(g, 2), L.stream>>>(g, ao, an, aw, dt);
  k_ad_update_gz<<<g.nlat, L.threads, row_smem(g, 2), L.stream>>>(g, ao, an, aw, dt, zero, nzero);
}
void ad_forward(const DGrid &g, const Launch &L, const Slot<double> &s, const Work<double> &w, const Slot<double> &a,
                const Work<double> &aw) {
  k_ad_dgz_momentum<<<g.nlat, L.threads, 0, L.stream>>>(g, s, a, aw);
  k_ad_pv_edges<<<g.nlat, L.threads, 0, L.stream>>>(g, s, w, a, aw);
  k_ad_pv_ke<<<g.nlat, L.threads, 0, L.stream>>>(g, s, a, aw);
  k_ad_tangent<<<g.nlat, L.threads, 0, L.stream>>>(g, s, w, a, aw);
  k_ad_mass_flux<<<g.nlat, L.threads, 0, L.stream>>>(g, s, a);
}
void ad_prologue(const DGrid &g, const Launch &L, const Slot<double> &a) {
  allow_smem(k_ad_prologue, row_smem(g, 1));
  k_ad_prologue<<<dim3(g.nlat, 3), L.threads, row_smem(g, 1), L.stream>>>(g, a);
}

}  // namespace gmc
