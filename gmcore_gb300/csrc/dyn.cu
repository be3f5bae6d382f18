// Dynamics kernels of one forward-backward stage on the lat-lon C-grid.
//
// Most kernels run one thread block per latitude row and level (grid
// = rows x levels): a row is contiguous in HBM, pole rows reduce their ring
// inside the block, and row filters keep the whole row in shared memory.
// Column kernels (vertical sweeps) run one thread per (i, j) column.
// Reference routines are cited per kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "kernels.hpp"
#include "stencil.cuh"

namespace gmc {

namespace {

template <class R>
__device__ __forceinline__ MassField<R> mass_of(const DGrid &g, const Slot<R> &s) {
  return MassField<R>{s.surf(), s.gz, s.gzs};
}

// ---------------------------------------------------------------------------
// calc_mf (operators_mod.F90:545-583): mfx_lon = m_lon u, mfy_lat = m_lat v
// with m_lon, m_lat the edge averages of the cell mass
// (interp_mod.F90:233-275).  Pole rows of mfx_lon stay zero.
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ LevMass<R> lev_mass(const DGrid &g, const Slot<R> &s, int k) {
  return LevMass<R>(g, s.surf(), s.gz, s.gzs, k);
}

template <class R, bool MB>
__global__ void GMC_BOUNDS(R, 8) k_mass_flux(DGrid g, Slot<R> s) {
  if constexpr (MB) { to_member(g, s); }   // member-batched launches
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  const LevMass<R> M = lev_mass(g, s, k);
  const unsigned fo = (unsigned)ix3(nlat, nlon, 1, j, k), ho = (unsigned)ix3(nhalf, nlon, 1, j, k);
  const unsigned mo = (unsigned)(j - 1) * nlon;   // cell row j of the 2D mass field
  if constexpr (std::is_same<R, float>::value) {
    if (g.baroclinic) {   // two points per thread, paired loads (layer mass dA + dB psr)
      const float dA = g.dmA[k - 1], dB = g.dmB[k - 1];
      for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x) {
        const float2 p0 = *reinterpret_cast<const float2 *>(s.psr + mo + i0);
        const float m0 = fmaf(dB, p0.x, dA), m1 = fmaf(dB, p0.y, dA);
        if (j == 1 || j == nlat) {
          *reinterpret_cast<float2 *>(s.mfx_lon + fo + i0) = make_float2(0.0f, 0.0f);
        } else {
          const float m2 = fmaf(dB, s.psr[mo + (i0 + 2 == nlon ? 0 : i0 + 2)], dA);
          const float2 u2 = *reinterpret_cast<const float2 *>(s.u_f + fo + i0);
          *reinterpret_cast<float2 *>(s.mfx_lon + fo + i0) = make_float2((m0 + m1) * 0.5f * u2.x, (m1 + m2) * 0.5f * u2.y);
        }
        if (j <= nhalf) {
          const float2 pn = *reinterpret_cast<const float2 *>(s.psr + mo + nlon + i0);
          const float2 v2 = *reinterpret_cast<const float2 *>(s.v_f + ho + i0);
          *reinterpret_cast<float2 *>(s.mfy_lat + ho + i0) =
              make_float2((m0 + fmaf(dB, pn.x, dA)) * 0.5f * v2.x, (m1 + fmaf(dB, pn.y, dA)) * 0.5f * v2.y);
        }
      }
      return;
    }
  }
  if (j == 1 || j == nlat) {
    for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) s.mfx_lon[fo + i0] = (R)0;
  } else {
    for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) {
      const int ip = i0 + 1 == nlon ? 0 : i0 + 1;
      s.mfx_lon[fo + i0] = (M.at(mo + i0) + M.at(mo + ip)) * (R)0.5 * s.u_f[fo + i0];
    }
  }
  if (j <= nhalf) {
    for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x)
      s.mfy_lat[ho + i0] = (M.at(mo + i0) + M.at(mo + nlon + i0)) * (R)0.5 * s.v_f[ho + i0];
  }
}

// FP32 tangential winds (operators_mod.F90:585-605) of two neighbouring points
// (0-based i0, i0+1) of a row at one level, over the edge mass dA + dB psr:
// v_lon on full row j from the meridional mass fluxes of half rows j-1 (hs) and
// j (hn); u_lat on half row j from the zonal mass fluxes of full rows j (fs) and
// j+1 (fn); mo: row j of the 2-D surface pressure.  Shared by the tangent-wind
// kernel and the edge PV, which forms them itself where each value has one
// reader (tangent_inline).
struct TangentRow {
  float w1, w2, dA, dB;
  unsigned a, b, mo;   // v_lon: hs, hn; u_lat: fs, fn
};
__device__ __forceinline__ float2 vlon_pair(const TangentRow &t, const float *__restrict__ mfy,
                                            const float *__restrict__ psr, int nlon, int i0) {
  const unsigned i2 = i0 + 2 == nlon ? 0 : i0 + 2;
  const float2 ys = *reinterpret_cast<const float2 *>(mfy + t.a + i0), yn = *reinterpret_cast<const float2 *>(mfy + t.b + i0);
  const float yse = mfy[t.a + i2], yne = mfy[t.b + i2];
  const float2 pc = *reinterpret_cast<const float2 *>(psr + t.mo + i0);
  const float pe = psr[t.mo + i2];
  const float mf0 = t.w1 * (ys.x + ys.y) + t.w2 * (yn.x + yn.y), mf1 = t.w1 * (ys.y + yse) + t.w2 * (yn.y + yne);
  const float ml0 = (fmaf(t.dB, pc.x, t.dA) + fmaf(t.dB, pc.y, t.dA)) * 0.5f;
  const float ml1 = (fmaf(t.dB, pc.y, t.dA) + fmaf(t.dB, pe, t.dA)) * 0.5f;
  return make_float2(fdiv(mf0, ml0), fdiv(mf1, ml1));
}
__device__ __forceinline__ float2 ulat_pair(const TangentRow &t, const float *__restrict__ mfx,
                                            const float *__restrict__ psr, int nlon, int i0) {
  const unsigned im = i0 == 0 ? nlon - 1 : i0 - 1;
  const float2 xs = *reinterpret_cast<const float2 *>(mfx + t.a + i0), xn = *reinterpret_cast<const float2 *>(mfx + t.b + i0);
  const float xsw = mfx[t.a + im], xnw = mfx[t.b + im];
  const float2 ps = *reinterpret_cast<const float2 *>(psr + t.mo + i0), pn = *reinterpret_cast<const float2 *>(psr + t.mo + nlon + i0);
  const float mf0 = t.w1 * (xsw + xs.x) + t.w2 * (xnw + xn.x), mf1 = t.w1 * (xs.x + xs.y) + t.w2 * (xn.x + xn.y);
  const float ml0 = (fmaf(t.dB, ps.x, t.dA) + fmaf(t.dB, pn.x, t.dA)) * 0.5f;
  const float ml1 = (fmaf(t.dB, ps.y, t.dA) + fmaf(t.dB, pn.y, t.dA)) * 0.5f;
  return make_float2(fdiv(mf0, ml0), fdiv(mf1, ml1));
}
// u_lat at one point (the first component of ulat_pair at i0)
__device__ __forceinline__ float ulat_at(const TangentRow &t, const float *__restrict__ mfx, const float *__restrict__ psr,
                                         int nlon, int i0) {
  const unsigned im = i0 == 0 ? nlon - 1 : i0 - 1;
  const float mf0 = t.w1 * (mfx[t.a + im] + mfx[t.a + i0]) + t.w2 * (mfx[t.b + im] + mfx[t.b + i0]);
  const float ml0 = (fmaf(t.dB, psr[t.mo + i0], t.dA) + fmaf(t.dB, psr[t.mo + nlon + i0], t.dA)) * 0.5f;
  return fdiv(mf0, ml0);
}
__device__ __forceinline__ TangentRow vlon_row(const DGrid &g, int j, int k) {
  const unsigned hn = (unsigned)ix3(g.nhalf, g.nlon, 1, j, k);
  return {ROWR(float, ftw1, j), ROWR(float, ftw2, j), g.dmA[k - 1], g.dmB[k - 1], hn - g.nlon, hn, (unsigned)(j - 1) * g.nlon};
}
__device__ __forceinline__ TangentRow ulat_row(const DGrid &g, int j, int k) {
  const unsigned fs = (unsigned)ix3(g.nlat, g.nlon, 1, j, k);
  return {ROWR(float, htw1, j), ROWR(float, htw2, j), g.dmA[k - 1], g.dmB[k - 1], fs, fs + g.nlon, (unsigned)(j - 1) * g.nlon};
}

// Tangential mass fluxes and winds (operators_mod.F90:585-605).
template <class R, bool MB>
__global__ void GMC_BOUNDS_MB(R, 8, MB) k_tangent_winds(DGrid g, Slot<R> s, Work<R> w) {
  if constexpr (MB) { to_member(g, s); to_member(g, w); }   // member-batched launches
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  const LevMass<R> M = lev_mass(g, s, k);
  const unsigned mo = (unsigned)(j - 1) * nlon;
  if constexpr (std::is_same<R, float>::value) {
    if (g.baroclinic) {   // two points per thread, paired loads
      if (j <= nhalf) {
        const TangentRow t = ulat_row(g, j, k);
        const unsigned ho = (unsigned)ix3(nhalf, nlon, 1, j, k);
        for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x)
          *reinterpret_cast<float2 *>(w.u_lat + ho + i0) = ulat_pair(t, s.mfx_lon, s.psr, nlon, i0);
      }
      const unsigned fo = (unsigned)ix3(nlat, nlon, 1, j, k);
      if (j == 1 || j == nlat) {
        for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x)
          *reinterpret_cast<float2 *>(w.v_lon + fo + i0) = make_float2(0.0f, 0.0f);
      } else {
        const TangentRow t = vlon_row(g, j, k);
        for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x)
          *reinterpret_cast<float2 *>(w.v_lon + fo + i0) = vlon_pair(t, s.mfy_lat, s.psr, nlon, i0);
      }
      return;
    }
  }
  if (j <= nhalf) {
    const R w1 = ROWR(R, htw1, j), w2 = ROWR(R, htw2, j);
    const unsigned fs = (unsigned)ix3(nlat, nlon, 1, j, k), fn = fs + nlon, ho = (unsigned)ix3(nhalf, nlon, 1, j, k);
    for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) {
      const int im = i0 == 0 ? nlon - 1 : i0 - 1;
      R mfx_lat = w1 * (s.mfx_lon[fs + im] + s.mfx_lon[fs + i0]) + w2 * (s.mfx_lon[fn + im] + s.mfx_lon[fn + i0]);
      R m_lat = (M.at(mo + i0) + M.at(mo + nlon + i0)) * (R)0.5;
      w.u_lat[ho + i0] = fdiv(mfx_lat, m_lat);
    }
  }
  const unsigned fo = (unsigned)ix3(nlat, nlon, 1, j, k);
  if (j == 1 || j == nlat) {
    for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) w.v_lon[fo + i0] = (R)0;
  } else {
    const R w1 = ROWR(R, ftw1, j), w2 = ROWR(R, ftw2, j);
    const unsigned hn = (unsigned)ix3(nhalf, nlon, 1, j, k), hs = hn - nlon;
    for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) {
      const int ip = i0 + 1 == nlon ? 0 : i0 + 1;
      R mfy_lon = w1 * (s.mfy_lat[hs + i0] + s.mfy_lat[hs + ip]) + w2 * (s.mfy_lat[hn + i0] + s.mfy_lat[hn + ip]);
      R m_lon = (M.at(mo + i0) + M.at(mo + ip)) * (R)0.5;
      w.v_lon[fo + i0] = fdiv(mfy_lon, m_lon);
    }
  }
}

// calc_ke (operators_mod.F90:234-352): cell KE, optionally blended with the
// four vertex KEs (ke_scheme 2); pole cells take the ring mean of v^2.
template <class R, bool MB>
__global__ void GMC_BOUNDS(R, 5) k_kinetic_energy(DGrid g, Slot<R> s, Work<R> w) {
  if constexpr (MB) { to_member(g, s); to_member(g, w); }   // member-batched launches
  __shared__ double red[32];
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const R *u = s.u_f, *v = s.v_f;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  if (j == 1 || j == nlat) {
    const int jv = j == 1 ? 1 : nhalf;
    double p = ring_sum(nlon, red, [&](int i) {
      double x = (double)v[ix3(nhalf, nlon, i, jv, k)];
      return x * x;
    });
    p = p / nlon;
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) w.ke[ix3(nlat, nlon, i, j, k)] = (R)p;
    return;
  }
  auto sq = [](R x) { return x * x; };
  const R alw = ROWR(R, area_lon_west, j), ale = ROWR(R, area_lon_east, j);
  const R aln = ROWR(R, area_lat_north, j - 1), als = ROWR(R, area_lat_south, j), ac = ROWR(R, area_cell, j);
  // row offsets at level k: u on full rows j-1, j, j+1; v on half rows j-1, j
  const unsigned uc = (unsigned)ix3(nlat, nlon, 1, j, k), us = uc - nlon, un = uc + nlon;
  const unsigned vc = (unsigned)ix3(nhalf, nlon, 1, j, k), vs = vc - nlon;
  const bool vtx = g.ke_scheme == 2;
  const R cw = SCALR(R, ke_cell_wgt);
  const R ate = ROWR(R, area_lat_east, j), atw = ROWR(R, area_lat_west, j), ate1 = ROWR(R, area_lat_east, j - 1),
          atw1 = ROWR(R, area_lat_west, j - 1);
  const R aon = ROWR(R, area_lon_north, j), aon1 = ROWR(R, area_lon_north, j - 1), aos = ROWR(R, area_lon_south, j),
          aosn = ROWR(R, area_lon_south, j + 1);
  const R av = ROWR(R, area_vtx, j), av1 = ROWR(R, area_vtx, j - 1), as2 = ROWR(R, area_subcell2, j),
          as1 = ROWR(R, area_subcell1, j);
  if constexpr (std::is_same<R, float>::value) {
    // Two points per thread (i0, i0+1): each row's columns i0-1 .. i0+2 as one
    // paired load and the scalars around it; the per-point arithmetic below is
    // the single-point form's.
    for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x) {
      const int im = i0 == 0 ? nlon - 1 : i0 - 1, i2 = i0 + 2 == nlon ? 0 : i0 + 2;
      auto P2 = [&](const float *p, unsigned o) { return *reinterpret_cast<const float2 *>(p + o + i0); };
      const float2 uc2 = P2(u, uc), un2 = P2(u, un), us2 = P2(u, us), vc2 = P2(v, vc), vs2 = P2(v, vs);
      const float ucw = u[uc + im], unw = u[un + im], usw = u[us + im];
      const float vcw = v[vc + im], vsw = v[vs + im], vce = v[vc + i2], vse = v[vs + i2];
      float out[2];
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        // columns im, i0, ip of point i0 + p
        const float uw = p ? uc2.x : ucw, ue = p ? uc2.y : uc2.x;
        const float vsc = p ? vs2.y : vs2.x, vnc = p ? vc2.y : vc2.x;
        float ke = fdiv(alw * sq(uw) + ale * sq(ue) + aln * sq(vsc) + als * sq(vnc), ac);
        if (vtx) {
          const float v_cm = p ? vc2.x : vcw, v_sm = p ? vs2.x : vsw, v_sp = p ? vse : vs2.y, v_cp = p ? vce : vc2.y;
          const float u_nm = p ? un2.x : unw, u_sm = p ? us2.x : usw, u_s0 = p ? us2.y : us2.x, u_n0 = p ? un2.y : un2.x;
          const float k1 = fdiv(ate * sq(v_cm) + atw * sq(vnc) + aon * sq(uw) + aosn * sq(u_nm), av);
          const float k2 = fdiv(ate1 * sq(v_sm) + atw1 * sq(vsc) + aon1 * sq(u_sm) + aos * sq(uw), av1);
          const float k3 = fdiv(ate1 * sq(vsc) + atw1 * sq(v_sp) + aon1 * sq(u_s0) + aos * sq(ue), av1);
          const float k4 = fdiv(ate * sq(vnc) + atw * sq(v_cp) + aon * sq(ue) + aosn * sq(u_n0), av);
          ke = fdiv((1.0f - cw) * ((k1 + k4) * as2 + (k2 + k3) * as1), ac) + cw * ke;
        }
        out[p] = ke;
      }
      *reinterpret_cast<float2 *>(w.ke + uc + i0) = make_float2(out[0], out[1]);
    }
    return;
  }
  for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) {
    const int im = i0 == 0 ? nlon - 1 : i0 - 1, ip = i0 + 1 == nlon ? 0 : i0 + 1;
    const R uw = u[uc + im], ue = u[uc + i0], vsc = v[vs + i0], vnc = v[vc + i0];
    R ke = fdiv(alw * sq(uw) + ale * sq(ue) + aln * sq(vsc) + als * sq(vnc), ac);
    if (vtx) {
      const R k1 = fdiv(ate * sq(v[vc + im]) + atw * sq(vnc) + aon * sq(uw) + aosn * sq(u[un + im]), av);
      const R k2 = fdiv(ate1 * sq(v[vs + im]) + atw1 * sq(vsc) + aon1 * sq(u[us + im]) + aos * sq(uw), av1);
      const R k3 = fdiv(ate1 * sq(vsc) + atw1 * sq(v[vs + ip]) + aon1 * sq(u[us + i0]) + aos * sq(ue), av1);
      const R k4 = fdiv(ate * sq(vnc) + atw * sq(v[vc + ip]) + aon * sq(ue) + aosn * sq(u[un + i0]), av);
      ke = fdiv(((R)1 - cw) * ((k1 + k4) * as2 + (k2 + k3) * as1), ac) + cw * ke;
    }
    w.ke[uc + i0] = ke;
  }
}

// calc_vor + calc_pv (operators_mod.F90:612-703) with the vertex mass of
// interp_cell_to_vtx (interp_mod.F90:438-463).
template <class R, bool MB>
__global__ void GMC_BOUNDS(R, 6) k_pv(DGrid g, Slot<R> s, Work<R> w) {
  if constexpr (MB) { to_member(g, s); to_member(g, w); }   // member-batched launches
  __shared__ double red[32];
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  const bool pole = g.pv_pole_stokes && (j == 1 || j == nhalf);
  double pole_vor = 0;
  if (pole) {
    const double le = ROW(g.le_lat, j);
    const double sgn = j == 1 ? -1.0 : 1.0;
    double p;
    if constexpr (std::is_same<R, float>::value) {
      if (g.tangent_inline) {   // u_lat of the pole half row, formed here
        const TangentRow t = ulat_row(g, j, k);
        p = ring_sum(nlon, red, [&](int i) { return sgn * (double)ulat_at(t, s.mfx_lon, s.psr, nlon, i - 1) * le; });
      } else {
        p = ring_sum(nlon, red, [&](int i) { return sgn * (double)w.u_lat[ix3(nhalf, nlon, i, j, k)] * le; });
      }
    } else {
      p = ring_sum(nlon, red, [&](int i) { return sgn * (double)w.u_lat[ix3(nhalf, nlon, i, j, k)] * le; });
    }
    pole_vor = p / nlon / ROW(g.area_cell, j == 1 ? 1 : nhalf + 1);
  }
  const R dl0 = ROWR(R, de_lon, j), dl1 = ROWR(R, de_lon, j + 1), dt = ROWR(R, de_lat, j), av = ROWR(R, area_vtx, j);
  const R as2 = ROWR(R, area_subcell2, j), as1 = ROWR(R, area_subcell1, j + 1), f = ROWR(R, half_f, j);
  const LevMass<R> LM = lev_mass(g, s, k);
  const unsigned us = (unsigned)ix3(nlat, nlon, 1, j, k), un = us + nlon, ho = (unsigned)ix3(nhalf, nlon, 1, j, k);
  const unsigned ms = (unsigned)(j - 1) * nlon, mn = ms + nlon;
  if constexpr (std::is_same<R, float>::value) {
    if (g.baroclinic) {   // two points per thread, paired loads
      const float dA = g.dmA[k - 1], dB = g.dmB[k - 1];
      auto P2 = [](const float *p, unsigned o) { return *reinterpret_cast<const float2 *>(p + o); };
      for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x) {
        const unsigned i2 = i0 + 2 == nlon ? 0 : i0 + 2;
        const float2 vv = P2(s.v_f, ho + i0);
        const float ve = s.v_f[ho + i2];
        float vor0, vor1;
        if (pole) {
          vor0 = vor1 = (float)pole_vor;
        } else {
          const float2 u0 = P2(s.u_f, us + i0), u1 = P2(s.u_f, un + i0);
          vor0 = fdiv(u0.x * dl0 - u1.x * dl1 + vv.y * dt - vv.x * dt, av);
          vor1 = fdiv(u0.y * dl0 - u1.y * dl1 + ve * dt - vv.y * dt, av);
        }
        const float2 a2 = P2(s.psr, ms + i0), b2 = P2(s.psr, mn + i0);
        const float ae = fmaf(dB, s.psr[ms + i2], dA), be = fmaf(dB, s.psr[mn + i2], dA);
        const float a0 = fmaf(dB, a2.x, dA), a1 = fmaf(dB, a2.y, dA), b0 = fmaf(dB, b2.x, dA), b1 = fmaf(dB, b2.y, dA);
        const float mv0 = fdiv((a0 + a1) * as2 + (b0 + b1) * as1, av), mv1 = fdiv((a1 + ae) * as2 + (b1 + be) * as1, av);
        *reinterpret_cast<float2 *>(s.pv + ho + i0) = make_float2(fdiv(vor0 + f, mv0), fdiv(vor1 + f, mv1));
      }
      return;
    }
  }
  for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) {
    const int ip = i0 + 1 == nlon ? 0 : i0 + 1;
    R vor;
    if (pole) {
      vor = (R)pole_vor;
    } else {
      vor = fdiv(s.u_f[us + i0] * dl0 - s.u_f[un + i0] * dl1 + s.v_f[ho + ip] * dt - s.v_f[ho + i0] * dt, av);
    }
    R m_vtx = fdiv((LM.at(ms + i0) + LM.at(ms + ip)) * as2 + (LM.at(mn + i0) + LM.at(mn + ip)) * as1, av);
    s.pv[ho + i0] = fdiv(vor + f, m_vtx);
  }
}


// interp_pv_midpoint / interp_pv_upwind (operators_mod.F90:705-795).  The
// half rows of pv a block reads are resolved once per block (row offset and
// the longitude shift of the rows mirrored beyond the poles, as rd_half reads
// them), so the per-point work is the interpolation itself.
struct PvRow {
  unsigned off;   // offset of the half row at the block's level
  int sh;         // longitude shift (nlon/2 beyond the poles, else 0)
};
__device__ __forceinline__ PvRow pv_row(const DGrid &g, int jj, int k) {
  int sh = 0;
  if (jj < 1) { jj = 1 - jj; sh = g.half; }
  else if (jj > g.nhalf) { jj = 2 * g.nhalf + 1 - jj; sh = g.half; }
  return {(unsigned)ix3(g.nhalf, g.nlon, 1, jj, k), sh};
}

template <class R, bool MB>
__global__ void GMC_BOUNDS_MB(R, 6, MB) k_pv_edges(DGrid g, Slot<R> s, Work<R> w, R dt) {
  if constexpr (MB) { to_member(g, s); to_member(g, w); }   // member-batched launches
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  const R eps = (R)2.220446049250313e-16;
  const R wgt = SCALR(R, upwind_wgt_pv);
  const R *__restrict__ pv = s.pv;
  const bool tvd = g.pv_scheme == GMC_PV_TVD, mid_only = g.pv_scheme == GMC_PV_MIDPOINT, up3 = g.upwind_order_pv == 3;
  // pv at 0-based longitude l (l + shift in [-nlon, 2 nlon)) of a resolved row
  auto P = [&](const PvRow &r, int l) {
    l += r.sh;
    l = l < 0 ? l + nlon : (l >= nlon ? l - nlon : l);
    return pv[r.off + l];
  };
  if constexpr (std::is_same<R, float>::value) {
    // Default options (upwind, order 3) in FP32: two points per thread with
    // paired loads.  A pv row beyond a pole is read shifted by nlon/2, which
    // keeps a pair aligned (and wrapping together) when nlon/2 is even.
    if (!tvd && !mid_only && up3 && (g.half & 1) == 0) {
      auto P2 = [](const float *p, unsigned o) { return *reinterpret_cast<const float2 *>(p + o); };
      // pv of a resolved row at 0-based columns i0, i0+1
      auto Q2 = [&](const PvRow &r, int i0) {
        int l = i0 + r.sh;
        l = l >= nlon ? l - nlon : l;
        return P2(pv, r.off + l);
      };
      auto face = [&](float pm, float pc, float p3, float p0, float un, float vt) {   // one edge
        const float bb = fdiv(fabsf(vt), sqrtf(un * un + vt * vt) + eps);
        const float dir = fsign(1.0f, vt);
        const float up = upwind3(dir, wgt, p0, pm, pc, p3);
        return bb * up + (1.0f - bb) * 0.5f * (pm + pc);
      };
      if (j == 1 || j == nlat) {
        for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x)
          *reinterpret_cast<float2 *>(s.pv_lon + ix3(nlat, nlon, i0 + 1, j, k)) = make_float2(0.0f, 0.0f);
      } else {
        const PvRow r0 = pv_row(g, j - 2, k), r1 = pv_row(g, j - 1, k), r2 = pv_row(g, j, k), r3 = pv_row(g, j + 1, k);
        const unsigned fo = (unsigned)ix3(nlat, nlon, 1, j, k);
        const TangentRow tv = vlon_row(g, j, k);
        for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x) {
          const float2 a0 = Q2(r0, i0), a1 = Q2(r1, i0), a2 = Q2(r2, i0), a3 = Q2(r3, i0);
          const float2 un = P2(s.u_f, fo + i0);
          const float2 vt = g.tangent_inline ? vlon_pair(tv, s.mfy_lat, s.psr, nlon, i0) : P2(w.v_lon, fo + i0);
          *reinterpret_cast<float2 *>(s.pv_lon + fo + i0) =
              make_float2(face(a1.x, a2.x, a3.x, a0.x, un.x, vt.x), face(a1.y, a2.y, a3.y, a0.y, un.y, vt.y));
        }
      }
      if (j <= nhalf) {   // pv_lat: pv of half row j at columns i-2 .. i+1 (0-based i0-2 .. i0+2 for the pair)
        const unsigned ho = (unsigned)ix3(nhalf, nlon, 1, j, k);
        const TangentRow tu = ulat_row(g, j, k);
        for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x) {
          const float2 w2 = P2(pv, ho + (i0 == 0 ? nlon - 2 : i0 - 2)), c2 = P2(pv, ho + i0);
          const float e = pv[ho + (i0 + 2 == nlon ? 0 : i0 + 2)];
          const float2 ut = g.tangent_inline ? ulat_pair(tu, s.mfx_lon, s.psr, nlon, i0) : P2(w.u_lat, ho + i0);
          const float2 vn = P2(s.v_f, ho + i0);
          *reinterpret_cast<float2 *>(s.pv_lat + ho + i0) =
              make_float2(face(w2.y, c2.x, c2.y, w2.x, vn.x, ut.x), face(c2.x, c2.y, e, w2.y, vn.y, ut.y));
        }
      }
      return;
    }
  }
  // pv_lon on full row j: pv of half rows j-2 .. j+1 at the same longitude
  if (j == 1 || j == nlat) {
    for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) s.pv_lon[ix3(nlat, nlon, i0 + 1, j, k)] = (R)0;
  } else {
    const PvRow r0 = pv_row(g, j - 2, k), r1 = pv_row(g, j - 1, k), r2 = pv_row(g, j, k), r3 = pv_row(g, j + 1, k);
    const unsigned fo = (unsigned)ix3(nlat, nlon, 1, j, k);
    const R le = ROWR(R, le_lon, j);
    for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) {
      R val;
      if (tvd) {   // interp_pv_tvd (operators_mod.F90:797-832)
        const R cfl = w.v_lon[fo + i0] * (R)dt / le;
        val = tvd_interp<R>(g.tvd_limiter, cfl, P(r0, i0), P(r1, i0), P(r2, i0), P(r3, i0));
      } else if (mid_only) {
        val = (R)0.5 * (P(r2, i0) + P(r1, i0));
      } else {
        const R pm = P(r1, i0), pc = P(r2, i0);
        const R un = s.u_f[fo + i0], vt = w.v_lon[fo + i0];
        const R bb = fdiv(fabs(vt), sqrt(un * un + vt * vt) + eps);
        const R dir = fsign((R)1, vt);
        const R up = up3 ? upwind3(dir, wgt, P(r0, i0), pm, pc, P(r3, i0)) : upwind1(dir, wgt, pm, pc);
        val = bb * up + ((R)1 - bb) * (R)0.5 * (pm + pc);
      }
      s.pv_lon[fo + i0] = val;
    }
  }
  // pv_lat on half row j: pv of the same row at longitudes i-2 .. i+1
  if (j <= nhalf) {
    const PvRow r = pv_row(g, j, k);
    const unsigned ho = r.off;
    const R le = ROWR(R, le_lat, j);
    for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) {
      R val;
      const R pm = P(r, i0 - 1), pc = pv[ho + i0];
      if (tvd) {
        const R cfl = w.u_lat[ho + i0] * (R)dt / le;
        val = tvd_interp<R>(g.tvd_limiter, cfl, P(r, i0 - 2), pm, pc, P(r, i0 + 1));
      } else if (mid_only) {
        val = (R)0.5 * (pm + pc);
      } else {
        const R ut = w.u_lat[ho + i0], vn = s.v_f[ho + i0];
        const R bb = fdiv(fabs(ut), sqrt(ut * ut + vn * vn) + eps);
        const R dir = fsign((R)1, ut);
        const R up = up3 ? upwind3(dir, wgt, P(r, i0 - 2), pm, pc, P(r, i0 + 1)) : upwind1(dir, wgt, pm, pc);
        val = bb * up + ((R)1 - bb) * (R)0.5 * (pm + pc);
      }
      s.pv_lat[ho + i0] = val;
    }
  }
}

// adv_batch_accum_uv_cell, CFL part (adv_batch_mod.F90:252-373): RK4
// departure points along each axis give the Courant numbers; divx/divy are
// the axis-split divergences (pole rows: ring sums).
template <class R, bool MB>
__global__ void k_batch_cfl(DGrid g, const R *u, const R *v, R *cflx, R *cfly, R *divx, R *divy, R dt_) {
  if constexpr (MB) { const size_t mo = member_offset(g); u = mshift(u, mo); v = mshift(v, mo); cflx = mshift(cflx, mo); cfly = mshift(cfly, mo); divx = mshift(divx, mo); divy = mshift(divy, mo); }
  __shared__ double red[32];
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  const double radius = g.radius, dlon = g.dlon;
  auto half_lon = [&](int i) { double f = 0.0 + (i - 1) * dlon; return f + 0.5 * dlon; };
  if (j == 1 || j == nlat) {
    const int jv = j == 1 ? 1 : nhalf;
    const double sgn = j == 1 ? 1.0 : -1.0;
    double p = ring_sum(nlon, red, [&](int i) { return sgn * (double)v[ix3(nhalf, nlon, i, jv, k)]; });
    p = p * ROW(g.le_lat, jv) / nlon / ROW(g.area_cell, j);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      size_t o = ix3(nlat, nlon, i, j, k);
      divy[o] = (R)p;
      divx[o] = (R)0;
    }
  } else if constexpr (std::is_same<R, float>::value) {
    // FP32 form of the x departure: positions in cells relative to face i,
    // (radius half_lon(l) cos - x) / dx = (l - i) - a exactly in real arithmetic.
    // The row is staged in shared memory.
    extern __shared__ float us[];
    const float cdx = (float)dt_ / ROWR(float, de_lon, j);
    const float lel = ROWR(float, le_lon, j), ac = ROWR(float, area_cell, j);
    const float la0 = ROWR(float, le_lat, j), la1 = ROWR(float, le_lat, j - 1);
    const float hx = (float)g.hx;
    const float *urow = u + ix3(nlat, nlon, 1, j, k);
    for (int l = threadIdx.x; l < nlon; l += blockDim.x) us[l] = urow[l];
    __syncthreads();
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      auto Ul = [&](int l) {   // any l: a corrupted wind must not index out of the row
        int lw = l - 1;
        if (lw < 0 || lw >= nlon) {
          lw %= nlon;
          if (lw < 0) lw += nlon;
        }
        return us[lw];
      };
      // the winds at i-1, i, i+1 are loaded once: a departure within one
      // cell of the face (floor(a) = 0 or -1) interpolates between them, a
      // longer one indexes the row (the same values either way)
      const float uw = Ul(i - 1), u1 = Ul(i), ue = Ul(i + 1);
      auto at = [&](float a) {   // wind at i + a
        float fl = floorf(a);
        float f = a - fl;
        if (fl == 0.0f) return (1.0f - f) * u1 + f * ue;
        if (fl == -1.0f) return (1.0f - f) * uw + f * u1;
        int l = i + (int)fl;
        return (1.0f - f) * Ul(l) + f * Ul(l + 1);
      };
      const float u2 = at(0.5f * cdx * u1);
      const float u3 = at(0.5f * cdx * u2);
      const float u4 = at(cdx * u3);
      const float c = div6(u1 + 2.0f * u2 + 2.0f * u3 + u4) * cdx;
      if (fabsf(c) > hx) raise_err(g, ERR_CFLX);   // NaN passes, as abs(cflx) > width does
      size_t o = ix3(nlat, nlon, i, j, k);
      cflx[o] = c;
      divx[o] = fdiv((u1 - uw) * lel, ac);
      divy[o] = fdiv(v[ix3(nhalf, nlon, i, j, k)] * la0 - v[ix3(nhalf, nlon, i, j - 1, k)] * la1, ac);
    }
  } else {
    const double dx = ROW(g.de_lon, j), cl = ROW(g.full_cos_lat, j);
    const double lel = ROW(g.le_lon, j), ac = ROW(g.area_cell, j), la0 = ROW(g.le_lat, j), la1 = ROW(g.le_lat, j - 1);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      auto Ul = [&](int l) {   // any l: a corrupted wind must not index out of the row
        int lw = ((l - 1) % nlon + nlon) % nlon + 1;
        return (double)u[ix3(nlat, nlon, lw, j, k)];
      };
      double x0 = radius * half_lon(i) * cl;
      double u1 = Ul(i);
      double x1 = x0 + dt_ / 2 * u1;
      int l = (int)floor(i + (x1 - x0) / dx);
      double u2 = ((radius * half_lon(l + 1) * cl - x1) * Ul(l) + (x1 - radius * half_lon(l) * cl) * Ul(l + 1)) / dx;
      double x2 = x0 + dt_ / 2 * u2;
      l = (int)floor(i + (x2 - x0) / dx);
      double u3 = ((radius * half_lon(l + 1) * cl - x2) * Ul(l) + (x2 - radius * half_lon(l) * cl) * Ul(l + 1)) / dx;
      double x3 = x0 + dt_ * u3;
      l = (int)floor(i + (x3 - x0) / dx);
      double u4 = ((radius * half_lon(l + 1) * cl - x3) * Ul(l) + (x3 - radius * half_lon(l) * cl) * Ul(l + 1)) / dx;
      double c = (u1 + 2 * u2 + 2 * u3 + u4) / 6 * dt_ / dx;
      if (fabs(c) > (double)g.hx) raise_err(g, ERR_CFLX);
      size_t o = ix3(nlat, nlon, i, j, k);
      cflx[o] = (R)c;
      double uw = Ul(i - 1);
      divx[o] = (R)((u1 - uw) * lel / ac);
      double vn = (double)v[ix3(nhalf, nlon, i, j, k)], vs = (double)v[ix3(nhalf, nlon, i, j - 1, k)];
      divy[o] = (R)((vn * la0 - vs * la1) / ac);
    }
  }
  if constexpr (std::is_same<R, float>::value) {
    if (j <= nhalf) {
      // FP32 form of the y departure: row offsets A(l) = radius (half_lat(l) - half_lat(j)) / dy.
      // A departure more than one row away (|cfly| > 1, flagged below) keeps v1.
      const float cdy = (float)dt_ / ROWR(float, de_lat, j);
      const float *A = g.cfl_yoff + (size_t)(j - 1) * 4;   // l = j-1 .. j+2
      // the four offsets and, per column, the four rows a departure can use
      // (j-1 .. j+2) are loaded before the RK4 stages, which then select among
      // them: no load waits on a computed row
      const float A0 = A[0], A1 = A[1], A2 = A[2], A3 = A[3];
      auto Asel = [&](int t) { return t == 0 ? A0 : t == 1 ? A1 : t == 2 ? A2 : A3; };
      for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
        const unsigned ov = (unsigned)ix3(nhalf, nlon, i, j, k);
        const float v1 = v[ov];
        const float vm = j >= 2 ? v[ov - nlon] : 0.0f, vp = j + 1 <= nhalf ? v[ov + nlon] : 0.0f,
                    vp2 = j + 2 <= nhalf ? v[ov + 2 * nlon] : 0.0f;
        auto Vsel = [&](int t) { return t == 0 ? vm : t == 1 ? v1 : t == 2 ? vp : vp2; };   // row j-1+t
        auto at = [&](float b) {
          int l = (int)floorf((float)j + b);
          if (l < 1 || l > nhalf - 1 || l < j - 1 || l > j + 1) return v1;
          const int t = l - j + 1;   // 0 .. 2
          return (Asel(t + 1) - b) * Vsel(t) + (b - Asel(t)) * Vsel(t + 1);
        };
        const float v2 = at(0.5f * cdy * v1);
        const float v3 = at(0.5f * cdy * v2);
        const float v4 = at(cdy * v3);
        const float c = div6(v1 + 2.0f * v2 + 2.0f * v3 + v4) * cdy;
        if (fabsf(c) > 1.0f) raise_err(g, ERR_CFLY);
        cfly[ix3(nhalf, nlon, i, j, k)] = c;
      }
    }
    return;
  }
  if (j <= nhalf) {
    const double dy = ROW(g.de_lat, j);
    const double y0 = radius * ROW(g.half_lat, j);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      auto Vl = [&](int l) { return (double)v[ix3(nhalf, nlon, i, l, k)]; };
      auto interp = [&](int l, double y) {
        return ((radius * ROW(g.half_lat, l + 1) - y) * Vl(l) + (y - radius * ROW(g.half_lat, l)) * Vl(l + 1)) / dy;
      };
      double v1 = Vl(j);
      double y1 = y0 + dt_ / 2 * v1;
      int l = (int)floor(j + (y1 - y0) / dy);
      double v2 = (l < 1 || l > nhalf - 1) ? v1 : interp(l, y1);
      double y2 = y0 + dt_ / 2 * v2;
      l = (int)floor(j + (y2 - y0) / dy);
      double v3 = (l < 1 || l > nhalf - 1) ? v1 : interp(l, y2);
      double y3 = y0 + dt_ * v3;
      l = (int)floor(j + (y3 - y0) / dy);
      double v4 = (l < 1 || l > nhalf - 1) ? v1 : interp(l, y3);
      double c = (v1 + 2 * v2 + 2 * v3 + v4) / 6 * dt_ / dy;
      if (fabs(c) > 1.0) raise_err(g, ERR_CFLY);
      cfly[ix3(nhalf, nlon, i, j, k)] = (R)c;
    }
  }
}

// calc_grad_mf + calc_dphsdt + calc_we_lev + the mass batch's accum_we_lev
// for one column (operators_mod.F90:939-1006, 1120-1143, 192-226).
template <class R, bool MB>
__global__ void k_column_mass(DGrid g, Slot<R> s, Work<R> w, R dt) {
  if constexpr (MB) { to_member(g, s); to_member(g, w); }   // member-batched launches
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
      double p = ring_sum(nlon, red, [&](int ii) { return sgn * (double)s.mfy_lat[ix3(nhalf, nlon, ii, jv, k)]; });
      if (threadIdx.x == 0) ring[k - 1] = p * ROW(g.le_lat, jv) / nlon / ROW(g.area_cell, j);
    }
    __syncthreads();
  }
  if (i > nlon) return;
  const size_t c2 = (size_t)(j - 1) * nlon + (i - 1);
  const int im = wrap(i - 1, nlon);
  if constexpr (std::is_same<R, float>::value) {
    // FP32 form: divergences with per-row factors, layer masses from psr; the
    // column's prefix sums and then wm = we / ml * half_dlev live in shared
    // memory (one slot per level and thread).
    float *col = reinterpret_cast<float *>(ring + nlev + 2) + threadIdx.x;
    const int st = blockDim.x;
    const float ac = ROWR(float, area_cell, j);
    const float clon = ROWR(float, le_lon, j) / ac, cn = ROWR(float, le_lat, j) / ac, cs = ROWR(float, le_lat, j - 1) / ac;
    float mf = 0;
    for (int k = 1; k <= nlev; ++k) {
      float d;
      if (pole) {
        d = (float)ring[k - 1];
      } else {
        d = (s.mfx_lon[ix3(nlat, nlon, i, j, k)] - s.mfx_lon[ix3(nlat, nlon, im, j, k)]) * clon +
            (s.mfy_lat[ix3(nhalf, nlon, i, j, k)] * cn - s.mfy_lat[ix3(nhalf, nlon, i, j - 1, k)] * cs);
      }
      mf = mf + d;
      col[(k - 1) * st] = mf;   // prefix sum through level k
    }
    const float dphs = -mf;
    w.dphs[c2] = (double)dphs;
    const float psr = s.psr[c2];
    s.we_lev[ix3(nlat, nlon, i, j, 1)] = 0;
    float m_up = Mass<float>::layer(g, 1, psr);
    float p_prev = col[0];
    col[0] = 0;   // wm(1): we(1) = 0
    for (int k = 2; k <= nlev; ++k) {
      const float wv = -(g.hybi_f[k - 1] * dphs) - p_prev;
      s.we_lev[ix3(nlat, nlon, i, j, k)] = wv;
      const float m_lo = Mass<float>::layer(g, k, psr);
      const float ml = 0.5f * (m_up + m_lo);   // half-level mass
      p_prev = col[(k - 1) * st];
      col[(k - 1) * st] = fdiv(wv, ml) * g.half_dlev_f[k - 1];
      m_up = m_lo;
    }
    col[nlev * st] = 0;   // wm(nlev+1): we = 0
    s.we_lev[ix3(nlat, nlon, i, j, nlev + 1)] = 0;
    bool bad = false;
    const float dtf = (float)dt;
    for (int k = 2; k <= nlev; ++k) {
      float c = cflz_of_f(g.half_lev_f, g.full_dlev_f, g.full_dlev_rf, nlev, col, st, k, dtf, bad);
      if (c == c) w.cflz[ix3(nlat, nlon, i, j, k)] = c;
    }
    if (bad) raise_err(g, ERR_CFLZ);
  } else {
    double mfp[66], we[66], ml[66];
    const double lel = ROW(g.le_lon, j), ac = ROW(g.area_cell, j), la0 = ROW(g.le_lat, j), la1 = ROW(g.le_lat, j - 1);
    double dphs = 0, mf = 0;
    for (int k = 1; k <= nlev; ++k) {
      double dlon, dlat;
      if (pole) {
        dlon = 0;
        dlat = ring[k - 1];
      } else {
        dlon = ((double)s.mfx_lon[ix3(nlat, nlon, i, j, k)] - (double)s.mfx_lon[ix3(nlat, nlon, im, j, k)]) * lel / ac;
        dlat = ((double)s.mfy_lat[ix3(nhalf, nlon, i, j, k)] * la0 - (double)s.mfy_lat[ix3(nhalf, nlon, i, j - 1, k)] * la1) / ac;
      }
      dphs = dphs - dlon - dlat;
      mf = mf + dlon + dlat;
      mfp[k - 1] = mf;
    }
    w.dphs[c2] = dphs;
    s.we_lev[ix3(nlat, nlon, i, j, 1)] = 0;
    we[0] = 0;
    for (int k = 2; k <= nlev; ++k) {
      double wv = -(g.hybi[k - 1] * dphs) - mfp[k - 2];
      s.we_lev[ix3(nlat, nlon, i, j, k)] = wv;
      we[k - 1] = wv;
    }
    we[nlev] = 0;
    s.we_lev[ix3(nlat, nlon, i, j, nlev + 1)] = 0;
    // half-level mass from the hybrid pressures (calc_m, operators_mod.F90:505-525)
    const double phs = s.phs_f[c2];
    double plo = ph_lev(g, 1, phs), ph_prev = 0;
    for (int k = 1; k <= nlev; ++k) {
      double phi = ph_lev(g, k + 1, phs);
      double ph = 0.5 * (plo + phi);
      ml[k - 1] = k == 1 ? ph - plo : ph - ph_prev;
      ph_prev = ph;
      plo = phi;
    }
    ml[nlev] = plo - ph_prev;
    bool bad = false;
    for (int k = 2; k <= nlev; ++k) {
      double c = cflz_of<double>(g, we, ml, k, dt, bad);
      if (c == c) w.cflz[ix3(nlat, nlon, i, j, k)] = (R)c;
    }
    if (bad) raise_err(g, ERR_CFLZ);
  }
}

// FP32 form of k_column_mass over column tiles: layer divergences, their
// prefix sums along the column (warp scans), we_lev, dphs and the vertical
// Courant numbers, each phase parallel over (column, level).
template <bool MB>
__global__ void GMC_BOUNDS_FMB(8, 6, MB) k_column_mass_f(DGrid g, Slot<float> s, Work<float> w, float dt) {
  if constexpr (MB) { to_member(g, s); to_member(g, w); }   // member-batched launches
  extern __shared__ double shd[];
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon, nlev = g.nlev;
  const int j = blockIdx.y + 1;
  const int ti = threadIdx.x, kt = threadIdx.y, KT = blockDim.y;
  const int i = blockIdx.x * kTileI + ti + 1;
  const int ld = kTileI + 1;
  const bool pole = j == 1 || j == nlat, valid = i <= nlon;
  float *ring = reinterpret_cast<float *>(shd);          // [nlev] (FP64 sums rounded once)
  float *P = reinterpret_cast<float *>(shd + nlev);      // [nlev][ld]   prefix sums
  float *WM = P + nlev * ld;                             // [nlev+1][ld] we / ml * half_dlev
  float *HL = WM + (nlev + 1) * ld, *FD = HL + nlev + 1, *RFD = FD + nlev;   // level tables
  for (int t = kt * kTileI + ti; t <= nlev; t += kTileI * KT) {
    HL[t] = g.half_lev_f[t];
    if (t < nlev) {
      FD[t] = g.full_dlev_f[t];
      RFD[t] = g.full_dlev_rf[t];
    }
  }
  if (pole) tile_pole_ring(g, j, ring, [&](int ii, int jv, int k) { return s.mfy_lat[ix3(nhalf, nlon, ii, jv, k)]; });
  __syncthreads();
  const float ac = ROWR(float, area_cell, j);
  const float clon = ROWR(float, le_lon, j) / ac, cn = ROWR(float, le_lat, j) / ac, cs = ROWR(float, le_lat, j - 1) / ac;
  const int ic = valid ? i : nlon, im = wrap(ic - 1, nlon);
  for (int k = 1 + kt; k <= nlev; k += KT) {
    float d;
    if (pole)
      d = ring[k - 1];
    else
      d = (s.mfx_lon[ix3(nlat, nlon, ic, j, k)] - s.mfx_lon[ix3(nlat, nlon, im, j, k)]) * clon +
          (s.mfy_lat[ix3(nhalf, nlon, ic, j, k)] * cn - s.mfy_lat[ix3(nhalf, nlon, ic, j - 1, k)] * cs);
    P[(k - 1) * ld + ti] = d;
  }
  __syncthreads();
  {   // inclusive prefix sums along k, one warp per column at a time
    const int lt = kt * kTileI + ti, lane = lt & 31, warp = lt >> 5, nw = (kTileI * KT) >> 5;
    for (int c = warp; c < kTileI; c += nw) {
      float carry = 0;
      for (int base = 0; base < nlev; base += 32) {
        const int k0 = base + lane;
        float v = k0 < nlev ? P[k0 * ld + c] : 0.f;
        for (int o = 1; o < 32; o <<= 1) {
          float t = __shfl_up_sync(0xffffffffu, v, o);
          if (lane >= o) v += t;
        }
        v += carry;
        if (k0 < nlev) P[k0 * ld + c] = v;
        carry = __shfl_sync(0xffffffffu, v, 31);
      }
    }
  }
  __syncthreads();
  const size_t c2 = (size_t)(j - 1) * nlon + (ic - 1);
  const float dphs = -P[(nlev - 1) * ld + ti];
  if (kt == 0 && valid) w.dphs[c2] = (double)dphs;
  const float psr = s.psr[c2];
  for (int k = 1 + kt; k <= nlev + 1; k += KT) {
    float wv = 0, wm = 0;
    if (k != 1 && k != nlev + 1) {
      wv = -(g.hybi_f[k - 1] * dphs) - P[(k - 2) * ld + ti];
      const float ml = 0.5f * (Mass<float>::layer(g, k - 1, psr) + Mass<float>::layer(g, k, psr));
      wm = fdiv(wv, ml) * g.half_dlev_f[k - 1];
    }
    if (valid) s.we_lev[ix3(nlat, nlon, i, j, k)] = wv;
    WM[(k - 1) * ld + ti] = wm;
  }
  __syncthreads();
  if (!valid) return;
  bool bad = false;
  const float dtf = (float)dt;
  for (int k = 2 + kt; k <= nlev; k += KT) {
    float c = cflz_of_f(HL, FD, RFD, nlev, WM + ti, ld, k, dtf, bad);
    if (c == c) w.cflz[ix3(nlat, nlon, i, j, k)] = c;
  }
  if (bad) raise_err(g, ERR_CFLZ);
}

// Momentum tendencies of the forward pass (gmcore_mod.F90:478-490 / 507-518):
// du = qhv - dke/dlon - we du/dlev, dv = -qhu - dke/dlat - we dv/dlev with the
// energy-conserving Coriolis term (calc_coriolis, operators_mod.F90:846-906),
// the KE gradient (:908-937) and SB81 vertical advection (:1145-1216).
template <class R, bool MB>
__global__ void k_momentum_tend(DGrid g, Slot<R> s, Work<R> w) {
  if constexpr (MB) { to_member(g, s); to_member(g, w); }   // member-batched launches
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon, nlev = g.nlev;
  const MassField<R> M = mass_of(g, s);
  auto MFX = [&](int i, int jj) { return s.mfx_lon[ix3(nlat, nlon, wrap(i, nlon), jj, k)]; };
  auto MFY = [&](int i, int jj) { return s.mfy_lat[ix3(nhalf, nlon, wrap(i, nlon), jj, k)]; };
  auto PVLON = [&](int i, int jj) { return s.pv_lon[ix3(nlat, nlon, wrap(i, nlon), jj, k)]; };
  auto PVLAT = [&](int i, int jj) { return s.pv_lat[ix3(nhalf, nlon, wrap(i, nlon), jj, k)]; };
  if (j != 1 && j != nlat) {
    const R t1 = ROWR(R, ftw1, j), t2 = ROWR(R, ftw2, j), de = ROWR(R, de_lon, j);
    const R aw = ROWR(R, area_lon_west, j), ae = ROWR(R, area_lon_east, j), al = ROWR(R, area_lon, j);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      const size_t o = ix3(nlat, nlon, i, j, k);
      const R pl = s.pv_lon[o];
      R qhv;
      if (g.coriolis_scheme == 1) {
        qhv = (t1 * (MFY(i, j - 1) * (pl + PVLAT(i, j - 1)) + MFY(i + 1, j - 1) * (pl + PVLAT(i + 1, j - 1))) +
               t2 * (MFY(i, j) * (pl + PVLAT(i, j)) + MFY(i + 1, j) * (pl + PVLAT(i + 1, j)))) * (R)0.5;
      } else {
        R mfy_lon = t1 * (MFY(i, j - 1) + MFY(i + 1, j - 1)) + t2 * (MFY(i, j) + MFY(i + 1, j));
        qhv = mfy_lon * pl;
      }
      R dkedlon = (w.ke[ix3(nlat, nlon, wrap(i + 1, nlon), j, k)] - w.ke[o]) / de;
      R du = qhv - dkedlon;
      if (g.baroclinic) {
        auto WEL = [&](int kk) {
          R a = s.we_lev[ix3(nlat, nlon, i, j, kk)], b = s.we_lev[ix3(nlat, nlon, wrap(i + 1, nlon), j, kk)];
          return (aw * a + ae * b) / al;
        };
        auto Uk = [&](int kk) { return s.u_f[ix3(nlat, nlon, i, j, kk)]; };
        R m_lon = (M.at(g, i, j, k) + M.at(g, i + 1, j, k)) * (R)0.5;
        R wd;
        if (k == 1)
          wd = (WEL(k + 1) * (Uk(k + 1) - Uk(k))) / m_lon / (R)2;
        else if (k == nlev)
          wd = (WEL(k) * (Uk(k) - Uk(k - 1))) / m_lon / (R)2;
        else
          wd = (WEL(k + 1) * (Uk(k + 1) - Uk(k)) + WEL(k) * (Uk(k) - Uk(k - 1))) / m_lon / (R)2;
        du = du - wd;
      }
      w.du[o] = du;
    }
  }
  if (j <= nhalf) {
    const R t1 = ROWR(R, htw1, j), t2 = ROWR(R, htw2, j), de = ROWR(R, de_lat, j);
    const R an = ROWR(R, area_lat_north, j), as = ROWR(R, area_lat_south, j), al = ROWR(R, area_lat, j);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      const size_t o = ix3(nhalf, nlon, i, j, k);
      const R pl = s.pv_lat[o];
      R qhu;
      if (g.coriolis_scheme == 1) {
        qhu = (t1 * (MFX(i - 1, j) * (pl + PVLON(i - 1, j)) + MFX(i, j) * (pl + PVLON(i, j))) +
               t2 * (MFX(i - 1, j + 1) * (pl + PVLON(i - 1, j + 1)) + MFX(i, j + 1) * (pl + PVLON(i, j + 1)))) * (R)0.5;
      } else {
        R mfx_lat = t1 * (MFX(i - 1, j) + MFX(i, j)) + t2 * (MFX(i - 1, j + 1) + MFX(i, j + 1));
        qhu = mfx_lat * pl;
      }
      R dkedlat = (w.ke[ix3(nlat, nlon, i, j + 1, k)] - w.ke[ix3(nlat, nlon, i, j, k)]) / de;
      R dv = -qhu - dkedlat;
      if (g.baroclinic) {
        auto WEL = [&](int kk) {
          R a = s.we_lev[ix3(nlat, nlon, i, j + 1, kk)], b = s.we_lev[ix3(nlat, nlon, i, j, kk)];
          return (an * a + as * b) / al;
        };
        auto Vk = [&](int kk) { return s.v_f[ix3(nhalf, nlon, i, j, kk)]; };
        R m_lat = (M.at(g, i, j, k) + M.at(g, i, j + 1, k)) * (R)0.5;
        R wd;
        if (k == 1)
          wd = (WEL(k + 1) * (Vk(k + 1) - Vk(k))) / m_lat / (R)2;
        else if (k == nlev)
          wd = (WEL(k) * (Vk(k) - Vk(k - 1))) / m_lat / (R)2;
        else
          wd = (WEL(k + 1) * (Vk(k + 1) - Vk(k)) + WEL(k) * (Vk(k) - Vk(k - 1))) / m_lat / (R)2;
        dv = dv - wd;
      }
      w.dv[o] = dv;
    }
  }
}

// FP32 form of k_momentum_tend (baroclinic): the same terms with the arrays
// passed as non-aliasing kernel arguments addressed by 32-bit row offsets (the
// base pointers stay in the parameter bank, so the kernel fits in 32
// registers) and the divisions taken as reciprocal products (fdiv).
template <bool MB>
__global__ void GMC_BOUNDS_FMB(5, 5, MB) k_momentum_f(DGrid g, const float *__restrict__ mfx, const float *__restrict__ mfy,
                                             const float *__restrict__ pvlon, const float *__restrict__ pvlat,
                                             const float *__restrict__ ke, const float *__restrict__ we,
                                             const float *__restrict__ uf, const float *__restrict__ vf,
                                             const float *__restrict__ psr, float *__restrict__ du,
                                             float *__restrict__ dv) {
  if constexpr (MB) { const size_t mo = member_offset(g); mfx = mshift(mfx, mo); mfy = mshift(mfy, mo); pvlon = mshift(pvlon, mo); pvlat = mshift(pvlat, mo); ke = mshift(ke, mo); we = mshift(we, mo); uf = mshift(uf, mo); vf = mshift(vf, mo); psr = mshift(psr, mo); du = mshift(du, mo); dv = mshift(dv, mo); }
  const int k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon, nlev = g.nlev;
  const bool cor1 = g.coriolis_scheme == 1;
  const float dA = g.dmA[k - 1], dB = g.dmB[k - 1];
  const unsigned lf = (unsigned)nlat * nlon, lh = (unsigned)nhalf * nlon;   // level strides
  // Each thread takes two neighbouring points i0, i0 + 1 (nlon is even and
  // row offsets are multiples of nlon, so the pair is one aligned 8-byte
  // load) and the stencil's third column as one more value: three values of a
  // row for two points where the single-point form loads four.
  struct T3 { float a, b, c; };
  auto east = [nlon](const float *__restrict__ p, unsigned o, int i0) {   // values at i0, i0+1, i0+2
    const float2 t = *reinterpret_cast<const float2 *>(p + o + i0);
    return T3{t.x, t.y, p[o + (i0 + 2 == nlon ? 0 : i0 + 2)]};
  };
  auto west = [nlon](const float *__restrict__ p, unsigned o, int i0) {   // values at i0-1, i0, i0+1
    const float2 t = *reinterpret_cast<const float2 *>(p + o + i0);
    return T3{p[o + (i0 == 0 ? nlon - 1 : i0 - 1)], t.x, t.y};
  };
  auto pair = [](const float *__restrict__ p, unsigned o) { return *reinterpret_cast<const float2 *>(p + o); };
  // blocks 0 .. nlat-3: du on full rows 2 .. nlat-1; then dv on half rows 1 .. nhalf
  const bool urow = (int)blockIdx.x < nlat - 2;
  const int j = urow ? blockIdx.x + 2 : blockIdx.x - (nlat - 2) + 1;
  if (urow) {
    const float t1 = ROWR(float, ftw1, j), t2 = ROWR(float, ftw2, j), de = ROWR(float, de_lon, j);
    const float aw = ROWR(float, area_lon_west, j), ae = ROWR(float, area_lon_east, j), al = ROWR(float, area_lon, j);
    const unsigned hs = (unsigned)ix3(nhalf, nlon, 1, j - 1, k), hn = hs + nlon;   // half rows j-1, j
    const unsigned fo = (unsigned)ix3(nlat, nlon, 1, j, k), po = (unsigned)(j - 1) * nlon;
    for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x) {
      const float2 pl2 = pair(pvlon, fo + i0), u2 = pair(uf, fo + i0);
      const T3 ms = east(mfy, hs, i0), ps = east(pvlat, hs, i0), mn = east(mfy, hn, i0), pn = east(pvlat, hn, i0);
      const T3 ke3 = east(ke, fo, i0), pr = east(psr, po, i0);
      T3 wu{0, 0, 0}, wl{0, 0, 0};
      float2 uu = make_float2(0, 0), ul = make_float2(0, 0);
      if (k < nlev) { wl = east(we, fo + lf, i0); ul = pair(uf, fo + lf + i0); }
      if (k > 1) { wu = east(we, fo, i0); uu = pair(uf, fo - lf + i0); }
      float out[2];
#pragma unroll
      for (int p = 0; p < 2; ++p) {   // point i0 + p: its own column and the next (ip)
        const float pl = p ? pl2.y : pl2.x;
        const float ms0 = p ? ms.b : ms.a, ms1 = p ? ms.c : ms.b, ps0 = p ? ps.b : ps.a, ps1 = p ? ps.c : ps.b;
        const float mn0 = p ? mn.b : mn.a, mn1 = p ? mn.c : mn.b, pn0 = p ? pn.b : pn.a, pn1 = p ? pn.c : pn.b;
        float qhv;
        if (cor1)
          qhv = (t1 * (ms0 * (pl + ps0) + ms1 * (pl + ps1)) + t2 * (mn0 * (pl + pn0) + mn1 * (pl + pn1))) * 0.5f;
        else
          qhv = (t1 * (ms0 + ms1) + t2 * (mn0 + mn1)) * pl;
        const float d = qhv - fdiv((p ? ke3.c : ke3.b) - (p ? ke3.b : ke3.a), de);
        const float m_lon = (fmaf(dB, p ? pr.b : pr.a, dA) + fmaf(dB, p ? pr.c : pr.b, dA)) * 0.5f;
        const float u0 = p ? u2.y : u2.x;
        float wd = 0;
        if (k < nlev) wd = fdiv(aw * (p ? wl.b : wl.a) + ae * (p ? wl.c : wl.b), al) * ((p ? ul.y : ul.x) - u0);
        if (k > 1) wd += fdiv(aw * (p ? wu.b : wu.a) + ae * (p ? wu.c : wu.b), al) * (u0 - (p ? uu.y : uu.x));
        out[p] = d - fdiv(wd, m_lon) * 0.5f;
      }
      *reinterpret_cast<float2 *>(du + fo + i0) = make_float2(out[0], out[1]);
    }
    return;
  }
  {
    const float t1 = ROWR(float, htw1, j), t2 = ROWR(float, htw2, j), de = ROWR(float, de_lat, j);
    const float an = ROWR(float, area_lat_north, j), as = ROWR(float, area_lat_south, j), al = ROWR(float, area_lat, j);
    const unsigned fs = (unsigned)ix3(nlat, nlon, 1, j, k), fn = fs + nlon;   // full rows j, j+1
    const unsigned ho = (unsigned)ix3(nhalf, nlon, 1, j, k), ps = (unsigned)(j - 1) * nlon, pn = ps + nlon;
    for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x) {
      const float2 pl2 = pair(pvlat, ho + i0), v2 = pair(vf, ho + i0);
      const T3 xs = west(mfx, fs, i0), qs = west(pvlon, fs, i0), xn = west(mfx, fn, i0), qn = west(pvlon, fn, i0);
      const float2 kn = pair(ke, fn + i0), ks = pair(ke, fs + i0), rs = pair(psr, ps + i0), rn = pair(psr, pn + i0);
      float2 wnl = make_float2(0, 0), wsl = make_float2(0, 0), wnu = make_float2(0, 0), wsu = make_float2(0, 0);
      float2 vl = make_float2(0, 0), vu = make_float2(0, 0);
      if (k < nlev) { wnl = pair(we, fn + lf + i0); wsl = pair(we, fs + lf + i0); vl = pair(vf, ho + lh + i0); }
      if (k > 1) { wnu = pair(we, fn + i0); wsu = pair(we, fs + i0); vu = pair(vf, ho - lh + i0); }
      float out[2];
#pragma unroll
      for (int p = 0; p < 2; ++p) {   // point i0 + p: the previous column (im) and its own
        const float pl = p ? pl2.y : pl2.x;
        const float xs0 = p ? xs.b : xs.a, xs1 = p ? xs.c : xs.b, qs0 = p ? qs.b : qs.a, qs1 = p ? qs.c : qs.b;
        const float xn0 = p ? xn.b : xn.a, xn1 = p ? xn.c : xn.b, qn0 = p ? qn.b : qn.a, qn1 = p ? qn.c : qn.b;
        float qhu;
        if (cor1)
          qhu = (t1 * (xs0 * (pl + qs0) + xs1 * (pl + qs1)) + t2 * (xn0 * (pl + qn0) + xn1 * (pl + qn1))) * 0.5f;
        else
          qhu = (t1 * (xs0 + xs1) + t2 * (xn0 + xn1)) * pl;
        const float d = -qhu - fdiv((p ? kn.y : kn.x) - (p ? ks.y : ks.x), de);
        const float m_lat = (fmaf(dB, p ? rs.y : rs.x, dA) + fmaf(dB, p ? rn.y : rn.x, dA)) * 0.5f;
        const float v0 = p ? v2.y : v2.x;
        float wd = 0;
        if (k < nlev) wd = fdiv(an * (p ? wnl.y : wnl.x) + as * (p ? wsl.y : wsl.x), al) * ((p ? vl.y : vl.x) - v0);
        if (k > 1) wd += fdiv(an * (p ? wnu.y : wnu.x) + as * (p ? wsu.y : wsu.x), al) * (v0 - (p ? vu.y : vu.x));
        out[p] = d - fdiv(wd, m_lat) * 0.5f;
      }
      *reinterpret_cast<float2 *>(dv + ho + i0) = make_float2(out[0], out[1]);
    }
  }
}

// Shallow-water thickness tendency dgz = -(dmf/dlon + dmf/dlat) g
// (gmcore_mod.F90:520-524) with the pole ring of calc_grad_mf.
template <class R, bool MB>
__global__ void k_swm_dgz(DGrid g, Slot<R> s, Work<R> w) {
  if constexpr (MB) { to_member(g, s); to_member(g, w); }   // member-batched launches
  __shared__ double red[32];
  const int j = blockIdx.x + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  if (j == 1 || j == nlat) {
    const int jv = j == 1 ? 1 : nhalf;
    const double sgn = j == 1 ? 1.0 : -1.0;
    double p = ring_sum(nlon, red, [&](int i) { return sgn * (double)s.mfy_lat[ix3(nhalf, nlon, i, jv, 1)]; });
    p = p * ROW(g.le_lat, jv) / nlon / ROW(g.area_cell, j);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) w.dgz[ix3(nlat, nlon, i, j, 1)] = (R)(-(0.0 + p) * g.g);
    return;
  }
  const R lel = ROWR(R, le_lon, j), ac = ROWR(R, area_cell, j), la0 = ROWR(R, le_lat, j), la1 = ROWR(R, le_lat, j - 1);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    R dlon = (s.mfx_lon[ix3(nlat, nlon, i, j, 1)] - s.mfx_lon[ix3(nlat, nlon, wrap(i - 1, nlon), j, 1)]) * lel / ac;
    R dlat = (s.mfy_lat[ix3(nhalf, nlon, i, j, 1)] * la0 - s.mfy_lat[ix3(nhalf, nlon, i, j - 1, 1)] * la1) / ac;
    w.dgz[ix3(nlat, nlon, i, j, 1)] = -(dlon + dlat) * SCALR(R, g);
  }
}

// ---------------------------------------------------------------------------
// update_state (time_schemes_mod.F90:120-242): row updates fused with the
// polar filters.
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T *smem_rows(double *base, int nlon, int which) {
  return reinterpret_cast<T *>(base) + (size_t)which * nlon;
}

// Error checks of one column's new surface pressure phs (unfiltered) and its
// filtered value phs_f: ERR_NAN when either is not finite, ERR_NONMONO when
// a layer mass from phs_f is not positive (calc_m, operators_mod.F90:489-500).
// The FP32 form checks its own layer masses dA_k + dB_k psr (psr = phs_f - ptop
// in FP32); the FP64 form the hybrid-formula difference ph_lev(k+1) - ph_lev(k).
__device__ __forceinline__ void check_column(const DGrid &g, double phs, double phs_f, float psr) {
  if (!isfinite(phs) || !isfinite(phs_f)) {
    raise_err(g, ERR_NAN);
    return;
  }
  bool bad = false;
  if (g.f_layer_mass) {
    for (int k = 1; k <= g.nlev; ++k) bad |= !(fmaf(g.dmB[k - 1], psr, g.dmA[k - 1]) > 0.0f);
  } else {
    for (int k = 1; k <= g.nlev; ++k) bad |= !(Mass<double>::layer(g, k, phs_f) > 0.0);
  }
  if (bad) raise_err(g, ERR_NONMONO);
}

// phs = phs_old + dt dphs; phs_f = big filter(phs)   (:134-143)
template <class R, bool MB>
__global__ void k_update_phs(DGrid g, Slot<R> o, Slot<R> n, Work<R> w, double dt) {
  if constexpr (MB) { to_member(g, o); to_member(g, n); to_member(g, w); }   // member-batched launches
  extern __shared__ double sh[];
  const int j = blockIdx.x + 1, nlon = g.nlon;
  double *row = sh, *ext = sh + nlon;
  if constexpr (std::is_same<R, float>::value) {
    // FP32 form: the filter runs on FP32 deviations from the row's first
    // value; phs itself stays FP64.
    float *dev = reinterpret_cast<float *>(sh + nlon), *fext = dev + nlon;
    const size_t c0 = (size_t)(j - 1) * nlon;
    const double ref = o.phs[c0] + dt * w.dphs[c0];
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
      const size_t c = c0 + i;
      const double v = o.phs[c] + dt * w.dphs[c];
      n.phs[c] = v;
      row[i] = v;
      dev[i] = (float)(v - ref);
    }
    const bool filtered = filter_row<float, float>(g.big, true, j, nlon, dev, fext);
    __syncthreads();
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
      const double f = filtered ? ref + (double)dev[i] : row[i];
      const float psr = (float)(f - g.ptop);
      n.phs_f[c0 + i] = f;
      n.psr[c0 + i] = psr;
      check_column(g, row[i], f, psr);
    }
    return;
  }
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    size_t c = (size_t)(j - 1) * nlon + i;
    double v = o.phs[c] + dt * w.dphs[c];
    n.phs[c] = v;
    row[i] = v;
  }
  filter_row<double>(g.big, true, j, nlon, row, ext);
  __syncthreads();
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    n.phs_f[(size_t)(j - 1) * nlon + i] = row[i];
    if (n.psr) n.psr[(size_t)(j - 1) * nlon + i] = (float)(row[i] - g.ptop);
    check_column(g, n.phs[(size_t)(j - 1) * nlon + i], row[i], 0.0f);
  }
}

// Column checks of a new surface pressure: a non-finite value, and the
// layer masses of calc_m (operators_mod.F90:489-500, m = ph_lev(k+1) -
// ph_lev(k) <= 0 stops the reference with 'The pressure levels are not
// monotonic!') from the filtered surface pressure phs_f, as each form forms
// them (FP64 hybrid formula; FP32 dA_k + dB_k psr).
__global__ void k_check_columns(DGrid g, const double *__restrict__ phs_f, const float *__restrict__ psr, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    check_column(g, phs_f[t], phs_f[t], psr ? psr[t] : 0.0f);
}

// FP32 form: psr = phs_f - ptop
__global__ void k_surface_rel(const double *phs_f, float *psr, size_t n, double ptop) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    psr[t] = (float)(phs_f[t] - ptop);
}

// pt = small1 filter(pt_old m_old + dt dpt) / m_new   (:153-173); a block
// takes one row at kPtLevels(R) consecutive levels (shared filter weights).
template <class R>
constexpr int kPtLevels = std::is_same<R, float>::value ? 2 : 1;

template <class R, bool MB>
__global__ void k_update_pt(DGrid g, Slot<R> o, Slot<R> n, Work<R> w, R dt) {
  if constexpr (MB) { to_member(g, o); to_member(g, n); to_member(g, w); }   // member-batched launches
  constexpr int KB = kPtLevels<R>;
  extern __shared__ double sh[];
  const int j = blockIdx.x + 1, k0 = blockIdx.y * KB + 1, nlon = g.nlon, nlat = g.nlat, nlev = g.nlev;
  const int nk = min(KB, nlev - k0 + 1);
  const int es = nlon + 2 * ((g.big.max_taps - 1) / 2) + 8;
  R *row = reinterpret_cast<R *>(sh), *ext = row + KB * nlon;
  const R dtr = (R)dt;
  const SurfP<R> so = o.surf(), sn = n.surf();
  const unsigned m0 = (unsigned)(j - 1) * nlon;
  constexpr bool kPair = std::is_same<R, float>::value;   // FP32: two points per thread, paired loads
  for (int kk = 0; kk < nk; ++kk) {
    const int k = k0 + kk;
    const unsigned c0 = (unsigned)ix3(nlat, nlon, 1, j, k);
    if constexpr (kPair) {
      for (int i = 2 * threadIdx.x; i < nlon; i += 2 * blockDim.x) {
        const float2 p = *reinterpret_cast<const float2 *>(so.psr + m0 + i);
        const float2 t = *reinterpret_cast<const float2 *>(o.pt + c0 + i);
        const float2 d = *reinterpret_cast<const float2 *>(w.dpt + c0 + i);
        *reinterpret_cast<float2 *>(row + kk * nlon + i) = make_float2(
            t.x * Mass<float>::layer(g, k, p.x) + dtr * d.x, t.y * Mass<float>::layer(g, k, p.y) + dtr * d.y);
      }
    } else {
      for (int i = threadIdx.x; i < nlon; i += blockDim.x)
        row[kk * nlon + i] = o.pt[c0 + i] * Mass<R>::layer(g, k, so.at(m0 + i)) + dtr * w.dpt[c0 + i];
    }
  }
  if (nk == KB) {
    filter_rows<KB, R, R>(g.small1, true, j, nlon, row, nlon, ext, es);
  } else {
    for (int kk = 0; kk < nk; ++kk) filter_row<R, R>(g.small1, true, j, nlon, row + kk * nlon, ext);
  }
  __syncthreads();
  for (int kk = 0; kk < nk; ++kk) {
    const int k = k0 + kk;
    const unsigned c0 = (unsigned)ix3(nlat, nlon, 1, j, k);
    if constexpr (kPair) {
      for (int i = 2 * threadIdx.x; i < nlon; i += 2 * blockDim.x) {
        const float2 p = *reinterpret_cast<const float2 *>(sn.psr + m0 + i);
        const float2 r = *reinterpret_cast<const float2 *>(row + kk * nlon + i);
        const float2 v = make_float2(r.x / Mass<float>::layer(g, k, p.x), r.y / Mass<float>::layer(g, k, p.y));
        *reinterpret_cast<float2 *>(n.pt + c0 + i) = v;
        if (!isfinite(v.x) || !isfinite(v.y)) raise_err(g, ERR_NAN);
      }
    } else {
      for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
        const R v = row[kk * nlon + i] / Mass<R>::layer(g, k, sn.at(m0 + i));
        n.pt[c0 + i] = v;
        if (!isfinite(v)) raise_err(g, ERR_NAN);
      }
    }
  }
}

// Shallow water: gz = gz_old + dt dgz; gz_f = big(gz); gz = small1(gz) (:178-192)
template <class R, bool MB>
__global__ void k_update_gz(DGrid g, Slot<R> o, Slot<R> n, Work<R> w, R dt) {
  if constexpr (MB) { to_member(g, o); to_member(g, n); to_member(g, w); }   // member-batched launches
  extern __shared__ double sh[];
  const int j = blockIdx.x + 1, nlon = g.nlon;
  R *row = reinterpret_cast<R *>(sh), *row2 = row + nlon, *ext = row2 + nlon;
  const R dtr = (R)dt;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    size_t c = (size_t)(j - 1) * nlon + i;
    R v = o.gz[c] + dtr * w.dgz[c];
    row[i] = v;
    row2[i] = v;
  }
  filter_row<R>(g.big, true, j, nlon, row2, ext);
  __syncthreads();
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) n.gz_f[(size_t)(j - 1) * nlon + i] = row2[i];
  filter_row<R>(g.small1, true, j, nlon, row, ext);
  __syncthreads();
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    n.gz[(size_t)(j - 1) * nlon + i] = row[i];
    if (!isfinite(row[i])) raise_err(g, ERR_NAN);
  }
}

// Backward-pass column sweep (operators_prepare_2 backward,
// operators_mod.F90:124-131): hybrid pressures and their Exner power
// (calc_ph :136-168), temperature (calc_t :170-190) and the hydrostatic
// geopotential integrated upward from the surface (calc_gz_lev :433-469).
template <class R, bool MB>
__global__ void k_column_backward(DGrid g, Slot<R> n, Work<R> w) {
  if constexpr (MB) { to_member(g, n); to_member(g, w); }   // member-batched launches
  const int j = blockIdx.y + 1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int nlat = g.nlat, nlon = g.nlon, nlev = g.nlev;
  if (i > nlon) return;
  const size_t c2 = (size_t)(j - 1) * nlon + (i - 1);
  const double phs = n.phs_f[c2];
  const double gzs = n.gzs[c2];
  if constexpr (std::is_same<R, float>::value) {
    // FP32 form about the reference column: p(k) = p_ref(k) (1 + r(k)) with
    // r(k) = pr_c(k) (phs - ps_ref), so
    //   p^kappa       = pe_ref(k) + pe_ref(k) expm1(kappa log1p(r))   (pea holds the second term)
    //   ln(p(k+1)/p(k)) = dlnp_ref(k) + log1p(r(k+1)) - log1p(r(k))
    //   (ph/p0)^kappa = tf_ref(k) exp(kappa log1p(rf)),  rf = cf(k) (phs - ps_ref).
    // Every FP32 quantity is either small or relative, and the geopotential
    // is summed upward as an unevaluated (hi, lo) FP32 pair, so differences
    // between neighbours keep ~1e-7 relative accuracy without FP64 issue.
    const float kap = g.kappa_f, Rd = g.Rd_f;
    const float dps = (float)(phs - g.ps_ref);
    float hi = (float)gzs;
    float lo = (float)(gzs - (double)hi);
    w.gzhl[ix3(nlat, nlon, i, j, nlev + 1)] = make_float2(hi, lo);
    float L_hi = log1pf(g.pr_c[nlev] * dps);
    w.pea[ix3(nlat, nlon, i, j, nlev + 1)] = g.pe_ref[nlev] * expm1f(kap * L_hi);
    for (int k = nlev; k >= 1; --k) {
      const float L_lo = log1pf(g.pr_c[k - 1] * dps);
      w.pea[ix3(nlat, nlon, i, j, k)] = g.pe_ref[k - 1] * expm1f(kap * L_lo);
      const float t = n.pt[ix3(nlat, nlon, i, j, k)] * (g.tf_ref[k - 1] * expf(kap * log1pf(g.cf[k - 1] * dps)));
      const float x = Rd * t * (g.dlnp_ref[k - 1] + (L_hi - L_lo));
      // (hi, lo) += x: two-sum, then renormalise
      const float s1 = hi + x, bp = s1 - hi;
      const float e = (hi - (s1 - bp)) + (x - bp);
      lo = lo + e;
      hi = s1 + lo;
      lo = lo - (hi - s1);
      w.gzhl[ix3(nlat, nlon, i, j, k)] = make_float2(hi, lo);
      L_hi = L_lo;
    }
    return;
  }
  w.gz_lev[ix3(nlat, nlon, i, j, nlev + 1)] = gzs;
  double pl[66];
  for (int k = 1; k <= nlev + 1; ++k) {
    pl[k - 1] = ph_lev(g, k, phs);
    w.ph_exn_lev[ix3(nlat, nlon, i, j, k)] = pow(pl[k - 1], g.kappa);
  }
  double acc = 0;
  for (int k = nlev; k >= 1; --k) {
    double ph = 0.5 * (pl[k - 1] + pl[k]);
    double t = (double)n.pt[ix3(nlat, nlon, i, j, k)] * pow(ph / g.p0, g.kappa);
    acc = g.Rd * t * log(pl[k] / pl[k - 1]) + acc;
    w.gz_lev[ix3(nlat, nlon, i, j, k)] = gzs + acc;
  }
}

// u, v = old + dt (du_fwd - pgf); small2 filter (baroclinic); v blended next
// to the poles; big filter into u_f, v_f   (time_schemes_mod.F90:198-238,
// pgf_lin97_run pgf_lin97_mod.F90:59-105, pgf_swm_run pgf_swm_mod.F90:18-46,
// backward pass gmcore_mod.F90:529-571).
// Difference of two (hi, lo) FP32 pairs: the hi parts of neighbouring
// geopotentials are within a factor two of each other, so their difference is
// exact and the result carries the pair's full accuracy.
__device__ __forceinline__ float hl_diff(float2 a, float2 b) { return (a.x - b.x) + (a.y - b.y); }

template <class R>
__device__ __forceinline__ R pgf_lon(const DGrid &g, const Slot<R> &n, const Work<R> &w, int i, int j, int k, R inv_d) {
  const int nlat = g.nlat, nlon = g.nlon;
  const int ip = wrap(i + 1, nlon);
  if (g.baroclinic) {
    if constexpr (std::is_same<R, float>::value) {
      const float *pa = w.pea;
      const float2 *gz = w.gzhl;
      const float dref = g.dpe_ref[k - 1];
      float dph1 = dref + (pa[ix3(nlat, nlon, ip, j, k + 1)] - pa[ix3(nlat, nlon, i, j, k)]);
      float dph2 = dref + (pa[ix3(nlat, nlon, i, j, k + 1)] - pa[ix3(nlat, nlon, ip, j, k)]);
      float dgz1 = hl_diff(gz[ix3(nlat, nlon, i, j, k + 1)], gz[ix3(nlat, nlon, ip, j, k)]);
      float dgz2 = hl_diff(gz[ix3(nlat, nlon, i, j, k)], gz[ix3(nlat, nlon, ip, j, k + 1)]);
      return fdiv(-(dph1 * dgz1 + dph2 * dgz2) * inv_d, dph1 + dph2);
    }
    const double *pe = w.ph_exn_lev, *gz = w.gz_lev;
    double dph1 = pe[ix3(nlat, nlon, ip, j, k + 1)] - pe[ix3(nlat, nlon, i, j, k)];
    double dph2 = pe[ix3(nlat, nlon, i, j, k + 1)] - pe[ix3(nlat, nlon, ip, j, k)];
    double dgz1 = gz[ix3(nlat, nlon, i, j, k + 1)] - gz[ix3(nlat, nlon, ip, j, k)];
    double dgz2 = gz[ix3(nlat, nlon, i, j, k)] - gz[ix3(nlat, nlon, ip, j, k + 1)];
    return (R)(-(dph1 * dgz1 + dph2 * dgz2) / ROW(g.de_lon, j) / (dph1 + dph2));
  }
  return (n.gz_f[ix3(nlat, nlon, ip, j, 1)] - n.gz_f[ix3(nlat, nlon, i, j, 1)]) / ROWR(R, de_lon, j);
}
template <class R>
__device__ __forceinline__ R pgf_lat(const DGrid &g, const Slot<R> &n, const Work<R> &w, int i, int j, int k, R inv_d) {
  const int nlat = g.nlat, nlon = g.nlon;
  if (g.baroclinic) {
    if constexpr (std::is_same<R, float>::value) {
      const float *pa = w.pea;
      const float2 *gz = w.gzhl;
      const float dref = g.dpe_ref[k - 1];
      float dph1 = dref + (pa[ix3(nlat, nlon, i, j + 1, k + 1)] - pa[ix3(nlat, nlon, i, j, k)]);
      float dph2 = dref + (pa[ix3(nlat, nlon, i, j, k + 1)] - pa[ix3(nlat, nlon, i, j + 1, k)]);
      float dgz1 = hl_diff(gz[ix3(nlat, nlon, i, j, k + 1)], gz[ix3(nlat, nlon, i, j + 1, k)]);
      float dgz2 = hl_diff(gz[ix3(nlat, nlon, i, j, k)], gz[ix3(nlat, nlon, i, j + 1, k + 1)]);
      return fdiv(-(dph1 * dgz1 + dph2 * dgz2) * inv_d, dph1 + dph2);
    }
    const double *pe = w.ph_exn_lev, *gz = w.gz_lev;
    double dph1 = pe[ix3(nlat, nlon, i, j + 1, k + 1)] - pe[ix3(nlat, nlon, i, j, k)];
    double dph2 = pe[ix3(nlat, nlon, i, j, k + 1)] - pe[ix3(nlat, nlon, i, j + 1, k)];
    double dgz1 = gz[ix3(nlat, nlon, i, j, k + 1)] - gz[ix3(nlat, nlon, i, j + 1, k)];
    double dgz2 = gz[ix3(nlat, nlon, i, j, k)] - gz[ix3(nlat, nlon, i, j + 1, k + 1)];
    return (R)(-(dph1 * dgz1 + dph2 * dgz2) / ROW(g.de_lat, j) / (dph1 + dph2));
  }
  return (n.gz_f[ix3(nlat, nlon, i, j + 1, 1)] - n.gz_f[ix3(nlat, nlon, i, j, 1)]) / ROWR(R, de_lat, j);
}

// FP32 Lin97 pressure-gradient force at the edge between cells p (west or
// south) and q (east or north), offsets at level k; level k+1 is lf further.
// The same operations as the FP32 branch of pgf_lon / pgf_lat.
__device__ __forceinline__ float pgf_pq(const float *__restrict__ pa, const float2 *__restrict__ gz, unsigned p, unsigned q,
                                        unsigned lf, float dref, float inv_d) {
  const float dph1 = dref + (pa[q + lf] - pa[p]);
  const float dph2 = dref + (pa[p + lf] - pa[q]);
  const float dgz1 = hl_diff(gz[p + lf], gz[q]);
  const float dgz2 = hl_diff(gz[p], gz[q + lf]);
  return fdiv(-(dph1 * dgz1 + dph2 * dgz2) * inv_d, dph1 + dph2);
}

__device__ __forceinline__ bool filter_on(const FilterDev &f, bool full_lat, int j) {
  return (full_lat ? f.ntaps_full[j - 1] : f.ntaps_half[j - 1]) > 1;
}

// FP32 Lin97 pressure-gradient force at two neighbouring edges, pgf_pq(p, q)
// and pgf_pq(p2, q2), from the Exner pressures and geopotentials at the four
// distinct points p, p2 (= p + 1 along a row) and q, q2 of a level and the
// level below (lf further); pa_* / gz_* hold those values.  The same
// operations as two pgf_pq calls.
__device__ __forceinline__ float pgf_from(float pa_p, float pa_q, float pa_pl, float pa_ql, float2 gz_p, float2 gz_q,
                                          float2 gz_pl, float2 gz_ql, float dref, float inv_d) {
  const float dph1 = dref + (pa_ql - pa_p);
  const float dph2 = dref + (pa_pl - pa_q);
  const float dgz1 = hl_diff(gz_pl, gz_q);
  const float dgz2 = hl_diff(gz_p, gz_ql);
  return fdiv(-(dph1 * dgz1 + dph2 * dgz2) * inv_d, dph1 + dph2);
}

// Each row is staged in shared memory (also where no filter touches it: the
// stores then do not order the next points' loads behind them).  A block takes
// one row at kUvLevels(R) consecutive levels, so that the filters load each
// weight once for all of them and each thread has more independent loads.
template <class R>
constexpr int kUvLevels = std::is_same<R, float>::value ? 2 : 1;

template <class R, bool MB>
__global__ void GMC_BOUNDS_MB(R, 8, MB) k_update_uv(DGrid g, Slot<R> o, Slot<R> n, Work<R> w, R dt) {
  if constexpr (MB) { to_member(g, o); to_member(g, n); to_member(g, w); }   // member-batched launches
  constexpr int KB = kUvLevels<R>;
  extern __shared__ double sh[];
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon, nlev = g.nlev;
  const int k0 = blockIdx.y * KB + 1;
  const bool bc = g.baroclinic;
  const R dtr = (R)dt;
  const unsigned lf = (unsigned)nlat * nlon;   // level stride of the half-level pea / gzhl
  const int es = nlon + 2 * ((g.big.max_taps - 1) / 2) + 8;   // ext row stride
  R *row = reinterpret_cast<R *>(sh), *nb = row + KB * nlon, *ext = nb + KB * nlon;
  float dref[KB];
#pragma unroll
  for (int kk = 0; kk < KB; ++kk) {
    dref[kk] = 0;
    if constexpr (std::is_same<R, float>::value) dref[kk] = bc && k0 + kk <= nlev ? g.dpe_ref[k0 + kk - 1] : 0.0f;
  }
  // the group's filter: all KB levels together, or one by one for a partial
  // last group
  const int nk = min(KB, nlev - k0 + 1);
  auto filt = [&](const FilterDev &f, bool full, int jj, R *rows) {
    if (nk == KB) return filter_rows<KB, R, R>(f, full, jj, nlon, rows, nlon, ext, es);
    bool any = false;
    for (int kk = 0; kk < nk; ++kk) any = filter_row<R, R>(f, full, jj, nlon, rows + kk * nlon, ext) || any;
    return any;
  };
  if ((int)blockIdx.x < nlat) {
    const int j = blockIdx.x + 1;
    if (j == 1 || j == nlat) {   // pole rows are not updated; the big filter copies them
      for (int kk = 0; kk < nk; ++kk) {
        const unsigned c0 = (unsigned)ix3(nlat, nlon, 1, j, k0 + kk);
        for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) n.u_f[c0 + i0] = n.u_lon[c0 + i0];
      }
      return;
    }
    const R inv_d = (R)1 / ROWR(R, de_lon, j);
    auto val = [&](int kk, int i0) {
      const int k = k0 + kk;
      const unsigned c0 = (unsigned)ix3(nlat, nlon, 1, j, k);
      R p;
      if constexpr (std::is_same<R, float>::value) {
        if (bc) p = pgf_pq(w.pea, w.gzhl, c0 + i0, c0 + (i0 + 1 == nlon ? 0 : i0 + 1), lf, dref[kk], inv_d);
        else p = pgf_lon(g, n, w, i0 + 1, j, k, inv_d);
      } else {
        p = pgf_lon(g, n, w, i0 + 1, j, k, inv_d);
      }
      return o.u_lon[c0 + i0] + dtr * (w.du[c0 + i0] - p);
    };
    const bool small = bc && filter_on(g.small2, true, j), big = filter_on(g.big, true, j);
    bool done = false;
    if constexpr (std::is_same<R, float>::value) {
      if (bc) {   // two points per thread: the pairs (i0, i0+1) and column i0+2 of each row, paired loads
        const float *__restrict__ pa = w.pea;
        const float2 *__restrict__ gz = w.gzhl;
        for (int kk = 0; kk < nk; ++kk) {
          const unsigned c0 = (unsigned)ix3(nlat, nlon, 1, j, k0 + kk);
          for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x) {
            const unsigned a = c0 + i0, e = c0 + (i0 + 2 == nlon ? 0 : i0 + 2);
            const float2 pk = *reinterpret_cast<const float2 *>(pa + a), pl = *reinterpret_cast<const float2 *>(pa + a + lf);
            const float pke = pa[e], ple = pa[e + lf];
            const float4 gk = *reinterpret_cast<const float4 *>(gz + a), gl = *reinterpret_cast<const float4 *>(gz + a + lf);
            const float2 gke = gz[e], gle = gz[e + lf];
            const float2 u2 = *reinterpret_cast<const float2 *>(o.u_lon + a), d2 = *reinterpret_cast<const float2 *>(w.du + a);
            const float p0 = pgf_from(pk.x, pk.y, pl.x, pl.y, make_float2(gk.x, gk.y), make_float2(gk.z, gk.w),
                                      make_float2(gl.x, gl.y), make_float2(gl.z, gl.w), dref[kk], inv_d);
            const float p1 = pgf_from(pk.y, pke, pl.y, ple, make_float2(gk.z, gk.w), gke, make_float2(gl.z, gl.w), gle,
                                      dref[kk], inv_d);
            *reinterpret_cast<float2 *>(row + kk * nlon + i0) =
                make_float2(u2.x + dtr * (d2.x - p0), u2.y + dtr * (d2.y - p1));
          }
        }
        done = true;
      }
    }
    if (!done)
      for (int kk = 0; kk < nk; ++kk)
        for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) row[kk * nlon + i0] = val(kk, i0);
    if (small) filt(g.small2, true, j, row);
    __syncthreads();
    for (int kk = 0; kk < nk; ++kk) {
      const unsigned c0 = (unsigned)ix3(nlat, nlon, 1, j, k0 + kk);
      for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) {
        const R v = row[kk * nlon + i0];
        n.u_lon[c0 + i0] = v;
        if (!isfinite(v)) raise_err(g, ERR_NAN);
        if (!big) n.u_f[c0 + i0] = v;
      }
    }
    if (!big) return;
    filt(g.big, true, j, row);
    __syncthreads();
    for (int kk = 0; kk < nk; ++kk) {
      const unsigned c0 = (unsigned)ix3(nlat, nlon, 1, j, k0 + kk);
      for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) n.u_f[c0 + i0] = row[kk * nlon + i0];
    }
    return;
  }
  const int j = blockIdx.x - nlat + 1;
  auto vval = [&](int kk, int jj, R inv_d, int i0) {
    const int k = k0 + kk;
    const unsigned cv = (unsigned)ix3(nhalf, nlon, 1, jj, k);
    R p;
    if constexpr (std::is_same<R, float>::value) {
      const unsigned ps = (unsigned)ix3(nlat, nlon, 1, jj, k);
      if (bc) p = pgf_pq(w.pea, w.gzhl, ps + i0, ps + nlon + i0, lf, dref[kk], inv_d);
      else p = pgf_lat(g, n, w, i0 + 1, jj, k, inv_d);
    } else {
      p = pgf_lat(g, n, w, i0 + 1, jj, k, inv_d);
    }
    return o.v_lat[cv + i0] + dtr * (w.dv[cv + i0] - p);
  };
  auto load_v = [&](int jj, R *dst) {
    const R inv_d = (R)1 / ROWR(R, de_lat, jj);
    bool done = false;
    if constexpr (std::is_same<R, float>::value) {
      if (bc) {   // two points per thread, paired loads of the full rows jj, jj+1 at both levels
        const float *__restrict__ pa = w.pea;
        const float2 *__restrict__ gz = w.gzhl;
        for (int kk = 0; kk < nk; ++kk) {
          const int k = k0 + kk;
          const unsigned cv = (unsigned)ix3(nhalf, nlon, 1, jj, k), ps = (unsigned)ix3(nlat, nlon, 1, jj, k);
          for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x) {
            const unsigned pp = ps + i0, qq = pp + nlon;
            const float2 ap = *reinterpret_cast<const float2 *>(pa + pp), aq = *reinterpret_cast<const float2 *>(pa + qq);
            const float2 apl = *reinterpret_cast<const float2 *>(pa + pp + lf),
                         aql = *reinterpret_cast<const float2 *>(pa + qq + lf);
            const float4 gp = *reinterpret_cast<const float4 *>(gz + pp), gq = *reinterpret_cast<const float4 *>(gz + qq);
            const float4 gpl = *reinterpret_cast<const float4 *>(gz + pp + lf),
                         gql = *reinterpret_cast<const float4 *>(gz + qq + lf);
            const float2 v2 = *reinterpret_cast<const float2 *>(o.v_lat + cv + i0),
                         d2 = *reinterpret_cast<const float2 *>(w.dv + cv + i0);
            const float p0 = pgf_from(ap.x, aq.x, apl.x, aql.x, make_float2(gp.x, gp.y), make_float2(gq.x, gq.y),
                                      make_float2(gpl.x, gpl.y), make_float2(gql.x, gql.y), dref[kk], inv_d);
            const float p1 = pgf_from(ap.y, aq.y, apl.y, aql.y, make_float2(gp.z, gp.w), make_float2(gq.z, gq.w),
                                      make_float2(gpl.z, gpl.w), make_float2(gql.z, gql.w), dref[kk], inv_d);
            *reinterpret_cast<float2 *>(dst + kk * nlon + i0) =
                make_float2(v2.x + dtr * (d2.x - p0), v2.y + dtr * (d2.y - p1));
          }
        }
        done = true;
      }
    }
    if (!done)
      for (int kk = 0; kk < nk; ++kk)
        for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) dst[kk * nlon + i0] = vval(kk, jj, inv_d, i0);
    if (bc) filt(g.small2, false, jj, dst);
    __syncthreads();
  };
  load_v(j, row);
  if (j == 1 || j == nhalf) {
    load_v(j == 1 ? 2 : nhalf - 1, nb);
    const R wgt = (R)0.6;
    for (int t = threadIdx.x; t < nk * nlon; t += blockDim.x) row[t] = ((R)1 - wgt) * row[t] + wgt * nb[t];
    __syncthreads();
  }
  const bool big = filter_on(g.big, false, j);
  for (int kk = 0; kk < nk; ++kk) {
    const unsigned cj = (unsigned)ix3(nhalf, nlon, 1, j, k0 + kk);
    for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) {
      const R v = row[kk * nlon + i0];
      n.v_lat[cj + i0] = v;
      if (!isfinite(v)) raise_err(g, ERR_NAN);
      if (!big) n.v_f[cj + i0] = v;
    }
  }
  if (!big) return;
  filt(g.big, false, j, row);
  __syncthreads();
  for (int kk = 0; kk < nk; ++kk) {
    const unsigned cj = (unsigned)ix3(nhalf, nlon, 1, j, k0 + kk);
    for (int i0 = threadIdx.x; i0 < nlon; i0 += blockDim.x) n.v_f[cj + i0] = row[kk * nlon + i0];
  }
}

// Run-prologue filters (gmcore_mod.F90:112-122): u_f, v_f, phs_f | gz_f.
template <class R, class T>
__global__ void k_filter_copy(DGrid g, const T *src, T *dst, int which, int full_lat, int nrow) {
  extern __shared__ double sh[];
  const int j = blockIdx.x + 1, k = blockIdx.y + 1, nlon = g.nlon;
  const FilterDev &f = which == 0 ? g.big : which == 1 ? g.small1 : g.small2;
  T *row = reinterpret_cast<T *>(sh), *ext = row + nlon;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) row[i] = src[ix3(nrow, nlon, i + 1, j, k)];
  // FP32 rows of the FP32 form accumulate in FP32 like the step's own filters
  filter_row<T, typename std::conditional<std::is_same<T, float>::value, float, double>::type>(f, full_lat != 0, j, nlon,
                                                                                               row, ext);
  __syncthreads();
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) dst[ix3(nrow, nlon, i + 1, j, k)] = row[i];
}

// ---------------------------------------------------------------------------
// diagnose (gmcore_mod.F90:213-341): block partial sums with compensated
// (Neumaier) accumulation, reduced by one block in fixed order.
// ---------------------------------------------------------------------------
struct KSum {
  double s = 0, c = 0;
  __device__ void add(double x) {
    double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x; else c += (x - t) + s;
    s = t;
  }
  __device__ double value() const { return s + c; }
};

template <class R>
__global__ void k_diag_partial(DGrid g, Slot<R> s, double *partial) {
  __shared__ double red[32];
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  const MassField<R> M = mass_of(g, s);
  KSum tm, teke, teie, tepe, tav, tpe, tpt;
  const double ac = ROW(g.area_cell, j);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const size_t o = ix3(nlat, nlon, i, j, k);
    const size_t c2 = (size_t)(j - 1) * nlon + (i - 1);
    double m = (double)M.at(g, i, j, k);
    tm.add(m * ac);
    if (j != 1 && j != nlat) teke.add((double)s.mfx_lon[o] * 0.5 * (double)s.u_lon[o] * ROW(g.area_lon, j) * 2);
    if (g.baroclinic) {
      double pl0 = ph_lev(g, k, s.phs_f[c2]), pl1 = ph_lev(g, k + 1, s.phs_f[c2]);
      double ph = 0.5 * (pl0 + pl1);
      double t = (double)s.pt[o] * pow(ph / g.p0, g.kappa);
      teie.add(m * g.cpd * t * ac);
      tpt.add(m * (double)s.pt[o] * ac);
      if (k == 1) tepe.add(s.gzs[c2] * s.phs[c2] * ac);
    } else {
      tepe.add((m * m * g.g * 0.5 + m * s.gzs[c2]) * ac);
    }
    if (j != 1 && j != nlat) {
      double m_lon = 0.5 * ((double)M.at(g, i, j, k) + (double)M.at(g, i + 1, j, k));
      double pl = (double)s.pv_lon[o];
      tpe.add(m_lon * (pl * pl) * 0.5 * ROW(g.area_lon, j));
    }
    if (j <= nhalf) {
      const size_t oh = ix3(nhalf, nlon, i, j, k);
      teke.add((double)s.mfy_lat[oh] * 0.5 * (double)s.v_lat[oh] * ROW(g.area_lat, j) * 2);
      tav.add((double)s.pv[oh] * ROW(g.area_vtx, j));
      double m_lat = 0.5 * ((double)M.at(g, i, j, k) + (double)M.at(g, i, j + 1, k));
      double pl = (double)s.pv_lat[oh];
      tpe.add(m_lat * (pl * pl) * 0.5 * ROW(g.area_lat, j));
    }
  }
  double vals[7] = {tm.value(), teke.value(), teie.value(), tepe.value(), tav.value(), tpe.value(), tpt.value()};
  const size_t b = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
  for (int q = 0; q < 7; ++q) {
    double t = block_sum(vals[q], red);
    if (threadIdx.x == 0) partial[(size_t)q * gridDim.x * gridDim.y + b] = t;
  }
}

__global__ void k_diag_final(const double *partial, int nblk, double *out) {
  __shared__ double red[32];
  for (int q = 0; q < 7; ++q) {
    KSum acc;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc.add(partial[(size_t)q * nblk + b]);
    // combine the per-thread compensated sums in fixed order
    double s = block_sum(acc.s, red), c = block_sum(acc.c, red);
    if (threadIdx.x == 0) out[q] = s + c;
  }
}

inline size_t filter_smem(const DGrid &g, int rows, size_t elem) {
  int hmax = (g.big.max_taps - 1) / 2;
  return (size_t)(rows * g.nlon + g.nlon + 2 * hmax + 8) * elem;
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
template <class R>
void launch_mass_flux(const DGrid &g, const Launch &L, const Slot<R> &s) {
  const int bt = std::is_same<R, float>::value && g.baroclinic ? 128 : L.threads;   // FP32: two points per thread
  mb_launch(L, [&](auto mb) { k_mass_flux<R, decltype(mb)::value><<<dim3(g.nlat, g.nlev, L.members), bt, 0, L.stream>>>(g, s); });
}
template <class R>
void launch_tangent_winds(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w) {
  const int bt = std::is_same<R, float>::value && g.baroclinic ? 128 : L.threads;   // FP32: two points per thread
  mb_launch(L, [&](auto mb) { k_tangent_winds<R, decltype(mb)::value><<<dim3(g.nlat, g.nlev, L.members), bt, 0, L.stream>>>(g, s, w); });
}
template <class R>
void launch_kinetic_energy(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w) {
  // FP32: two points per thread, so smaller blocks
  const int bt = std::is_same<R, float>::value ? 128 : L.threads;
  mb_launch(L, [&](auto mb) { k_kinetic_energy<R, decltype(mb)::value><<<dim3(g.nlat, g.nlev, L.members), bt, 0, L.stream>>>(g, s, w); });
}
template <class R>
void launch_pv(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w) {
  const int bt = std::is_same<R, float>::value && g.baroclinic ? 128 : L.threads;   // FP32: two points per thread
  mb_launch(L, [&](auto mb) { k_pv<R, decltype(mb)::value><<<dim3(g.nhalf, g.nlev, L.members), bt, 0, L.stream>>>(g, s, w); });
}
template <class R>
void launch_pv_edges(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w, double dt) {
  const int bt = std::is_same<R, float>::value && g.baroclinic ? 128 : L.threads;   // FP32: two points per thread
  mb_launch(L, [&](auto mb) { k_pv_edges<R, decltype(mb)::value><<<dim3(g.nlat, g.nlev, L.members), bt, 0, L.stream>>>(g, s, w, dt); });
}
template <class R>
void launch_batch_cfl(const DGrid &g, const Launch &L, const R *u, const R *v, R *cflx, R *cfly, R *divx, R *divy, double dt) {
  const size_t smem = std::is_same<R, float>::value ? g.nlon * sizeof(float) : 0;
  mb_launch(L, [&](auto mb) { k_batch_cfl<R, decltype(mb)::value><<<dim3(g.nlat, g.nlev, L.members), L.threads, smem, L.stream>>>(g, u, v, cflx, cfly, divx, divy, dt); });
}
template <class R>
void launch_column_mass(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w, double dt) {
  if constexpr (std::is_same<R, float>::value) {
    const size_t smem = g.nlev * sizeof(double) + (size_t)(2 * g.nlev + 1) * (kTileI + 1) * sizeof(float) +
                        (size_t)(3 * g.nlev + 1) * sizeof(float);
    if (smem > 48 * 1024) { cudaFuncSetAttribute(k_column_mass_f<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); cudaFuncSetAttribute(k_column_mass_f<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); }
    mb_launch(L, [&](auto mb) { k_column_mass_f<decltype(mb)::value><<<dim3((g.nlon + kTileI - 1) / kTileI, g.nlat, L.members), dim3(kTileI, kTileK), smem, L.stream>>>(g, s, w, dt); });
    return;
  }
  const int bt = 64;
  size_t smem = (32 + g.nlev + 2) * sizeof(double);
  mb_launch(L, [&](auto mb) { k_column_mass<R, decltype(mb)::value><<<dim3((g.nlon + bt - 1) / bt, g.nlat, L.members), bt, smem, L.stream>>>(g, s, w, dt); });
}
template <class R>
void launch_momentum_tend(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w) {
  if constexpr (std::is_same<R, float>::value) {
    if (g.baroclinic) {
      mb_launch(L, [&](auto mb) { k_momentum_f<decltype(mb)::value><<<dim3(g.nlat - 2 + g.nhalf, g.nlev, L.members), 128, 0, L.stream>>>(g, s.mfx_lon, s.mfy_lat, s.pv_lon, s.pv_lat, w.ke, s.we_lev,
                                                              s.u_f, s.v_f, s.psr, w.du, w.dv); });
      return;
    }
  }
  mb_launch(L, [&](auto mb) { k_momentum_tend<R, decltype(mb)::value><<<dim3(g.nlat, g.nlev, L.members), L.threads, 0, L.stream>>>(g, s, w); });
}
template <class R>
void launch_swm_dgz(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w) {
  mb_launch(L, [&](auto mb) { k_swm_dgz<R, decltype(mb)::value><<<dim3(g.nlat, 1, L.members), L.threads, 0, L.stream>>>(g, s, w); });
}
template <class R>
void launch_update_phs(const DGrid &g, const Launch &L, const Slot<R> &o, const Slot<R> &n, const Work<R> &w, double dt) {
  allow_smem(k_update_phs<R, false>, filter_smem(g, 1, sizeof(double))); allow_smem(k_update_phs<R, true>, filter_smem(g, 1, sizeof(double)));
  mb_launch(L, [&](auto mb) { k_update_phs<R, decltype(mb)::value><<<dim3(g.nlat, 1, L.members), L.threads, filter_smem(g, 1, sizeof(double)), L.stream>>>(g, o, n, w, dt); });
}
template <class R>
void launch_update_pt(const DGrid &g, const Launch &L, const Slot<R> &o, const Slot<R> &n, const Work<R> &w, double dt) {
  constexpr int KB = kPtLevels<R>;
  const int hmax = (g.big.max_taps - 1) / 2;
  const size_t smem = (size_t)KB * (g.nlon + g.nlon + 2 * hmax + 8) * sizeof(R);
  allow_smem(k_update_pt<R, false>, smem); allow_smem(k_update_pt<R, true>, smem);
  mb_launch(L, [&](auto mb) { k_update_pt<R, decltype(mb)::value><<<dim3(g.nlat, (g.nlev + KB - 1) / KB, L.members), L.threads, smem, L.stream>>>(g, o, n, w, dt); });
}
template <class R>
void launch_update_gz(const DGrid &g, const Launch &L, const Slot<R> &o, const Slot<R> &n, const Work<R> &w, double dt) {
  allow_smem(k_update_gz<R, false>, filter_smem(g, 2, sizeof(R))); allow_smem(k_update_gz<R, true>, filter_smem(g, 2, sizeof(R)));
  mb_launch(L, [&](auto mb) { k_update_gz<R, decltype(mb)::value><<<dim3(g.nlat, 1, L.members), L.threads, filter_smem(g, 2, sizeof(R)), L.stream>>>(g, o, n, w, dt); });
}
template <class R>
void launch_column_backward(const DGrid &g, const Launch &L, const Slot<R> &n, const Work<R> &w) {
  const int bt = 64;
  mb_launch(L, [&](auto mb) { k_column_backward<R, decltype(mb)::value><<<dim3((g.nlon + bt - 1) / bt, g.nlat, L.members), bt, 0, L.stream>>>(g, n, w); });
}
template <class R>
void launch_update_uv(const DGrid &g, const Launch &L, const Slot<R> &o, const Slot<R> &n, const Work<R> &w, double dt) {
  constexpr int KB = kUvLevels<R>;
  const int hmax = (g.big.max_taps - 1) / 2;
  const size_t smem = (size_t)KB * (2 * g.nlon + g.nlon + 2 * hmax + 8) * sizeof(R);
  allow_smem(k_update_uv<R, false>, smem); allow_smem(k_update_uv<R, true>, smem);
  mb_launch(L, [&](auto mb) { k_update_uv<R, decltype(mb)::value><<<dim3(g.nlat + g.nhalf, (g.nlev + KB - 1) / KB, L.members), L.threads, smem, L.stream>>>(g, o, n, w, dt); });
}
template <class R>
void launch_filter_prologue(const DGrid &g, const Launch &L, const Slot<R> &s) {
  allow_smem(k_filter_copy<R, R>, filter_smem(g, 1, sizeof(R)));
  allow_smem(k_filter_copy<R, double>, filter_smem(g, 1, sizeof(double)));
  k_filter_copy<R, R><<<dim3(g.nlat, g.nlev), L.threads, filter_smem(g, 1, sizeof(R)), L.stream>>>(g, s.u_lon, s.u_f, 0, 1, g.nlat);
  k_filter_copy<R, R><<<dim3(g.nhalf, g.nlev), L.threads, filter_smem(g, 1, sizeof(R)), L.stream>>>(g, s.v_lat, s.v_f, 0, 0, g.nhalf);
  if (g.baroclinic)
    k_filter_copy<R, double><<<dim3(g.nlat, 1), L.threads, filter_smem(g, 1, sizeof(double)), L.stream>>>(g, s.phs, s.phs_f, 0, 1, g.nlat);
  else
    k_filter_copy<R, R><<<dim3(g.nlat, 1), L.threads, filter_smem(g, 1, sizeof(R)), L.stream>>>(g, s.gz, s.gz_f, 0, 1, g.nlat);
}
template <class R>
void launch_surface_rel(const DGrid &g, const Launch &L, const Slot<R> &s) {
  if (!s.psr || !s.phs_f) return;
  const size_t n = (size_t)g.nlat * g.nlon;
  k_surface_rel<<<(int)std::min<size_t>((n + 255) / 256, 152 * 8), 256, 0, L.stream>>>(s.phs_f, s.psr, n, g.ptop);
}
template <class R>
void launch_check_columns(const DGrid &g, const Launch &L, const Slot<R> &s) {
  if (!s.phs_f) return;
  const size_t n = (size_t)g.nlat * g.nlon;
  k_check_columns<<<(int)std::min<size_t>((n + 255) / 256, 152 * 8), 256, 0, L.stream>>>(g, s.phs_f, s.psr, n);
}
template <class R>
void launch_diagnose(const DGrid &g, const Launch &L, const Slot<R> &s, double *partial, double *out) {
  k_diag_partial<R><<<dim3(g.nlat, g.nlev), L.threads, 0, L.stream>>>(g, s, partial);
  k_diag_final<<<1, 256, 0, L.stream>>>(partial, g.nlat * g.nlev, out);
}

#define INSTANTIATE(R)                                                                                              \
  template void launch_mass_flux<R>(const DGrid &, const Launch &, const Slot<R> &);                              \
  template void launch_tangent_winds<R>(const DGrid &, const Launch &, const Slot<R> &, const Work<R> &);         \
  template void launch_kinetic_energy<R>(const DGrid &, const Launch &, const Slot<R> &, const Work<R> &);        \
  template void launch_pv<R>(const DGrid &, const Launch &, const Slot<R> &, const Work<R> &);                    \
  template void launch_pv_edges<R>(const DGrid &, const Launch &, const Slot<R> &, const Work<R> &, double);      \
  template void launch_batch_cfl<R>(const DGrid &, const Launch &, const R *, const R *, R *, R *, R *, R *, double); \
  template void launch_column_mass<R>(const DGrid &, const Launch &, const Slot<R> &, const Work<R> &, double);   \
  template void launch_momentum_tend<R>(const DGrid &, const Launch &, const Slot<R> &, const Work<R> &);         \
  template void launch_swm_dgz<R>(const DGrid &, const Launch &, const Slot<R> &, const Work<R> &);               \
  template void launch_update_phs<R>(const DGrid &, const Launch &, const Slot<R> &, const Slot<R> &, const Work<R> &, double); \
  template void launch_update_pt<R>(const DGrid &, const Launch &, const Slot<R> &, const Slot<R> &, const Work<R> &, double);  \
  template void launch_update_gz<R>(const DGrid &, const Launch &, const Slot<R> &, const Slot<R> &, const Work<R> &, double);  \
  template void launch_column_backward<R>(const DGrid &, const Launch &, const Slot<R> &, const Work<R> &);       \
  template void launch_surface_rel<R>(const DGrid &, const Launch &, const Slot<R> &);                             \
  template void launch_check_columns<R>(const DGrid &, const Launch &, const Slot<R> &);                           \
  template void launch_update_uv<R>(const DGrid &, const Launch &, const Slot<R> &, const Slot<R> &, const Work<R> &, double);  \
  template void launch_filter_prologue<R>(const DGrid &, const Launch &, const Slot<R> &);                        \
  template void launch_diagnose<R>(const DGrid &, const Launch &, const Slot<R> &, double *, double *);

INSTANTIATE(double)
INSTANTIATE(float)

}  // namespace gmc

namespace gmc {
namespace {

// calc_div, order-2 branch (operators_mod.F90:354-412), on the filtered wind.
template <class R, bool MB>
__global__ void k_div(DGrid g, Slot<R> n, R *div) {
  if constexpr (MB) { to_member(g, n); div = mshift(div, member_offset(g)); }   // member-batched launches
  __shared__ double red[32];
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  if (j == 1 || j == nlat) {
    const int jv = j == 1 ? 1 : nhalf;
    const double sgn = j == 1 ? 1.0 : -1.0;
    double p = ring_sum(nlon, red, [&](int i) { return sgn * (double)n.v_f[ix3(nhalf, nlon, i, jv, k)]; });
    p = p * ROW(g.le_lat, jv) / nlon / ROW(g.area_cell, j);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) div[ix3(nlat, nlon, i, j, k)] = (R)p;
    return;
  }
  const R lel = ROWR(R, le_lon, j), ac = ROWR(R, area_cell, j), la0 = ROWR(R, le_lat, j), la1 = ROWR(R, le_lat, j - 1);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    R ue = n.u_f[ix3(nlat, nlon, i, j, k)], uw = n.u_f[ix3(nlat, nlon, wrap(i - 1, nlon), j, k)];
    R vn = n.v_f[ix3(nhalf, nlon, i, j, k)], vs = n.v_f[ix3(nhalf, nlon, i, j - 1, k)];
    div[ix3(nlat, nlon, i, j, k)] = ((ue * lel - uw * lel) + (vn * la0 - vs * la1)) / ac;
  }
}

// div2 = Laplacian of div on non-pole rows (operators_mod.F90:412-425); pole
// rows stay zero as the reference's zero-initialised array leaves them.
template <class R, bool MB>
__global__ void k_div2(DGrid g, const R *div, R *div2) {
  if constexpr (MB) { const size_t mo = member_offset(g); div = mshift(div, mo); div2 = mshift(div2, mo); }
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nlon = g.nlon;
  if (j == 1 || j == nlat) {
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) div2[ix3(nlat, nlon, i, j, k)] = (R)0;
    return;
  }
  const R dl = ROWR(R, de_lon, j), c0 = ROWR(R, half_cos_lat, j), c1 = ROWR(R, half_cos_lat, j - 1);
  const R d0 = ROWR(R, de_lat, j), d1 = ROWR(R, de_lat, j - 1), le = ROWR(R, le_lon, j), cf = ROWR(R, full_cos_lat, j);
  auto D = [&](int i, int jj) { return div[ix3(nlat, nlon, wrap(i, nlon), jj, k)]; };
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    const R d = D(i, j);
    div2[ix3(nlat, nlon, i, j, k)] =
        (D(i + 1, j) - (R)2 * d + D(i - 1, j)) / (dl * dl) + ((D(i, j + 1) - d) * c0 / d0 - (d - D(i, j - 1)) * c1 / d1) / le / cf;
  }
}

// order 2: u += c (div(i+1) - div(i)) / de; order 4: u -= c (div2(i+1) - div2(i)) / de
template <class R, bool MB>
__global__ void k_div_damp(DGrid g, Slot<R> n, const R *div) {
  if constexpr (MB) { to_member(g, n); div = mshift(div, member_offset(g)); }   // member-batched launches
  const R sgn = g.div_damp_order == 4 ? (R)-1 : (R)1;
  const int k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  if ((int)blockIdx.x < nlat) {
    const int j = blockIdx.x + 1;
    if (j == 1 || j == nlat) return;
    const R c = (R)g.div_c_lon[(size_t)(k - 1) * nlat + (j - 1)], de = ROWR(R, de_lon, j);
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      size_t o = ix3(nlat, nlon, i, j, k);
      n.u_lon[o] = n.u_lon[o] + sgn * (c * (div[ix3(nlat, nlon, wrap(i + 1, nlon), j, k)] - div[o]) / de);
    }
    return;
  }
  const int j = blockIdx.x - nlat + 1;
  const R c = (R)g.div_c_lat[(size_t)(k - 1) * nhalf + (j - 1)], de = ROWR(R, de_lat, j);
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
    size_t o = ix3(nhalf, nlon, i, j, k);
    n.v_lat[o] = n.v_lat[o] + sgn * (c * (div[ix3(nlat, nlon, i, j + 1, k)] - div[ix3(nlat, nlon, i, j, k)]) / de);
  }
}

// Held-Suarez forcing of the new state after the integrator (test_forcing_run,
// gmcore_mod.F90:586; held_suarez_test_apply_forcing,
// held_suarez_test_mod.F90:74-112): Rayleigh friction kv(sigma) of u (no pole
// rows) and v below sigma_b = 0.7, and Newtonian relaxation of pt at rate
// kt(sigma, lat) toward the equilibrium temperature Teq(p, lat).  The pressure
// is the full-level mean of the half levels from phs_f and the temperature
// pt (p/p0)^kappa, as calc_ph and calc_t (operators_mod.F90:136-190) leave
// them in the new state.  Blocks 0 .. nlat-1 take the full rows (u and pt),
// the rest the half rows (v).
template <class R, bool MB>
__global__ void k_held_suarez(DGrid g, Slot<R> n, double dt) {
  if constexpr (MB) { to_member(g, n); }   // member-batched launches
  const int k = blockIdx.y + 1, nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  constexpr double sig_b = 0.7, kf = 1.0 / 86400.0, ka = 0.025 / 86400.0, ks = 0.25 / 86400.0;
  constexpr double dt_lat = 60.0, dpt_lev = 10.0, p0 = 1.0e5;   // K, K, Pa
  const double sfac = fmax(0.0, (g.full_lev[k - 1] - sig_b) / (1.0 - sig_b));
  const R ckv = (R)(dt * (kf * sfac));
  if ((int)blockIdx.x >= nlat) {
    const int j = blockIdx.x - nlat + 1;
    const unsigned c0 = (unsigned)ix3(nhalf, nlon, 1, j, k);
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) n.v_lat[c0 + i] = n.v_lat[c0 + i] - ckv * n.v_lat[c0 + i];
    return;
  }
  const int j = blockIdx.x + 1;
  const unsigned c0 = (unsigned)ix3(nlat, nlon, 1, j, k), m0 = (unsigned)(j - 1) * nlon;
  if (j != 1 && j != nlat)
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) n.u_lon[c0 + i] = n.u_lon[c0 + i] - ckv * n.u_lon[c0 + i];
  const double c = ROW(g.full_cos_lat, j), sn = ROW(g.full_sin_lat, j), c2 = c * c;
  const double kt = ka + (ks - ka) * sfac * (c2 * c2);
  if constexpr (std::is_same<R, double>::value) {
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
      const double phs = n.phs_f[m0 + i];
      const double ph = 0.5 * (ph_lev(g, k, phs) + ph_lev(g, k + 1, phs));
      const double p_p0 = ph / p0, pw = pow(p_p0, g.kappa);
      const double pt = n.pt[c0 + i], t = pt * pw;
      const double teq = fmax(200.0, (315.0 - dt_lat * (sn * sn) - dpt_lev * log(p_p0) * c2) * pw);
      n.pt[c0 + i] = pt - dt * kt * pt * (1.0 - teq / t);
    }
  } else {   // FP32: pressure from psr = phs_f - ptop
    const float a0 = g.ph_lev_a[k - 1], a1 = g.ph_lev_a[k], b0 = g.hybi_f[k - 1], b1 = g.hybi_f[k];
    const float s2 = (float)(dt_lat * (sn * sn)), d2 = (float)(dpt_lev * c2), ckt = (float)(dt * kt);
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
      const float psr = n.psr[m0 + i];
      const float ph = 0.5f * (fmaf(b0, psr, a0) + fmaf(b1, psr, a1));
      const float p_p0 = ph * (float)(1.0 / p0), pw = powf(p_p0, g.kappa_f);
      const float pt = n.pt[c0 + i], t = pt * pw;
      const float teq = fmaxf(200.0f, (315.0f - s2 - d2 * logf(p_p0)) * pw);
      n.pt[c0 + i] = pt - ckt * pt * (1.0f - teq / t);
    }
  }
}

// Smagorinsky damping (smag_damp_run, smag_damp_mod.F90:52-190, with
// decay_from_top = 1 as smag_damp_init leaves it, :36): horizontal tension at
// cells (full rows 2 .. nlat-1; the pole rows hold the zero the reference's
// working array was allocated with) and shear at vertices.  Blocks 0 .. nlat-1
// take the full rows, the rest the half rows.
template <class R, bool MB>
__global__ void k_smag_ts(DGrid g, Slot<R> n, R *st, R *ss) {
  if constexpr (MB) { to_member(g, n); const size_t mo = member_offset(g); st = mshift(st, mo); ss = mshift(ss, mo); }
  const int k = blockIdx.y + 1, nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  const R *u = n.u_lon, *v = n.v_lat;
  if ((int)blockIdx.x < nlat) {
    const int j = blockIdx.x + 1;
    const unsigned c0 = (unsigned)ix3(nlat, nlon, 1, j, k);
    if (j == 1 || j == nlat) {
      for (int i = threadIdx.x; i < nlon; i += blockDim.x) st[c0 + i] = (R)0;
      return;
    }
    const unsigned hn = (unsigned)ix3(nhalf, nlon, 1, j, k), hs = hn - nlon;
    const R dx = ROWR(R, de_lon, j), ly = ROWR(R, le_lon, j), fc = ROWR(R, full_cos_lat, j);
    const R hcn = ROWR(R, half_cos_lat, j), hcs = ROWR(R, half_cos_lat, j - 1);
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
      const int iw = i == 0 ? nlon - 1 : i - 1;
      st[c0 + i] = (u[c0 + i] - u[c0 + iw]) / dx - (v[hn + i] * hcn - v[hs + i] * hcs) / ly / fc;
    }
    return;
  }
  const int j = blockIdx.x - nlat + 1;
  const unsigned h0 = (unsigned)ix3(nhalf, nlon, 1, j, k), fs = (unsigned)ix3(nlat, nlon, 1, j, k), fn = fs + nlon;
  const R lx = ROWR(R, le_lat, j), dy = ROWR(R, de_lat, j), hc = ROWR(R, half_cos_lat, j);
  const R fcs = ROWR(R, full_cos_lat, j), fcn = ROWR(R, full_cos_lat, j + 1);
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    const int ie = i + 1 == nlon ? 0 : i + 1;
    ss[h0 + i] = (v[h0 + ie] - v[h0 + i]) / lx + (u[fn + i] * fcn - u[fs + i] * fcs) / dy / hc;
  }
}

// The damping tendencies with the eddy viscosities at the u and v points
// formed from the tension and shear around them (kmh_lon, kmh_lat).
template <class R, bool MB>
__global__ void k_smag_tend(DGrid g, Slot<R> n, const R *st, const R *ss, R *du, R *dv) {
  if constexpr (MB) {
    to_member(g, n);
    const size_t mo = member_offset(g);
    st = mshift(st, mo); ss = mshift(ss, mo); du = mshift(du, mo); dv = mshift(dv, mo);
  }
  const int k = blockIdx.y + 1, nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  const R *u = n.u_lon, *v = n.v_lat;
  const R coef = (R)g.smag_coef;
  auto sq = [](R x) { return x * x; };
  if ((int)blockIdx.x < nlat) {
    const int j = blockIdx.x + 1;
    if (j == 1 || j == nlat) return;
    const unsigned c0 = (unsigned)ix3(nlat, nlon, 1, j, k), hn = (unsigned)ix3(nhalf, nlon, 1, j, k), hs = hn - nlon;
    const R dx = ROWR(R, de_lon, j), ly = ROWR(R, le_lon, j), fc = ROWR(R, full_cos_lat, j);
    const R dyn = ROWR(R, de_lat, j), dys = ROWR(R, de_lat, j - 1), hcn = ROWR(R, half_cos_lat, j),
            hcs = ROWR(R, half_cos_lat, j - 1);
    const R ls2 = coef / ((R)1 / sq(dx) + (R)1 / sq(ly));
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
      const int iw = i == 0 ? nlon - 1 : i - 1, ie = i + 1 == nlon ? 0 : i + 1;
      const R kmh = ls2 * sqrt((R)0.5 * (sq(st[c0 + i]) + sq(st[c0 + ie])) + (R)0.5 * (sq(ss[hn + i]) + sq(ss[hs + i])));
      const R uc = u[c0 + i];
      du[c0 + i] = kmh * ((u[c0 + iw] - (R)2 * uc + u[c0 + ie]) / sq(dx) +
                          ((u[c0 + nlon + i] - uc) / dyn * hcn - (uc - u[c0 - nlon + i]) / dys * hcs) / ly / fc);
    }
    return;
  }
  const int j = blockIdx.x - nlat + 1;
  const unsigned h0 = (unsigned)ix3(nhalf, nlon, 1, j, k), fs = (unsigned)ix3(nlat, nlon, 1, j, k);
  const R lx = ROWR(R, le_lat, j), dy = ROWR(R, de_lat, j), hc = ROWR(R, half_cos_lat, j);
  const R ls2 = coef / ((R)1 / sq(lx) + (R)1 / sq(dy));
  const bool edge = j == 1 || j == nhalf;
  const R lyn = ROWR(R, le_lon, j + 1), lys = ROWR(R, le_lon, j), fcn = ROWR(R, full_cos_lat, j + 1),
          fcs = ROWR(R, full_cos_lat, j);
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    const int iw = i == 0 ? nlon - 1 : i - 1, ie = i + 1 == nlon ? 0 : i + 1;
    const R kmh = ls2 * sqrt((R)0.5 * (sq(st[fs + i]) + sq(st[fs + nlon + i])) + (R)0.5 * (sq(ss[h0 + i]) + sq(ss[h0 + iw])));
    const R vc = v[h0 + i];
    R t = (v[h0 + iw] - (R)2 * vc + v[h0 + ie]) / sq(lx);
    if (!edge) t = t + ((v[h0 + nlon + i] - vc) / lyn * fcn - (vc - v[h0 - nlon + i]) / lys * fcs) / dy / hc;
    dv[h0 + i] = kmh * t;
  }
}

// u += dt dudt (rows 2 .. nlat-1), v += dt dvdt
template <class R, bool MB>
__global__ void k_smag_update(DGrid g, Slot<R> n, const R *du, const R *dv, R dt) {
  if constexpr (MB) { to_member(g, n); const size_t mo = member_offset(g); du = mshift(du, mo); dv = mshift(dv, mo); }
  const int k = blockIdx.y + 1, nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  if ((int)blockIdx.x < nlat) {
    const int j = blockIdx.x + 1;
    if (j == 1 || j == nlat) return;
    const unsigned c0 = (unsigned)ix3(nlat, nlon, 1, j, k);
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) n.u_lon[c0 + i] = n.u_lon[c0 + i] + dt * du[c0 + i];
    return;
  }
  const int j = blockIdx.x - nlat + 1;
  const unsigned h0 = (unsigned)ix3(nhalf, nlon, 1, j, k);
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) n.v_lat[h0 + i] = n.v_lat[h0 + i] + dt * dv[h0 + i];
}

}  // namespace

template <class R>
void launch_smag_damp(const DGrid &g, const Launch &L, const Slot<R> &n, R *st, R *ss, R *du, R *dv, double dt) {
  const dim3 grid(g.nlat + g.nhalf, g.nlev, L.members);
  mb_launch(L, [&](auto mb) { k_smag_ts<R, decltype(mb)::value><<<grid, L.threads, 0, L.stream>>>(g, n, st, ss); });
  mb_launch(L, [&](auto mb) { k_smag_tend<R, decltype(mb)::value><<<grid, L.threads, 0, L.stream>>>(g, n, st, ss, du, dv); });
  mb_launch(L, [&](auto mb) { k_smag_update<R, decltype(mb)::value><<<grid, L.threads, 0, L.stream>>>(g, n, du, dv, (R)dt); });
}
template void launch_smag_damp<double>(const DGrid &, const Launch &, const Slot<double> &, double *, double *, double *,
                                       double *, double);
template void launch_smag_damp<float>(const DGrid &, const Launch &, const Slot<float> &, float *, float *, float *,
                                      float *, double);

template <class R>
void launch_div_damp(const DGrid &g, const Launch &L, const Slot<R> &n, R *div, R *div2) {
  mb_launch(L, [&](auto mb) { k_div<R, decltype(mb)::value><<<dim3(g.nlat, g.nlev, L.members), L.threads, 0, L.stream>>>(g, n, div); });
  if (g.div_damp_order == 4) {
    mb_launch(L, [&](auto mb) { k_div2<R, decltype(mb)::value><<<dim3(g.nlat, g.nlev, L.members), L.threads, 0, L.stream>>>(g, div, div2); });
    mb_launch(L, [&](auto mb) { k_div_damp<R, decltype(mb)::value><<<dim3(g.nlat + g.nhalf, g.nlev, L.members), L.threads, 0, L.stream>>>(g, n, div2); });
  } else {
    mb_launch(L, [&](auto mb) { k_div_damp<R, decltype(mb)::value><<<dim3(g.nlat + g.nhalf, g.nlev, L.members), L.threads, 0, L.stream>>>(g, n, div); });
  }
}
template void launch_div_damp<double>(const DGrid &, const Launch &, const Slot<double> &, double *, double *);
template void launch_div_damp<float>(const DGrid &, const Launch &, const Slot<float> &, float *, float *);

template <class R>
void launch_held_suarez(const DGrid &g, const Launch &L, const Slot<R> &n, double dt) {
  mb_launch(L, [&](auto mb) { k_held_suarez<R, decltype(mb)::value><<<dim3(g.nlat + g.nhalf, g.nlev, L.members), L.threads, 0, L.stream>>>(g, n, dt); });
}
template void launch_held_suarez<double>(const DGrid &, const Launch &, const Slot<double> &, double);
template void launch_held_suarez<float>(const DGrid &, const Launch &, const Slot<float> &, double);

}  // namespace gmc
