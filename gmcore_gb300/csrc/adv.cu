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

#include <algorithm>
#include <type_traits>

#include "kernels.hpp"
#include "stencil.cuh"

namespace gmc {

namespace {

// One horizontal pass of hflx_ppm_cell (ffsl_mod.F90:778-881): x fluxes on
// full-latitude rows without the poles, y fluxes on half-latitude rows.
//   u, v  : advecting velocities (or mass fluxes for the outer operator)
//   mx    : field reconstructed along x;  my : field reconstructed along y.
// Along x a block takes one full row: the row is staged in shared memory
// with wrapped ends, each cell's slope formed once, and each face forms the
// limited coefficients of its upwind cell.  Along y each thread marches one
// column north through a band of rows with a rolling window in registers
// (YMarch).  Pole halo rows are read as the reference's fill_halo leaves them
// (mirrored row shifted by nlon/2).

// x fluxes of full row j (2 .. nlat-1) at level k of NF fields that share the
// Courant numbers cflx: field f is fld[f] advected by the multiplier mul[f]
// (a velocity or a mass flux); out(i0, o, flux[NF]) per face i0 (0-based; the
// face east of cell i0) at 32-bit offset o.  Shared memory: xs holds the NF
// rows with wrapped cells beyond both ends, X_f[l] = xs[f * (nlon + 5) + 2 + l]
// for l = -2 .. nlon+2, and ss their limited slopes, S_f[l] = ss[f * (nlon + 3)
// + 1 + l] for l = -1 .. nlon+1, so no face indexes modulo nlon.  Each cell's
// slope (slope_mono, ffsl_mod.F90:1183-1194) is formed once and read by the
// faces whose upwind cell or neighbour it is; the upwind cell, the whole-cell
// count and the fractional Courant number are formed once per face for all
// fields.  Row offsets are 32-bit (grids are validated to < 2^31 cells).
template <int NF, class R, class Out>
__device__ __forceinline__ void hflx_xrows(const DGrid &g, int j, int k, const R *const (&mul)[NF],
                                           const R *__restrict__ cflx, const R *const (&fld)[NF], R *xs, R *ss,
                                           Out out) {
  const int nlon = g.nlon, lim = g.limiter, xw = nlon + 5, sw = nlon + 3;
  auto Wg = [nlon](int l) {   // any l (a Courant number may exceed nlon on coarse grids)
    if (l >= 0 && l < nlon) return l;
    l %= nlon;
    return l < 0 ? l + nlon : l;
  };
  const unsigned ro = (unsigned)ix3(g.nlat, nlon, 1, j, k);
  // face inputs of this thread's first faces are requested before the rows
  // are staged so that their latency overlaps it
  constexpr int kPre = 3;
  R cpre[kPre], mpre[NF][kPre];
#pragma unroll
  for (int t = 0; t < kPre; ++t) {
    const int i0 = threadIdx.x + t * blockDim.x;
    if (i0 < nlon) {
      cpre[t] = cflx[ro + i0];
#pragma unroll
      for (int f = 0; f < NF; ++f) mpre[f][t] = mul[f][ro + i0];
    }
  }
  __syncthreads();   // xs may still be read by a previous use
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    R *X = xs + f * xw + 2;
    for (int l = threadIdx.x; l < nlon; l += blockDim.x) X[l] = fld[f][ro + l];
    if (threadIdx.x < 5) {   // wrapped cells -2, -1 and nlon .. nlon+2
      const int l = threadIdx.x < 2 ? (int)threadIdx.x - 2 : nlon + (int)threadIdx.x - 2;
      X[l] = fld[f][ro + (threadIdx.x < 2 ? l + nlon : l - nlon)];
    }
  }
  __syncthreads();
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    const R *X = xs + f * xw + 2;
    R *S = ss + f * sw + 1;
    for (int l = (int)threadIdx.x - 1; l <= nlon + 1; l += blockDim.x) S[l] = slope(lim, X[l - 1], X[l], X[l + 1]);
  }
  __syncthreads();
  const bool vl = g.flux_type == GMC_FLUX_VAN_LEER;
  const R hxr = (R)g.hx;
  // the flux through face i0 (between cells i0 and i0 + 1, 0-based) with
  // Courant number c and multipliers mo
  auto face = [&](int i0, R c, const R (&mo)[NF]) {
    R flux[NF];
    if (fabs(c) > hxr) {   // |cflx| beyond the reach the reference allows: error, no flux (NaN: no flux below)
      raise_err(g, ERR_CFLX);
#pragma unroll
      for (int f = 0; f < NF; ++f) flux[f] = 0;
    } else {
      // c > 0: upwind cell i - ci (1-based face i = i0 + 1), whole cells
      // i+1-ci .. i, parabola over [1 - cf, 1]; c < 0: upwind cell i + 1 - ci,
      // whole cells i+1 .. i-ci, parabola over [0, -cf] and the flux's sign
      // reversed (hflx_ppm_cell, ffsl_mod.F90:833-875).  Both directions run
      // the same instructions, so a warp whose faces differ in sign does not
      // diverge; |c| < 1 needs no whole cells and no modulo.
      const int ci = (int)c;
      const R cf = c - (R)ci;
      const bool pos = c > 0;
      const int i = i0 + 1;
      const int iu = ci == 0 ? (pos ? i0 : i0 + 1) : Wg(pos ? i - ci - 1 : i - ci);   // 0-based upwind cell, 0 .. nlon
      const R s1 = pos ? (R)1 - cf : (R)0, s2 = pos ? (R)1 : -cf;
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        const R *X = xs + f * xw + 2, *S = ss + f * sw + 1;
        R sum = 0;
        if (ci != 0) {
          const int l0 = pos ? i + 1 - ci : i + 1, l1 = pos ? i : i - ci;
          for (int l = l0; l <= l1; ++l) sum = sum + X[Wg(l - 1)];
        }
        R num;
        if (vl) {   // hflx_van_leer_cell (ffsl_mod.F90:585-594)
          const R su = S[iu];
          num = mo[f] * (pos ? cf * (X[iu] + su * (R)0.5 * ((R)1 - cf)) + sum
                             : cf * (X[iu] - su * (R)0.5 * ((R)1 + cf)) - sum);
        } else {
          // PPM coefficients of the upwind cell: ppm() on the slopes of cells iu-1, iu, iu+1
          const R b = X[iu - 1], cc = X[iu], d = X[iu + 1], sm = S[iu - 1], s0 = S[iu], sp = S[iu + 1];
          R fl, df, f6;
          ppm_cell(cc, s0, ppm_edge(b, cc, sm, s0), ppm_edge(cc, d, s0, sp), fl, df, f6);
          num = (pos ? mo[f] : -mo[f]) * ppm_tail(sum, fl, df, f6, s1, s2);
        }
        flux[f] = c != 0 ? fdiv(num, c) : (R)0;
      }
    }
    out(i0, ro + i0, flux);
  };
#pragma unroll
  for (int t = 0; t < kPre; ++t) {
    const int i0 = threadIdx.x + t * blockDim.x;
    if (i0 < nlon) {
      R mo[NF];
#pragma unroll
      for (int f = 0; f < NF; ++f) mo[f] = mpre[f][t];
      face(i0, cpre[t], mo);
    }
  }
  for (int i0 = threadIdx.x + kPre * blockDim.x; i0 < nlon; i0 += blockDim.x) {
    R mo[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) mo[f] = mul[f][ro + i0];
    face(i0, cflx[ro + i0], mo);
  }
}

// Row pointer and column shift of row jj of a full-latitude field as the
// reference's fill_halo leaves it beyond the poles.
template <class R>
__device__ __forceinline__ const R *halo_row(const DGrid &g, const R *f, int jj, int k, int &shift) {
  shift = 0;
  if (jj < 1) { jj = 2 - jj; shift = g.half; }
  else if (jj > g.nlat) { jj = 2 * g.nlat - jj; shift = g.half; }
  if (jj > g.nlat) jj = g.nlat;   // only rows the caller never reads
  if (jj < 1) jj = 1;
  return f + ix3(g.nlat, g.nlon, 1, jj, k);
}

// y flux through half row f (between full rows f and f+1) from the values
// y(f), y(f+1), limited slopes s(f), s(f+1) and PPM edge values e(f), e(f+1),
// e(f+2) (e(r) = ppm_edge(y(r-1), y(r), s(r-1), s(r)), shared by the faces on
// both sides of a row) (hflx_ppm_cell along y, ffsl_mod.F90:841-875).  c > 0
// takes upwind row f, c < 0 row f + 1; both run the same instructions
// (selects), so a warp with faces of both signs does not diverge.
template <class R>
__device__ __forceinline__ R yface(const DGrid &g, R c, R vv, R y0, R y1, R s0, R s1, R e0, R e1, R e2) {
  if (fabs(c) > (R)1) {   // a NaN Courant number falls through to a NaN flux
    raise_err(g, ERR_CFLY);
    return 0;
  }
  const bool pos = c > 0;
  if (g.flux_type == GMC_FLUX_VAN_LEER) {   // hflx_van_leer_cell (ffsl_mod.F90:603-610)
    const R yu = pos ? y0 : y1, su = pos ? s0 : s1;   // upwind cell f (c > 0) or f + 1
    return vv * (yu + su * (R)0.5 * (fsign((R)1, c) - c));
  }
  const R yc = pos ? y0 : y1, sc = pos ? s0 : s1;
  const R el = pos ? e0 : e1, er = pos ? e1 : e2;
  R fl, df, f6;
  ppm_cell(yc, sc, el, er, fl, df, f6);
  const R num = (pos ? vv : -vv) * ppm_tail((R)0, fl, df, f6, pos ? (R)1 - c : (R)0, pos ? (R)1 : -c);
  return c != 0 ? fdiv(num, c) : (R)0;
}

// One column (0-based longitude i, level k) of a full-latitude field marching
// north one half row at a time, for the y passes.  At face f it holds the
// rows y(f-1 .. f+3), the limited slopes s(f-1 .. f+2) and the edge values
// e(f .. f+2); each advance reads one new row and forms one slope and one
// edge, so every row's slope and edges are formed once.  Rows beyond the
// poles are read as the reference's fill_halo leaves them.
template <class R>
struct YMarch {
  const DGrid &g;
  const R *fld;
  int k, i, f;
  R y0, y1, y2, y3, y4;   // y(f-1) .. y(f+3)
  R s0, s1, s2, s3;       // s(f-1) .. s(f+2)
  R e0, e1, e2;           // e(f) .. e(f+2)
  R p0, p1;               // rows f+4, f+5, requested ahead of their use (rows
                          // past the field's end read valid halo rows, unused)
  __device__ __forceinline__ R row(int jj) const {
    int sh;
    const R *p = halo_row(g, fld, jj, k, sh);
    const int l = i + sh;
    return p[l >= g.nlon ? l - g.nlon : l];
  }
  __device__ __forceinline__ YMarch(const DGrid &g_, const R *fld_, int k_, int i_, int f0)
      : g(g_), fld(fld_), k(k_), i(i_), f(f0) {
    const int lim = g.limiter;
    const R ym = row(f0 - 2);
    y0 = row(f0 - 1); y1 = row(f0); y2 = row(f0 + 1); y3 = row(f0 + 2); y4 = row(f0 + 3);
    p0 = row(f0 + 4);
    p1 = row(f0 + 5);
    s0 = slope(lim, ym, y0, y1);
    s1 = slope(lim, y0, y1, y2);
    s2 = slope(lim, y1, y2, y3);
    s3 = slope(lim, y2, y3, y4);
    e0 = ppm_edge(y0, y1, s0, s1);
    e1 = ppm_edge(y1, y2, s1, s2);
    e2 = ppm_edge(y2, y3, s2, s3);
  }
  __device__ __forceinline__ R flux(R c, R vv) const { return yface(g, c, vv, y1, y2, s1, s2, e0, e1, e2); }
  // f -> f + 1
  __device__ __forceinline__ void advance() {
    const R y5 = p0;
    p0 = p1;
    p1 = row(f + 6);
    const R s4 = slope(g.limiter, y3, y4, y5);   // s(f+3)
    const R e3 = ppm_edge(y3, y4, s3, s4);        // e(f+3)
    y0 = y1; y1 = y2; y2 = y3; y3 = y4; y4 = y5;
    s0 = s1; s1 = s2; s2 = s3; s3 = s4;
    e0 = e1; e1 = e2; e2 = e3;
    ++f;
  }
};

// Rows (or half rows) per band of the y passes: each thread marches one
// column through a band.
constexpr int kYBand = 24;
constexpr int kYThreads = 128;

// Outer pass: fluxes fy of qx along y with the meridional mass flux, one
// column per thread marching north through a band of half rows.
template <class R, bool MB>
__global__ void __launch_bounds__(kYThreads) k_hflx_y(DGrid g, const R *__restrict__ v, const R *__restrict__ cfly,
                                                      const R *__restrict__ my, R *__restrict__ fy) {
  if constexpr (MB) {   // grid z = member x level
    const size_t mo = (size_t)(blockIdx.z / g.nlev) * g.mstride;
    v = mshift(v, mo); cfly = mshift(cfly, mo); my = mshift(my, mo); fy = mshift(fy, mo);
  }
  const int k = blockIdx.z % g.nlev + 1;
  const int nhalf = g.nhalf, nlon = g.nlon;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int fb = blockIdx.y * kYBand + 1, fe = min(nhalf, fb + kYBand - 1);
  if (i >= nlon || fb > nhalf) return;
  YMarch<R> ym(g, my, k, i, fb);
  unsigned o = (unsigned)ix3(nhalf, nlon, i + 1, fb, k);
  R c = cfly[o], vv = v[o];
  for (int f = fb;; ++f, o += nlon) {
    R cn = 0, vn = 0;
    if (f < fe) {   // the next face's inputs, requested before this face's arithmetic
      cn = cfly[o + nlon];
      vn = v[o + nlon];
    }
    fy[o] = ym.flux(c, vv);
    if (f == fe) break;
    ym.advance();
    c = cn;
    vv = vn;
  }
}

// Inner pass fused with the advective-form update (ffsl_mod.F90:353-406):
// the advective fluxes of q stay on chip and the kernels write
//   qx = q - dt/2 (dflux_x/dx - divx q),  qy = q - dt/2 (dflux_y/dy - divy q)
// (pole rows: qx = q, qy from the ring mean of the polar half row's flux).
// x: one full row per block, together with the outer x pass (fluxes fx of qy
// with the zonal mass flux), which shares the Courant numbers; qy comes from
// the y inner pass launched before.
template <class R, bool MB>
__global__ void GMC_BOUNDS(R, 6) k_ffsl_x2(DGrid g, const R *__restrict__ u, const R *__restrict__ mfx,
                                           const R *__restrict__ cflx, const R *__restrict__ q,
                                           const R *__restrict__ qy, const R *__restrict__ divx, R *__restrict__ qx,
                                           R *__restrict__ fx, R dt) {
  if constexpr (MB) { const size_t mo = member_offset(g); u = mshift(u, mo); mfx = mshift(mfx, mo); cflx = mshift(cflx, mo); q = mshift(q, mo); qy = mshift(qy, mo); divx = mshift(divx, mo); qx = mshift(qx, mo); fx = mshift(fx, mo); }
  extern __shared__ double sh_raw[];
  const int k = blockIdx.y + 1, j = blockIdx.x + 1;
  const int nlat = g.nlat, nlon = g.nlon;
  const R hdt = (R)dt;
  if (j == 1 || j == nlat) {   // no x flux on the pole rows (fx left as it is)
    for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) {
      const size_t o = ix3(nlat, nlon, i, j, k);
      qx[o] = q[o];
    }
    return;
  }
  R *xs = reinterpret_cast<R *>(sh_raw);   // [2][nlon + 5]: q, qy with wrapped ends
  R *ss = xs + 2 * (nlon + 5);             // [2][nlon + 3]: their limited slopes
  R *fr = ss + 2 * (nlon + 3) + 1;         // inner fluxes of q, fr[-1 .. nlon-1]
  const R *mul[2] = {u, mfx};
  const R *fld[2] = {q, qy};
  const unsigned ro = (unsigned)ix3(nlat, nlon, 1, j, k);
  // divx of this thread's first cells, requested now: it is read only after
  // the fluxes, behind two barriers
  constexpr int kPreD = 3;
  R dpre[kPreD];
#pragma unroll
  for (int t = 0; t < kPreD; ++t) {
    const int i0 = threadIdx.x + t * blockDim.x;
    dpre[t] = i0 < nlon ? divx[ro + i0] : (R)0;
  }
  hflx_xrows<2, R>(g, j, k, mul, cflx, fld, xs, ss, [&](int i0, unsigned o, const R (&f)[2]) {
    fr[i0] = f[0];
    if (i0 == nlon - 1) fr[-1] = f[0];
    fx[o] = f[1];
  });
  __syncthreads();
  const R lel = ROWR(R, le_lon, j), ac = ROWR(R, area_cell, j);
  const R *X = xs + 2;
  auto update = [&](int i0, R dv) {
    const R qv = X[i0];
    qx[ro + i0] = qv - (R)0.5 * (fdiv((fr[i0] - fr[i0 - 1]) * lel, ac) - dv * qv) * hdt;
  };
#pragma unroll
  for (int t = 0; t < kPreD; ++t) {
    const int i0 = threadIdx.x + t * blockDim.x;
    if (i0 < nlon) update(i0, dpre[t]);
  }
  for (int i0 = threadIdx.x + kPreD * blockDim.x; i0 < nlon; i0 += blockDim.x) update(i0, divx[ro + i0]);
}

// y: one column per thread marching north through a band of full rows
// 2 .. nlat-1 (the faces from the band's first south face on).  The pole rows
// get no qy: the outer x pass, its only reader, skips them (hflx on full
// latitudes without the poles, ffsl_mod.F90:787-829).
template <class R, bool MB>
__global__ void __launch_bounds__(kYThreads) k_ffsl_inner_y(DGrid g, const R *__restrict__ v, const R *__restrict__ cfly,
                                                            const R *__restrict__ q, const R *__restrict__ divy,
                                                            R *__restrict__ qy, R dt) {
  if constexpr (MB) {   // grid z = member x level
    const size_t mo = (size_t)(blockIdx.z / g.nlev) * g.mstride;
    v = mshift(v, mo); cfly = mshift(cfly, mo); q = mshift(q, mo); divy = mshift(divy, mo); qy = mshift(qy, mo);
  }
  const int k = blockIdx.z % g.nlev + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int jb = blockIdx.y * kYBand + 2, je = min(nlat - 1, jb + kYBand - 1);
  if (i >= nlon || jb > nlat - 1) return;
  const R hdt = dt;
  YMarch<R> ym(g, q, k, i, jb - 1);
  unsigned of = (unsigned)ix3(nhalf, nlon, i + 1, jb - 1, k);   // face jb-1
  unsigned oc = (unsigned)ix3(nlat, nlon, i + 1, jb, k);        // cell (i, jb)
  R prev = ym.flux(cfly[of], v[of]);
  R la1 = ROWR(R, le_lat, jb - 1);
  of += nlon;
  R c = cfly[of], vv = v[of], dy = divy[oc];
  for (int j = jb; j <= je; ++j, oc += nlon, of += nlon) {
    R cn = 0, vn = 0, dn = 0;
    if (j < je) {   // the next row's inputs, requested before this row's arithmetic
      cn = cfly[of + nlon];
      vn = v[of + nlon];
      dn = divy[oc + nlon];
    }
    ym.advance();
    const R cur = ym.flux(c, vv);
    const R la0 = ROWR(R, le_lat, j), ac = ROWR(R, area_cell, j);
    const R qv = ym.y1;   // y(j)
    qy[oc] = qv - (R)0.5 * ((cur * la0 - prev * la1) / ac - dy * qv) * hdt;
    prev = cur;
    la1 = la0;
    c = cn;
    vv = vn;
    dy = dn;
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
    raise_err(g, ERR_CFLZ);
    return 0;
  }
  const int ci = (int)c;
  const R cf = c - (R)ci;
  auto coef = [&](int ku, R &fl, R &df, R &f6) {
    if (ku < 1 || ku > nlev) { fl = df = f6 = 0; return; }
    ppm(lim, C(ku - 2), C(ku - 1), C(ku), C(ku + 1), C(ku + 2), fl, df, f6);
  };
  if (g.flux_type == GMC_FLUX_VAN_LEER) {   // vflx_van_leer_cell (ffsl_mod.F90:637-653)
    if (c > 0) {
      const int ku = k - ci - 1;
      R sum = 0;
      for (int l = k - ci; l <= k - 1; ++l) sum = sum + C(l);
      const R dm = slope(lim, C(ku - 1), C(ku), C(ku + 1));
      return fdiv(w * (cf * (C(ku) + dm * (R)0.5 * ((R)1 - cf)) + sum), c);
    }
    if (c < 0) {
      const int ku = k - ci;
      R sum = 0;
      for (int l = k; l <= k - ci - 1; ++l) sum = sum + C(l);
      const R dm = slope(lim, C(ku - 1), C(ku), C(ku + 1));
      return fdiv(w * (cf * (C(ku) - dm * (R)0.5 * ((R)1 + cf)) - sum), c);
    }
    return 0;
  }
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

// vflx_at in cell-centric form for the interfaces k = 2, 3, ... of a column
// in order.  The window holds C(k-2..k+2), the slopes s(k-2..k+1) and the
// edge values e(k-1..k+1) (e(l) between levels l-1 and l), so each step forms
// one slope and one edge.  For |c| < 1 the upwind cell is k-1 or k, always
// inside 1..nlev; larger Courant numbers take the general vflx_at.  The
// result equals vflx_at bit for bit.
template <class R>
struct VRoll {
  const DGrid &g;
  const R *col;   // col[l + 1] = C(l), l = -1 .. nlev+2
  int k;
  R c0, c1, c2, c3, c4;   // C(k-2) .. C(k+2)
  R s0, s1, s2, s3;       // s(k-2) .. s(k+1)
  R e0, e1, e2;           // e(k-1) .. e(k+1)
  __device__ VRoll(const DGrid &g_, const R *col_) : g(g_), col(col_), k(2) {
    const int lim = g.limiter;
    c0 = col[1]; c1 = col[2]; c2 = col[3]; c3 = col[4]; c4 = col[5];
    s0 = slope(lim, col[0], c0, c1);
    s1 = slope(lim, c0, c1, c2);
    s2 = slope(lim, c1, c2, c3);
    s3 = slope(lim, c2, c3, c4);
    e0 = ppm_edge(c0, c1, s0, s1);
    e1 = ppm_edge(c1, c2, s1, s2);
    e2 = ppm_edge(c2, c3, s2, s3);
  }
  // flux at the current interface k
  __device__ __forceinline__ R flux(R c, R w) const {
    if (!(fabs(c) < (R)1)) return vflx_at<R>(g, col, k, c, w);
    if (g.flux_type == GMC_FLUX_VAN_LEER) {   // upwind cell k-1 (c > 0) or k, slope s(k-1) or s(k)
      if (c > 0) return fdiv(w * (c * (c1 + s1 * (R)0.5 * ((R)1 - c))), c);
      if (c < 0) return fdiv(w * (c * (c2 - s2 * (R)0.5 * ((R)1 + c))), c);
      return 0;
    }
    R fl, df, f6;
    if (c > 0) {
      ppm_cell(c1, s1, e0, e1, fl, df, f6);
      return fdiv(w * ppm_tail((R)0, fl, df, f6, (R)1 - c, (R)1), c);
    }
    if (c < 0) {
      ppm_cell(c2, s2, e1, e2, fl, df, f6);
      return fdiv(-w * ppm_tail((R)0, fl, df, f6, (R)0, -c), c);
    }
    return 0;
  }
  // k -> k + 1 (requires k + 1 <= nlev)
  __device__ __forceinline__ void advance() {
    const R c5 = col[k + 4];   // C(k+3)
    const R s4 = slope(g.limiter, c3, c4, c5);
    const R e3 = ppm_edge(c3, c4, s3, s4);
    c0 = c1; c1 = c2; c2 = c3; c3 = c4; c4 = c5;
    s0 = s1; s1 = s2; s2 = s3; s3 = s4;
    e0 = e1; e1 = e2; e2 = e3;
    ++k;
  }
};

// calc_grad_ptf tail (operators_mod.F90:1034-1098) with the tendency
// assembly dpt = -(dptf/dlon + dptf/dlat + dptf/dlev) (gmcore_mod.F90:491-495).
template <class R, bool MB>
__global__ void k_pt_tendency(DGrid g, Slot<R> s, Work<R> w) {
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
  const R lel = ROWR(R, le_lon, j), ac = ROWR(R, area_cell, j), la0 = ROWR(R, le_lat, j), la1 = ROWR(R, le_lat, j - 1);
  const int im = wrap(i - 1, nlon);
  R f_top = 0;   // ptf_lev(1) = 0
  VRoll<R> vr(g, col);
  for (int k = 1; k <= nlev; ++k) {
    const size_t o = ix3(nlat, nlon, i, j, k);
    R f_bot = 0;
    if (k + 1 <= nlev) {
      const size_t ol = ix3(nlat, nlon, i, j, k + 1);
      if (k + 1 > 2) vr.advance();
      f_bot = vr.flux(w.cflz[ol], s.we_lev[ol]);
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


// General vertical flux at interface k from a column in shared memory (any
// Courant number): C(l) at C[(l + 1) * ld] for l = -1 .. nlev+2, limited cell
// coefficients of cell l at FL/DF/F6[(l - 1) * ld] for l = 1 .. nlev.
// Follows vflx_at term by term.
template <class R>
__device__ R vflx_tile(const DGrid &g, const R *C, const R *FL, const R *DF, const R *F6, int ld, int k, R c, R w) {
  const int nlev = g.nlev;
  if (!(fabs(c) <= (R)nlev)) {
    raise_err(g, ERR_CFLZ);
    return 0;
  }
  auto Cv = [&](int kk) { return C[(min(max(kk, -1), nlev + 2) + 1) * ld]; };
  const int ci = (int)c;
  const R cf = c - (R)ci;
  if (g.flux_type == GMC_FLUX_VAN_LEER) {   // vflx_van_leer_cell (ffsl_mod.F90:637-653)
    const int lim = g.limiter;
    if (c > 0) {
      const int ku = k - ci - 1;
      R sum = 0;
      for (int l = k - ci; l <= k - 1; ++l) sum = sum + Cv(l);
      const R dm = slope(lim, Cv(ku - 1), Cv(ku), Cv(ku + 1));
      return fdiv(w * (cf * (Cv(ku) + dm * (R)0.5 * ((R)1 - cf)) + sum), c);
    }
    if (c < 0) {
      const int ku = k - ci;
      R sum = 0;
      for (int l = k; l <= k - ci - 1; ++l) sum = sum + Cv(l);
      const R dm = slope(lim, Cv(ku - 1), Cv(ku), Cv(ku + 1));
      return fdiv(w * (cf * (Cv(ku) - dm * (R)0.5 * ((R)1 + cf)) - sum), c);
    }
    return 0;
  }
  auto coef = [&](int ku, R &fl, R &df, R &f6) {
    if (ku < 1 || ku > nlev) { fl = df = f6 = 0; return; }
    fl = FL[(ku - 1) * ld]; df = DF[(ku - 1) * ld]; f6 = F6[(ku - 1) * ld];
  };
  R fl, df, f6;
  if (c > 0) {
    R sum = 0;
    for (int l = k - ci; l <= k - 1; ++l) sum = sum + Cv(l);
    coef(k - ci - 1, fl, df, f6);
    return fdiv(w * ppm_tail(sum, fl, df, f6, (R)1 - cf, (R)1), c);
  }
  if (c < 0) {
    R sum = 0;
    for (int l = k; l <= k - ci - 1; ++l) sum = sum + Cv(l);
    coef(k - ci, fl, df, f6);
    return fdiv(-w * ppm_tail(sum, fl, df, f6, (R)0, -cf), c);
  }
  return 0;
}

// Interfaces per thread whose vertical inputs the column-tile kernels request
// at their start (levels are spread over kTileK thread rows: 5 covers 39 levels).
constexpr int kColPre = 5;

// FP32 form of k_pt_tendency over column tiles: the pt column with its
// extrapolated ghost levels, slopes, limited cell coefficients and interface
// fluxes are built in shared memory phase by phase, each phase parallel over
// (column, level).
template <bool MB>
__global__ void GMC_BOUNDS_F(8) k_pt_tendency_f(DGrid g, Slot<float> s, Work<float> w) {
  if constexpr (MB) { to_member(g, s); to_member(g, w); }   // member-batched launches
  extern __shared__ double shd[];
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon, nlev = g.nlev, lim = g.limiter;
  const int j = blockIdx.y + 1;
  const int ti = threadIdx.x, kt = threadIdx.y, KT = blockDim.y;
  const int i = blockIdx.x * kTileI + ti + 1;
  const int ld = kTileI + 1;
  const bool pole = j == 1 || j == nlat, valid = i <= nlon;
  const int ic = valid ? i : nlon;
  float *ring = reinterpret_cast<float *>(shd);           // [nlev] (FP64 sums rounded once)
  float *C = reinterpret_cast<float *>(shd + nlev) + ti;  // C(l) at [(l+1)*ld], l = -1 .. nlev+2
  float *S = C + (nlev + 4) * ld;                         // s(l) at [l*ld],     l = 0 .. nlev+1
  float *FL = S + (nlev + 2) * ld;                        // cell l at [(l-1)*ld]
  float *DF = FL + nlev * ld;
  float *F6 = DF + nlev * ld;
  float *FZ = F6 + nlev * ld;                             // interface flux k at [(k-1)*ld], k = 1 .. nlev+1
  if (pole) tile_pole_ring(g, j, ring, [&](int ii, int jv, int k) { return w.ptf_lat[ix3(nhalf, nlon, ii, jv, k)]; });
  for (int k = 1 + kt; k <= nlev; k += KT) C[(k + 1) * ld] = s.pt[ix3(nlat, nlon, ic, j, k)];
  // the Courant numbers and mass fluxes of this thread's interfaces, requested
  // with the column so that their latency overlaps the reconstruction below
  float cz[kColPre], wz[kColPre];
#pragma unroll
  for (int m = 0; m < kColPre; ++m) {
    const int k = 1 + kt + m * KT;
    cz[m] = wz[m] = 0;
    if (k >= 2 && k <= nlev) {
      const size_t ol = ix3(nlat, nlon, ic, j, k);
      cz[m] = w.cflz[ol];
      wz[m] = s.we_lev[ol];
    }
  }
  __syncthreads();
  if (kt == 0) {   // ghost levels by linear extrapolation
    C[1 * ld] = 2.0f * C[2 * ld] - C[3 * ld];                         // C(0)
    C[0] = 2.0f * C[1 * ld] - C[2 * ld];                              // C(-1)
    C[(nlev + 2) * ld] = 2.0f * C[(nlev + 1) * ld] - C[nlev * ld];    // C(nlev+1)
    C[(nlev + 3) * ld] = 2.0f * C[(nlev + 2) * ld] - C[(nlev + 1) * ld];   // C(nlev+2)
  }
  __syncthreads();
  for (int l = kt; l <= nlev + 1; l += KT) S[l * ld] = slope(lim, C[l * ld], C[(l + 1) * ld], C[(l + 2) * ld]);
  __syncthreads();
  for (int l = 1 + kt; l <= nlev; l += KT) {
    const float f = C[(l + 1) * ld], s0 = S[l * ld];
    float fl, df, f6;
    ppm_cell(f, s0, ppm_edge(C[l * ld], f, S[(l - 1) * ld], s0), ppm_edge(f, C[(l + 2) * ld], s0, S[(l + 1) * ld]), fl,
             df, f6);
    FL[(l - 1) * ld] = fl;
    DF[(l - 1) * ld] = df;
    F6[(l - 1) * ld] = f6;
  }
  __syncthreads();
  // vertical flux at interface k (2 .. nlev) with Courant number c and mass flux wv
  auto flux_at = [&](int k, float c, float wv) {
    float fz = 0;
    if (fabsf(c) < 1.0f && g.flux_type == GMC_FLUX_VAN_LEER) {   // upwind cell k-1 or k
      if (c > 0) fz = fdiv(wv * (c * (C[k * ld] + S[(k - 1) * ld] * 0.5f * (1.0f - c))), c);
      else if (c < 0) fz = fdiv(wv * (c * (C[(k + 1) * ld] - S[k * ld] * 0.5f * (1.0f + c))), c);
    } else if (fabsf(c) < 1.0f) {
      if (c > 0) {
        const int u = k - 2;   // cell k-1
        fz = fdiv(wv * ppm_tail(0.0f, FL[u * ld], DF[u * ld], F6[u * ld], 1.0f - c, 1.0f), c);
      } else if (c < 0) {
        const int u = k - 1;   // cell k
        fz = fdiv(-wv * ppm_tail(0.0f, FL[u * ld], DF[u * ld], F6[u * ld], 0.0f, -c), c);
      }
    } else if (valid) {
      fz = vflx_tile<float>(g, C, FL, DF, F6, ld, k, c, wv);
    }
    return fz;
  };
#pragma unroll
  for (int m = 0; m < kColPre; ++m) {
    const int k = 1 + kt + m * KT;
    if (k <= nlev + 1) FZ[(k - 1) * ld] = k != 1 && k != nlev + 1 ? flux_at(k, cz[m], wz[m]) : 0.0f;
  }
  for (int k = 1 + kt + kColPre * KT; k <= nlev + 1; k += KT) {
    float fz = 0;
    if (k != nlev + 1) {
      const size_t ol = ix3(nlat, nlon, ic, j, k);
      fz = flux_at(k, w.cflz[ol], s.we_lev[ol]);
    }
    FZ[(k - 1) * ld] = fz;
  }
  __syncthreads();
  if (!valid) return;
  const float ac = ROWR(float, area_cell, j);
  const float clon = ROWR(float, le_lon, j), la0 = ROWR(float, le_lat, j), la1 = ROWR(float, le_lat, j - 1);
  const int im = wrap(i - 1, nlon);
  for (int k = 1 + kt; k <= nlev; k += KT) {
    const size_t o = ix3(nlat, nlon, i, j, k);
    float dlon, dlat;
    if (pole) {
      dlon = 0;
      dlat = ring[k - 1];
    } else {
      dlon = (w.ptf_lon[o] - w.ptf_lon[ix3(nlat, nlon, im, j, k)]) * clon / ac;
      dlat = (w.ptf_lat[ix3(nhalf, nlon, i, j, k)] * la0 - w.ptf_lat[ix3(nhalf, nlon, i, j - 1, k)] * la1) / ac;
    }
    w.dpt[o] = -dlon - dlat - (FZ[k * ld] - FZ[(k - 1) * ld]);
  }
}

// ---------------------------------------------------------------------------
// Tracer batch (adv_run, adv_mod.F90:152-312)
// ---------------------------------------------------------------------------

// adv_batch_accum_*: copy (mode 0), add (1) or average (2) a field.
template <class T>
__global__ void k_accum(T *dst, const T *src, size_t n, int mode, double divisor) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    T s = src ? src[t] : (T)0;
    if (mode == 0) dst[t] = s;
    else if (mode == 1) dst[t] = dst[t] + s;
    else dst[t] = (T)((dst[t] + s) / (T)divisor);
  }
}

// Several accumulations in one launch (blockIdx.y = entry): the batch's
// winds, mass fluxes and vertical mass flux after a step.  Same arithmetic per
// element as k_accum; four elements per thread where the entry's length and
// addresses allow 16-byte vectors.
template <class T>
__global__ void k_accum_multi(AccumSet<T> set) {
  const AccumEntry<T> &e = set.e[blockIdx.y];
  const T dv = (T)e.divisor;
  auto one = [&](T d, T s) {
    if (e.mode == 0) return s;
    if (e.mode == 1) return d + s;
    return (T)((d + s) / dv);
  };
  const size_t stride = (size_t)gridDim.x * blockDim.x, t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if constexpr (std::is_same<T, float>::value) {
    if (e.n % 4 == 0 && ((uintptr_t)e.dst % 16) == 0 && (!e.src || ((uintptr_t)e.src % 16) == 0)) {
      float4 *d4 = reinterpret_cast<float4 *>(e.dst);
      const float4 *s4 = reinterpret_cast<const float4 *>(e.src);
      for (size_t t = t0; t < e.n / 4; t += stride) {
        const float4 s = s4 ? s4[t] : make_float4(0, 0, 0, 0);
        float4 d = e.mode == 0 ? s : d4[t];
        if (e.mode != 0) {
          d.x = one(d.x, s.x); d.y = one(d.y, s.y); d.z = one(d.z, s.z); d.w = one(d.w, s.w);
        }
        d4[t] = d;
      }
      return;
    }
  }
  for (size_t t = t0; t < e.n; t += stride) {
    const T s = e.src ? e.src[t] : (T)0;
    e.dst[t] = e.mode == 0 ? s : one(e.dst[t], s);
  }
}

// Half-level mass m_lev of calc_m (operators_mod.F90:505-525) folded into
// the batch accumulator; sp.phs_f null zeroes the sample.  The FP32 form
// takes (m(k-1) + m(k)) / 2 of the FP32 layer masses.
template <class R>
__global__ void k_half_level_mass(DGrid g, SurfP<R> sp, R *m_lev, int mode, double divisor) {
  const int j = blockIdx.y + 1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int nlat = g.nlat, nlon = g.nlon, nlev = g.nlev;
  if (i > nlon) return;
  R ml[66];
  const size_t c2 = (size_t)(j - 1) * nlon + (i - 1);
  if (!sp.phs_f) {
    for (int k = 0; k <= nlev; ++k) ml[k] = 0;
  } else if constexpr (std::is_same<R, float>::value) {
    const float psr = sp.at(c2);
    float mprev = 0;
    for (int k = 1; k <= nlev; ++k) {
      float m = Mass<float>::layer(g, k, psr);
      ml[k - 1] = 0.5f * (mprev + m);
      mprev = m;
    }
    ml[nlev] = 0.5f * mprev;
  } else {
    const double phs = sp.phs_f[c2];
    double plo = ph_lev(g, 1, phs), ph_prev = 0;
    for (int k = 1; k <= nlev; ++k) {
      double phi = ph_lev(g, k + 1, phs);
      double ph = 0.5 * (plo + phi);
      ml[k - 1] = k == 1 ? ph - plo : ph - ph_prev;
      ph_prev = ph;
      plo = phi;
    }
    ml[nlev] = plo - ph_prev;
  }
  const R dv = (R)divisor;
  for (int k = 1; k <= nlev + 1; ++k) {
    size_t o = ix3(nlat, nlon, i, j, k);
    if (mode == 0) m_lev[o] = ml[k - 1];
    else if (mode == 1) m_lev[o] = m_lev[o] + ml[k - 1];
    else m_lev[o] = (m_lev[o] + ml[k - 1]) / dv;
  }
}

// FP32 form of k_half_level_mass, elementwise over (half level, cell): half
// level k (1 .. nlev+1) takes (m(k-1) + m(k)) / 2 of the FP32 layer masses with
// m(0) = m(nlev+1) = 0, the same values as the column loop.
__global__ void __launch_bounds__(256) k_half_level_mass_f(DGrid g, const float *__restrict__ psr,
                                                           float *__restrict__ m_lev, int mode, float divisor) {
  const int H = g.nlat * g.nlon, k = blockIdx.y + 1;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= H) return;
  float ml = 0;
  if (psr) {
    const float ps = psr[c];
    const float mu = k > 1 ? fmaf(g.dmB[k - 2], ps, g.dmA[k - 2]) : 0.0f;          // layer k-1
    const float md = k <= g.nlev ? fmaf(g.dmB[k - 1], ps, g.dmA[k - 1]) : 0.0f;   // layer k
    ml = 0.5f * (mu + md);
  }
  float *o = m_lev + (size_t)(k - 1) * H + c;
  if (mode == 0) *o = ml;
  else if (mode == 1) *o = *o + ml;
  else *o = (*o + ml) / divisor;
}

template <class R>
__global__ void k_batch_cflz(DGrid g, const R *we_in, const R *ml_in, R *cflz, R dt) {
  extern __shared__ float colsh[];
  const int j = blockIdx.y + 1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int nlat = g.nlat, nlon = g.nlon, nlev = g.nlev;
  if (i > nlon) return;
  if constexpr (std::is_same<R, float>::value) {
    float *col = colsh + threadIdx.x;
    const int st = blockDim.x;
    for (int k = 1; k <= nlev + 1; ++k) {
      size_t o = ix3(nlat, nlon, i, j, k);
      col[(k - 1) * st] = fdiv(we_in[o], ml_in[o]) * g.half_dlev_f[k - 1];
    }
    bool bad = false;
    const float dtf = (float)dt;
    for (int k = 2; k <= nlev; ++k) {
      float c = cflz_of_f(g.half_lev_f, g.full_dlev_f, g.full_dlev_rf, nlev, col, st, k, dtf, bad);
      if (c == c) cflz[ix3(nlat, nlon, i, j, k)] = c;
    }
    if (bad) raise_err(g, ERR_CFLZ);
    return;
  }
  R we[66], ml[66];
  for (int k = 1; k <= nlev + 1; ++k) {
    size_t o = ix3(nlat, nlon, i, j, k);
    we[k - 1] = we_in[o];
    ml[k - 1] = ml_in[o];
  }
  bool bad = false;
  for (int k = 2; k <= nlev; ++k) {
    R c = cflz_of<R>(g, we, ml, k, (R)dt, bad);
    if (c == c) cflz[ix3(nlat, nlon, i, j, k)] = c;
  }
  if (bad) raise_err(g, ERR_CFLZ);
}

// q_new = (old_m q_old - dt div(qmf)) / m, then the zonal negative fixer,
// which walks the row in order and borrows from the neighbours; at the ends
// it reads the longitude halo of q_new as the reference leaves it (the row's
// values before this update, wrapped).
template <class R>
__global__ void GMC_BOUNDS(R, 8) k_tracer_horizontal(DGrid g, const R *q_old, R *q_new, const R *fx, const R *fy, SurfP<R> old_sp,
                                    SurfP<R> sp, double dt_adv) {
  extern __shared__ double sh[];
  double *red = sh;
  R *row = reinterpret_cast<R *>(sh + 32);
  R *mrow = row + g.nlon + 2;
  const int j = blockIdx.x + 1, k = blockIdx.y + 1;
  const int nlat = g.nlat, nhalf = g.nhalf, nlon = g.nlon;
  if (threadIdx.x == 0) {
    row[0] = q_new[ix3(nlat, nlon, nlon, j, k)];
    row[nlon + 1] = q_new[ix3(nlat, nlon, 1, j, k)];
  }
  __syncthreads();
  double pole = 0;
  const bool is_pole = j == 1 || j == nlat;
  if (is_pole) {
    const int jv = j == 1 ? 1 : nhalf;
    double p = ring_sum(nlon, red, [&](int i) { return (double)fy[ix3(nhalf, nlon, i, jv, k)]; });
    pole = p * ROW(g.le_lat, jv) / nlon / ROW(g.area_cell, j) * dt_adv;
  }
  const R lel = ROWR(R, le_lon, j), ac = ROWR(R, area_cell, j), la0 = ROWR(R, le_lat, j), la1 = ROWR(R, le_lat, j - 1);
  const R dta = (R)dt_adv;
  bool neg = false;
  if constexpr (std::is_same<R, float>::value) {
    if (!is_pole) {
      // Two points per thread (0-based i0, i0+1): paired loads of q_old, the
      // fluxes and the surface pressures, the west flux column as one scalar;
      // the per-point arithmetic is the loop's below.
      const unsigned fo = (unsigned)ix3(nlat, nlon, 1, j, k), hn = (unsigned)ix3(nhalf, nlon, 1, j, k), hs = hn - nlon;
      const unsigned po = (unsigned)(j - 1) * nlon;
      const float dA = g.dmA[k - 1], dB = g.dmB[k - 1];
      for (int i0 = 2 * threadIdx.x; i0 < nlon; i0 += 2 * blockDim.x) {
        auto P2 = [&](const float *p, unsigned o) { return *reinterpret_cast<const float2 *>(p + o + i0); };
        const float2 qo = P2(q_old, fo), fx2 = P2(fx, fo), fyn = P2(fy, hn), fys = P2(fy, hs);
        const float2 pso = P2(old_sp.psr, po), psn = P2(sp.psr, po);
        const float fxw = fx[fo + (i0 == 0 ? nlon - 1 : i0 - 1)];
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          const float om = fmaf(dB, p ? pso.y : pso.x, dA), m = fmaf(dB, p ? psn.y : psn.x, dA);
          const float a = ((p ? fx2.y : fx2.x) - (p ? fx2.x : fxw)) * lel;
          const float b = (p ? fyn.y : fyn.x) * la0 - (p ? fys.y : fys.x) * la1;
          float qn = om * (p ? qo.y : qo.x) - (a + b) / ac * dta;
          qn = qn / m;
          row[i0 + 1 + p] = qn;
          mrow[i0 + 1 + p] = m;
          neg |= qn < 0;
        }
      }
    }
  }
  for (int i = 1 + threadIdx.x; i <= nlon && !(std::is_same<R, float>::value && !is_pole); i += blockDim.x) {
    const size_t o = ix3(nlat, nlon, i, j, k);
    const size_t c2 = (size_t)(j - 1) * nlon + (i - 1);
    R om = Mass<R>::layer(g, k, old_sp.at(c2));
    R m = Mass<R>::layer(g, k, sp.at(c2));
    R qn;
    if (!is_pole) {
      R a = (fx[o] - fx[ix3(nlat, nlon, wrap(i - 1, nlon), j, k)]) * lel;
      R b = fy[ix3(nhalf, nlon, i, j, k)] * la0 - fy[ix3(nhalf, nlon, i, j - 1, k)] * la1;
      qn = om * q_old[o] - (a + b) / ac * dta;
    } else if (j == 1) {
      qn = om * q_old[o] - (R)pole;
    } else {
      qn = om * q_old[o] + (R)pole;
    }
    qn = qn / m;
    row[i] = qn;
    mrow[i] = m;
    neg |= qn < 0;
  }
  if (threadIdx.x == 0) {
    mrow[0] = Mass<R>::layer(g, k, sp.at((size_t)(j - 1) * nlon + (nlon - 1)));
    mrow[nlon + 1] = Mass<R>::layer(g, k, sp.at((size_t)(j - 1) * nlon));
  }
  // The fixer visits i = 1 .. nlon in order.  One warp walks the row 32
  // cells at a time: a ballot finds the negative cells, lane 0 fixes the
  // lowest one, and the cells after it are tested again (a fix changes its
  // right neighbour), which visits the negatives in the same order with the
  // same values as the sequential walk.
  if (__syncthreads_or(neg) && threadIdx.x < 32) {
    const int lane = threadIdx.x;
    for (int base = 1; base <= nlon; base += 32) {
      const int i = base + lane;
      unsigned mask = __ballot_sync(0xffffffffu, i <= nlon && row[i] < 0);
      while (mask) {
        const int p = base + __ffs(mask) - 1;
        if (lane == 0) {
          R qm0 = row[p] * mrow[p], qm1 = row[p - 1] * mrow[p - 1], qm2 = row[p + 1] * mrow[p + 1];
          R qm0_half = (R)0.5 * qm0;
          if (qm1 >= qm0_half && qm2 >= qm0_half) {
            row[p - 1] = (qm1 - qm0_half) / mrow[p - 1];
            row[p + 1] = (qm2 - qm0_half) / mrow[p + 1];
          } else if (qm1 > qm0) {
            row[p - 1] = (qm1 - qm0) / mrow[p - 1];
          } else if (qm2 > qm0) {
            row[p + 1] = (qm2 - qm0) / mrow[p + 1];
          } else {
            raise_err(g, ERR_NEGTRACER);
          }
          row[p] = 0;
        }
        __syncwarp();
        mask = __ballot_sync(0xffffffffu, i <= nlon && i > p && row[i] < 0);
      }
    }
  }
  __syncthreads();
  for (int i = 1 + threadIdx.x; i <= nlon; i += blockDim.x) q_new[ix3(nlat, nlon, i, j, k)] = row[i];
}

// Vertical FFSL of the tracer column with copied ghost levels, then the
// vertical negative fixer (adv_mod.F90:259-297).
template <class R>
__global__ void k_tracer_vertical(DGrid g, R *q, const R *cflz, const R *we, SurfP<R> sp, double dt_adv) {
  const int j = blockIdx.y + 1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int nlat = g.nlat, nlon = g.nlon, nlev = g.nlev;
  if (i > nlon) return;
  R col[70], mz[66], m[66];
  for (int k = 1; k <= nlev; ++k) col[k + 1] = q[ix3(nlat, nlon, i, j, k)];
  col[1] = col[0] = col[2];
  col[nlev + 2] = col[nlev + 3] = col[nlev + 1];
  const auto ps = sp.at((size_t)(j - 1) * nlon + (i - 1));
  for (int k = 1; k <= nlev; ++k) m[k - 1] = Mass<R>::layer(g, k, ps);
  mz[0] = 0;
  mz[nlev] = 0;
  VRoll<R> vr(g, col);
  for (int k = 2; k <= nlev; ++k) {
    size_t o = ix3(nlat, nlon, i, j, k);
    if (k > 2) vr.advance();
    mz[k - 1] = vr.flux(cflz[o], we[o]);
  }
  R *qc = col + 1;   // qc[k] = q(k)
  const R dta = (R)dt_adv;
  for (int k = 1; k <= nlev; ++k) qc[k] = qc[k] - ((mz[k] - mz[k - 1]) * dta) / m[k - 1];
  for (int k = 1; k <= nlev; ++k) {
    if (qc[k] < 0) {
      R qm0 = qc[k] * m[k - 1];
      R qm1 = k > 1 ? qc[k - 1] * m[k - 2] : (R)0;
      R qm2 = k < nlev ? qc[k + 1] * m[k] : (R)0;
      R qm0_half = (R)0.5 * qm0;
      if (qm1 >= qm0_half && qm2 >= qm0_half) {
        if (qm1 > 0) qc[k - 1] = (qm1 - qm0_half) / m[k - 2];
        if (qm2 > 0) qc[k + 1] = (qm2 - qm0_half) / m[k];
      } else if (qm1 > qm0) {
        if (qm1 > 0) qc[k - 1] = (qm1 - qm0) / m[k - 2];
      } else if (qm2 > qm0) {
        if (qm2 > 0) qc[k + 1] = (qm2 - qm0) / m[k];
      } else {
        raise_err(g, ERR_NEGTRACER);
      }
      qc[k] = 0;
    }
  }
  for (int k = 1; k <= nlev; ++k) q[ix3(nlat, nlon, i, j, k)] = qc[k];
}

// FP32 form of k_tracer_vertical over column tiles: the column with copied
// ghost levels, slopes, cell coefficients and interface fluxes in shared
// memory, the update parallel over (column, level); the vertical fixer walks
// a column in order and runs only in blocks that hold a negative value.
__global__ void GMC_BOUNDS_F(6) k_tracer_vertical_f(DGrid g, float *q, const float *cflz, const float *we, SurfP<float> sp,
                                    float dt_adv) {
  extern __shared__ float shf[];
  const int nlat = g.nlat, nlon = g.nlon, nlev = g.nlev, lim = g.limiter;
  const int j = blockIdx.y + 1;
  const int ti = threadIdx.x, kt = threadIdx.y, KT = blockDim.y;
  const int i = blockIdx.x * kTileI + ti + 1;
  const int ld = kTileI + 1;
  const bool valid = i <= nlon;
  const int ic = valid ? i : nlon;
  float *C = shf + ti;                  // C(l) at [(l+1)*ld], l = -1 .. nlev+2
  float *S = C + (nlev + 4) * ld;       // s(l) at [l*ld], l = 0 .. nlev+1
  float *FL = S + (nlev + 2) * ld;      // cell l at [(l-1)*ld]
  float *DF = FL + nlev * ld;
  float *F6 = DF + nlev * ld;
  float *FZ = F6 + nlev * ld;           // interface k at [(k-1)*ld], k = 1 .. nlev+1
  float *M = FZ + (nlev + 1) * ld;      // layer mass of level k at [(k-1)*ld]
  const float psr = sp.at((size_t)(j - 1) * nlon + (ic - 1));
  for (int k = 1 + kt; k <= nlev; k += KT) {
    C[(k + 1) * ld] = q[ix3(nlat, nlon, ic, j, k)];
    M[(k - 1) * ld] = Mass<float>::layer(g, k, psr);
  }
  // the Courant numbers and mass fluxes of this thread's interfaces, requested
  // with the column so that their latency overlaps the reconstruction below
  float cz[kColPre], wz[kColPre];
#pragma unroll
  for (int m = 0; m < kColPre; ++m) {
    const int k = 1 + kt + m * KT;
    cz[m] = wz[m] = 0;
    if (k >= 2 && k <= nlev) {
      const size_t ol = ix3(nlat, nlon, ic, j, k);
      cz[m] = cflz[ol];
      wz[m] = we[ol];
    }
  }
  __syncthreads();
  if (kt == 0) {   // ghost levels copy the end levels
    C[0] = C[1 * ld] = C[2 * ld];
    C[(nlev + 2) * ld] = C[(nlev + 3) * ld] = C[(nlev + 1) * ld];
  }
  __syncthreads();
  for (int l = kt; l <= nlev + 1; l += KT) S[l * ld] = slope(lim, C[l * ld], C[(l + 1) * ld], C[(l + 2) * ld]);
  __syncthreads();
  for (int l = 1 + kt; l <= nlev; l += KT) {
    const float f = C[(l + 1) * ld], s0 = S[l * ld];
    float fl, df, f6;
    ppm_cell(f, s0, ppm_edge(C[l * ld], f, S[(l - 1) * ld], s0), ppm_edge(f, C[(l + 2) * ld], s0, S[(l + 1) * ld]), fl,
             df, f6);
    FL[(l - 1) * ld] = fl;
    DF[(l - 1) * ld] = df;
    F6[(l - 1) * ld] = f6;
  }
  __syncthreads();
  auto flux_at = [&](int k, float c, float wv) {   // interface k (2 .. nlev)
    float fz = 0;
    if (fabsf(c) < 1.0f && g.flux_type == GMC_FLUX_VAN_LEER) {   // upwind cell k-1 or k
      if (c > 0) fz = fdiv(wv * (c * (C[k * ld] + S[(k - 1) * ld] * 0.5f * (1.0f - c))), c);
      else if (c < 0) fz = fdiv(wv * (c * (C[(k + 1) * ld] - S[k * ld] * 0.5f * (1.0f + c))), c);
    } else if (fabsf(c) < 1.0f) {
      if (c > 0) {
        const int u = k - 2;
        fz = fdiv(wv * ppm_tail(0.0f, FL[u * ld], DF[u * ld], F6[u * ld], 1.0f - c, 1.0f), c);
      } else if (c < 0) {
        const int u = k - 1;
        fz = fdiv(-wv * ppm_tail(0.0f, FL[u * ld], DF[u * ld], F6[u * ld], 0.0f, -c), c);
      }
    } else if (valid) {
      fz = vflx_tile<float>(g, C, FL, DF, F6, ld, k, c, wv);
    }
    return fz;
  };
#pragma unroll
  for (int m = 0; m < kColPre; ++m) {
    const int k = 1 + kt + m * KT;
    if (k <= nlev + 1) FZ[(k - 1) * ld] = k != 1 && k != nlev + 1 ? flux_at(k, cz[m], wz[m]) : 0.0f;
  }
  for (int k = 1 + kt + kColPre * KT; k <= nlev + 1; k += KT) {
    float fz = 0;
    if (k != nlev + 1) {
      const size_t ol = ix3(nlat, nlon, ic, j, k);
      fz = flux_at(k, cflz[ol], we[ol]);
    }
    FZ[(k - 1) * ld] = fz;
  }
  __syncthreads();
  const float dta = (float)dt_adv;
  bool neg = false;
  for (int k = 1 + kt; k <= nlev; k += KT) {
    float qn = C[(k + 1) * ld] - ((FZ[k * ld] - FZ[(k - 1) * ld]) * dta) / M[(k - 1) * ld];
    C[(k + 1) * ld] = qn;
    neg |= valid && qn < 0;
  }
  if (__syncthreads_or(neg) && kt == 0 && valid) {
    float *qc = C + ld;   // qc[k * ld] = q(k)
    for (int k = 1; k <= nlev; ++k) {
      float v = qc[k * ld];
      if (v < 0) {
        const float m0 = M[(k - 1) * ld];
        const float qm0 = v * m0;
        const float qm1 = k > 1 ? qc[(k - 1) * ld] * M[(k - 2) * ld] : 0.0f;
        const float qm2 = k < nlev ? qc[(k + 1) * ld] * M[k * ld] : 0.0f;
        const float qm0_half = 0.5f * qm0;
        if (qm1 >= qm0_half && qm2 >= qm0_half) {
          if (qm1 > 0) qc[(k - 1) * ld] = (qm1 - qm0_half) / M[(k - 2) * ld];
          if (qm2 > 0) qc[(k + 1) * ld] = (qm2 - qm0_half) / M[k * ld];
        } else if (qm1 > qm0) {
          if (qm1 > 0) qc[(k - 1) * ld] = (qm1 - qm0) / M[(k - 2) * ld];
        } else if (qm2 > qm0) {
          if (qm2 > 0) qc[(k + 1) * ld] = (qm2 - qm0) / M[k * ld];
        } else {
          raise_err(g, ERR_NEGTRACER);
        }
        qc[k * ld] = 0;
      }
    }
  }
  __syncthreads();
  if (!valid) return;
  for (int k = 1 + kt; k <= nlev; k += KT) q[ix3(nlat, nlon, i, j, k)] = C[(k + 1) * ld];
}

// Order-2 zonal smoother applied three times (lon_damp_1d, lon_damp_mod.F90:200-241).
template <class R>
__global__ void k_tracer_lon_damp(DGrid g, R *q) {
  extern __shared__ double sh[];
  const int j = blockIdx.x + 1, k = blockIdx.y + 1, nlon = g.nlon, nlat = g.nlat;
  if (j == 1 || j == nlat) return;
  const double wgt = g.lon_damp_full[j - 1];
  if (wgt == 0) return;
  R *f = reinterpret_cast<R *>(sh), *gw = f + nlon;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) f[i] = q[ix3(nlat, nlon, i + 1, j, k)];
  const R w = (R)wgt, c = (R)0.25;
  for (int pass = 0; pass < 3; ++pass) {
    __syncthreads();
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
      R fm = f[i == 0 ? nlon - 1 : i - 1], fc = f[i], fp = f[i == nlon - 1 ? 0 : i + 1];
      gw[i] = w * (fc + c * (fm - (R)2 * fc + fp)) + ((R)1 - w) * fc;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nlon; i += blockDim.x) f[i] = gw[i];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) q[ix3(nlat, nlon, i + 1, j, k)] = f[i];
}

}  // namespace

template <class R>
void launch_ffsl_inner_y(const DGrid &g, const Launch &L, const BatchView<R> &b, const R *q, R *qy, double dt) {
  // blocks: (column chunk, band of rows, level x member)
  const dim3 grid((g.nlon + kYThreads - 1) / kYThreads, (g.nlat - 2 + kYBand - 1) / kYBand, g.nlev * L.members);
  mb_launch(L, [&](auto mb) { k_ffsl_inner_y<R, decltype(mb)::value><<<grid, kYThreads, 0, L.stream>>>(g, b.v, b.cfly, q, b.divy, qy, dt); });
}
template <class R>
void launch_ffsl_x2(const DGrid &g, const Launch &L, const BatchView<R> &b, const R *q, const R *qy, R *qx, R *fx,
                    double dt) {
  const size_t smem_x = (size_t)(5 * g.nlon + 17) * sizeof(R);   // padded rows, slopes, inner fluxes
  if (smem_x > 48 * 1024) { cudaFuncSetAttribute(k_ffsl_x2<R, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_x); cudaFuncSetAttribute(k_ffsl_x2<R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_x); }
  mb_launch(L, [&](auto mb) { k_ffsl_x2<R, decltype(mb)::value><<<dim3(g.nlat, g.nlev, L.members), L.threads, smem_x, L.stream>>>(g, b.u, b.mfx, b.cflx, q, qy, b.divx, qx, fx, dt); });
}
template <class R>
void launch_hflx_y(const DGrid &g, const Launch &L, const BatchView<R> &b, const R *qx, R *fy) {
  const dim3 grid((g.nlon + kYThreads - 1) / kYThreads, (g.nhalf + kYBand - 1) / kYBand, g.nlev * L.members);
  mb_launch(L, [&](auto mb) { k_hflx_y<R, decltype(mb)::value><<<grid, kYThreads, 0, L.stream>>>(g, b.mfy, b.cfly, qx, fy); });
}

// One horizontal FFSL flux evaluation (fx, fy of q; qx, qy scratch): the y
// inner pass (qy), then both x passes (qx and fx), then the y outer pass on qx.
template <class R>
void launch_ffsl_hflx(const DGrid &g, const Launch &L, const BatchView<R> &b, const R *q, R *qx, R *qy, R *fx, R *fy,
                      double dt) {
  launch_ffsl_inner_y<R>(g, L, b, q, qy, dt);
  launch_ffsl_x2<R>(g, L, b, q, qy, qx, fx, dt);
  launch_hflx_y<R>(g, L, b, qx, fy);
}

template <class R>
void launch_pt_tendency(const DGrid &g, const Launch &L, const Slot<R> &s, const Work<R> &w) {
  if constexpr (std::is_same<R, float>::value) {
    const size_t smem = g.nlev * sizeof(double) + (size_t)(6 * g.nlev + 7) * (kTileI + 1) * sizeof(float);
    if (smem > 48 * 1024) { cudaFuncSetAttribute(k_pt_tendency_f<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); cudaFuncSetAttribute(k_pt_tendency_f<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); }
    mb_launch(L, [&](auto mb) { k_pt_tendency_f<decltype(mb)::value><<<dim3((g.nlon + kTileI - 1) / kTileI, g.nlat, L.members), dim3(kTileI, kTileK), smem, L.stream>>>(g, s, w); });
    return;
  }
  const int bt = 64;
  size_t smem = (32 + g.nlev + 2) * sizeof(double);
  mb_launch(L, [&](auto mb) { k_pt_tendency<R, decltype(mb)::value><<<dim3((g.nlon + bt - 1) / bt, g.nlat, L.members), bt, smem, L.stream>>>(g, s, w); });
}

template void launch_ffsl_hflx<double>(const DGrid &, const Launch &, const BatchView<double> &, const double *, double *,
                                       double *, double *, double *, double);
template void launch_ffsl_hflx<float>(const DGrid &, const Launch &, const BatchView<float> &, const float *, float *,
                                      float *, float *, float *, double);
#define INST_FFSL_PARTS(R)                                                                                           \
  template void launch_ffsl_inner_y<R>(const DGrid &, const Launch &, const BatchView<R> &, const R *, R *, double);  \
  template void launch_ffsl_x2<R>(const DGrid &, const Launch &, const BatchView<R> &, const R *, const R *, R *, R *, \
                                  double);                                                                            \
  template void launch_hflx_y<R>(const DGrid &, const Launch &, const BatchView<R> &, const R *, R *);
INST_FFSL_PARTS(double)
INST_FFSL_PARTS(float)
template void launch_pt_tendency<double>(const DGrid &, const Launch &, const Slot<double> &, const Work<double> &);
template void launch_pt_tendency<float>(const DGrid &, const Launch &, const Slot<float> &, const Work<float> &);

}  // namespace gmc

namespace gmc {

template <class T>
void launch_accum(const Launch &L, T *dst, const T *src, size_t n, int mode, double divisor) {
  int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  k_accum<T><<<blocks, 256, 0, L.stream>>>(dst, src, n, mode, divisor);
}
template void launch_accum<double>(const Launch &, double *, const double *, size_t, int, double);
template void launch_accum<float>(const Launch &, float *, const float *, size_t, int, double);

template <class T>
void launch_accum_multi(const Launch &L, const AccumSet<T> &set) {
  if (set.count <= 0) return;
  size_t nmax = 0;
  for (int t = 0; t < set.count; ++t) nmax = std::max(nmax, set.e[t].n);
  const int blocks = (int)std::min<size_t>((nmax / 4 + 255) / 256 + 1, 152 * 4);
  k_accum_multi<T><<<dim3(blocks, set.count), 256, 0, L.stream>>>(set);
}
template void launch_accum_multi<double>(const Launch &, const AccumSet<double> &);
template void launch_accum_multi<float>(const Launch &, const AccumSet<float> &);

template <class R>
void launch_half_level_mass(const DGrid &g, const Launch &L, const SurfP<R> &sp, R *m_lev, int mode, double divisor) {
  if constexpr (std::is_same<R, float>::value) {
    if (g.baroclinic) {
      const int H = g.nlat * g.nlon;
      k_half_level_mass_f<<<dim3((H + 255) / 256, g.nlev + 1), 256, 0, L.stream>>>(
          g, sp.phs_f ? sp.psr : nullptr, m_lev, mode, (float)divisor);
      return;
    }
  }
  const int bt = 64;
  k_half_level_mass<R><<<dim3((g.nlon + bt - 1) / bt, g.nlat), bt, 0, L.stream>>>(g, sp, m_lev, mode, divisor);
}

template <class R>
void launch_batch_cflz(const DGrid &g, const Launch &L, const R *we, const R *m_lev, R *cflz, double dt) {
  const int bt = 64;
  const size_t smem = std::is_same<R, float>::value ? (size_t)(g.nlev + 1) * bt * sizeof(float) : 0;
  k_batch_cflz<R><<<dim3((g.nlon + bt - 1) / bt, g.nlat), bt, smem, L.stream>>>(g, we, m_lev, cflz, dt);
}

template <class R>
void launch_tracer_horizontal(const DGrid &g, const Launch &L, const R *q_old, R *q_new, const R *fx, const R *fy,
                              const SurfP<R> &old_sp, const SurfP<R> &sp, double dt_adv) {
  size_t smem = 32 * sizeof(double) + 2 * (g.nlon + 2) * sizeof(R) + 16;
  const int bt = std::is_same<R, float>::value ? 128 : L.threads;   // FP32: two points per thread
  k_tracer_horizontal<R><<<dim3(g.nlat, g.nlev), bt, smem, L.stream>>>(g, q_old, q_new, fx, fy, old_sp, sp, dt_adv);
}

template <class R>
void launch_tracer_vertical(const DGrid &g, const Launch &L, R *q, const R *cflz, const R *we, const SurfP<R> &sp,
                            double dt_adv) {
  const int bt = 64;
  if constexpr (std::is_same<R, float>::value) {
    const size_t smem = (size_t)(7 * g.nlev + 7) * (kTileI + 1) * sizeof(float);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_tracer_vertical_f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tracer_vertical_f<<<dim3((g.nlon + kTileI - 1) / kTileI, g.nlat), dim3(kTileI, kTileK), smem, L.stream>>>(
        g, q, cflz, we, sp, dt_adv);
    return;
  }
  k_tracer_vertical<R><<<dim3((g.nlon + bt - 1) / bt, g.nlat), bt, 0, L.stream>>>(g, q, cflz, we, sp, dt_adv);
}

template <class R>
void launch_tracer_lon_damp(const DGrid &g, const Launch &L, R *q) {
  k_tracer_lon_damp<R><<<dim3(g.nlat, g.nlev), L.threads, 2 * g.nlon * sizeof(R), L.stream>>>(g, q);
}

#define INST_TRACER(R)                                                                                              \
  template void launch_half_level_mass<R>(const DGrid &, const Launch &, const SurfP<R> &, R *, int, double);      \
  template void launch_batch_cflz<R>(const DGrid &, const Launch &, const R *, const R *, R *, double);           \
  template void launch_tracer_horizontal<R>(const DGrid &, const Launch &, const R *, R *, const R *, const R *,  \
                                            const SurfP<R> &, const SurfP<R> &, double);                         \
  template void launch_tracer_vertical<R>(const DGrid &, const Launch &, R *, const R *, const R *,                \
                                          const SurfP<R> &, double);                                             \
  template void launch_tracer_lon_damp<R>(const DGrid &, const Launch &, R *);
INST_TRACER(double)
INST_TRACER(float)

}  // namespace gmc
