// Device helpers shared by the dynamics and advection kernels: layer mass,
// PPM reconstruction, polar-filter row convolution.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace gmc {

// ---------------------------------------------------------------------------
// Layer mass m = ph_lev(k+1) - ph_lev(k) from the filtered surface pressure
// (calc_ph + calc_m, operators_mod.F90:136-168, 471-503).  The FP64 form
// evaluates the reference's hybrid formula term by term; the FP32 form uses
// per-layer coefficients dA_k + dB_k (phs - ptop).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double ph_lev(const DGrid &g, int k, double phs) {
  return g.hyai[k - 1] * (g.p0h - g.ptop) + g.hybi[k - 1] * (phs - g.ptop) + g.ptop;
}

template <class R>
struct Mass;

template <>
struct Mass<double> {
  static __device__ __forceinline__ double layer(const DGrid &g, int k, double phs) {
    return ph_lev(g, k + 1, phs) - ph_lev(g, k, phs);
  }
};
template <>
struct Mass<float> {
  // psr = phs - ptop in FP32
  static __device__ __forceinline__ float layer(const DGrid &g, int k, float psr) {
    return fmaf(g.dmB[k - 1], psr, g.dmA[k - 1]);
  }
};

// Cell mass at (i, j, k): baroclinic from the surface pressure, shallow water
// (gz - gzs)/g.
template <class R>
struct MassField {
  SurfP<R> sp;           // baroclinic
  const R *gz;           // shallow water
  const double *gzs;
  __device__ __forceinline__ R at(const DGrid &g, int i, int j, int k) const {
    i = wrap(i, g.nlon);
    size_t o = (size_t)(j - 1) * g.nlon + (i - 1);
    if (g.baroclinic) return Mass<R>::layer(g, k, sp.at(o));
    return (R)(((double)gz[o] - gzs[o]) / g.g);
  }
};

// Cell mass on level k with the level's constants held by the block; at(o)
// takes the 0-based offset o = (j-1) nlon + (i-1) of the cell in a 2D field
// and gives MassField::at bit for bit.
template <class R>
struct LevMass {
  const DGrid &g;
  SurfP<R> sp;
  const R *gz;
  const double *gzs;
  int k;
  float a = 0, b = 0;   // FP32 form: dmA_k, dmB_k
  __device__ __forceinline__ LevMass(const DGrid &g_, SurfP<R> sp_, const R *gz_, const double *gzs_, int k_)
      : g(g_), sp(sp_), gz(gz_), gzs(gzs_), k(k_) {
    if constexpr (std::is_same<R, float>::value) {
      a = g.dmA[k - 1];
      b = g.dmB[k - 1];
    }
  }
  __device__ __forceinline__ R at(unsigned o) const {
    if (g.baroclinic) {
      if constexpr (std::is_same<R, float>::value) return fmaf(b, sp.psr[o], a);
      else return Mass<double>::layer(g, k, sp.phs_f[o]);
    }
    return (R)(((double)gz[o] - gzs[o]) / g.g);
  }
};

// TVD interpolation with flux limiter (tvd_mod.F90:44-84); eps is the
// default-kind literal 1.0e-6 of the reference widened to double.
template <class R>
__device__ __forceinline__ R tvd_interp(int limiter, R cfl, R fm1, R f, R fp1, R fp2) {
  const R eps = (R)(double)1.0e-6f;
  const R r = cfl > 0 ? (f - fm1 + eps) / (fp1 - f + eps) : (fp2 - fp1 + eps) / (fp1 - f + eps);
  R C;
  if (limiter == GMC_TVD_NONE) C = 1;
  else if (limiter == GMC_TVD_MC) C = fmax((R)0, fmin(fmin((R)2 * r, (R)0.5 * (1 + r)), (R)2));
  else C = (r + fabs(r)) / (1 + fabs(r));
  return (R)0.5 * (fp1 + f - ((1 - C) * fsign((R)1, cfl) + cfl * C) * (fp1 - f));
}

// Upwind interpolation of order 3 and 1 (upwind_mod.F90:27-39) along the
// direction dir = sign of the advecting wind, weighted by wgt.
template <class R>
__device__ __forceinline__ R upwind3(R dir, R wgt, R f1, R f2, R f3, R f4) {
  const R c31 = (R)(7.0 / 12.0), c32 = (R)(-1.0 / 12.0), c33 = (R)(1.0 / 12.0);
  return c31 * (f3 + f2) + c32 * (f4 + f1) + c33 * (f4 - f1 - (R)3 * (f3 - f2)) * wgt * dir;
}
template <class R>
__device__ __forceinline__ R upwind1(R dir, R wgt, R f1, R f2) {
  return (R)0.5 * (f2 + f1) + (R)(-0.5) * (f2 - f1) * wgt * dir;
}

// ---------------------------------------------------------------------------
// PPM sub-grid reconstruction with slope limiter (ffsl_mod.F90:1147-1205).
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ R slope(int limiter, R fm1, R f, R fp1) {
  R df = (fp1 - fm1) * (R)0.5;
  if (limiter == GMC_LIMITER_NONE) return df;
  if (limiter == GMC_LIMITER_PD) return fsign(fmin(fabs(df), (R)2 * f), df);
  R dmin = (R)2 * (f - fmin(fmin(fm1, f), fp1));
  R dmax = (R)2 * (fmax(fmax(fm1, f), fp1) - f);
  return fsign(fmin(fmin(fabs(df), dmin), dmax), df);
}

// x / 6 and x / 3: exact divisions in the FP64 form, products with the
// rounded reciprocal in the FP32 form.
__device__ __forceinline__ double div6(double x) { return x / 6.0; }
__device__ __forceinline__ float div6(float x) { return x * (1.0f / 6.0f); }
__device__ __forceinline__ double div3(double x) { return x / 3.0; }
__device__ __forceinline__ float div3(float x) { return x * (1.0f / 3.0f); }
// a / b: IEEE division in the FP64 form, the approximate division (MUFU
// reciprocal and product, within 2 ulp) in FP32.
__device__ __forceinline__ double fdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }

template <class R>
__device__ __forceinline__ void ppm(int limiter, R fm2, R fm1, R f, R fp1, R fp2, R &fl, R &df, R &f6) {
  R dfl = slope(limiter, fm2, fm1, f);
  df = slope(limiter, fm1, f, fp1);
  R dfr = slope(limiter, f, fp1, fp2);
  fl = (R)0.5 * (fm1 + f) + div6(dfl - df);
  R fr = (R)0.5 * (fp1 + f) + div6(df - dfr);
  fl = f - fsign(fmin(fabs(df), fabs(fl - f)), df);
  fr = f + fsign(fmin(fabs(df), fabs(fr - f)), df);
  f6 = (R)6 * f - (R)3 * (fl + fr);
  df = fr - fl;
}

// Cell-centric form of ppm(): the unlimited edge value between cells (fm, f)
// with slopes (sm, s) is shared by both cells, and the limited coefficients
// of a cell follow from its value, slope and two edges.  ppm_cell(f, s,
// ppm_edge(fm1, f, dfl, s), ppm_edge(f, fp1, s, dfr)) equals ppm() bit for bit
// (the edge sum is commutative).
template <class R>
__device__ __forceinline__ R ppm_edge(R fm, R f, R sm, R s) {
  return (R)0.5 * (fm + f) + div6(sm - s);
}
template <class R>
__device__ __forceinline__ void ppm_cell(R f, R s, R el, R er, R &fl, R &df, R &f6) {
  fl = f - fsign(fmin(fabs(s), fabs(el - f)), s);
  const R fr = f + fsign(fmin(fabs(s), fabs(er - f)), s);
  f6 = (R)6 * f - (R)3 * (fl + fr);
  df = fr - fl;
}

// Whole-cell sum plus the integral of the parabola over the upwind fraction
// [s1, s2] of the departure cell, the common tail of hflx_ppm_cell and
// vflx_ppm_cell (ffsl_mod.F90:833-875, 917-935).
template <class R>
__device__ __forceinline__ R ppm_tail(R sum, R fl, R df, R f6, R s1, R s2) {
  R ds1 = s2 - s1;
  R ds2 = s2 * s2 - s1 * s1;
  R ds3 = s2 * s2 * s2 - s1 * s1 * s1;
  return sum + fl * ds1 + (R)0.5 * df * ds2 + f6 * (ds2 / (R)2 - div3(ds3));
}

// Sum over a warp of a double (all 32 lanes take part).
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Column tiles of the FP32 form: a block holds kTileI columns (threadIdx.x)
// of one latitude row and spreads the levels over threadIdx.y, so every
// level of every column is worked on in parallel; per-column vertical
// quantities live in shared memory as [level][kTileI + 1] (padded against
// bank conflicts).
constexpr int kTileI = 32, kTileK = 8;

// Pole ring sums of one level field by the warps of a column-tile block:
// ring[k-1] = sgn * sum_i f(i, jv, k) * le_lat(jv) / nlon / area_cell(j).
template <class F>
__device__ __forceinline__ void tile_pole_ring(const DGrid &g, int j, float *ring, F f) {
  const int lt = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = lt & 31, warp = lt >> 5, nw = (blockDim.x * blockDim.y) >> 5;
  const int jv = j == 1 ? 1 : g.nhalf;
  const double sgn = j == 1 ? 1.0 : -1.0;
  for (int k = 1 + warp; k <= g.nlev; k += nw) {
    double acc = 0;
    for (int ii = 1 + lane; ii <= g.nlon; ii += 32) acc += (double)f(ii, jv, k);
    acc = warp_sum(acc);
    if (lane == 0) ring[k - 1] = (float)(sgn * acc * ROW(g.le_lat, jv) / g.nlon / ROW(g.area_cell, j));
  }
}

// FP32 form of cflz_of over a column held as wm(l) = we(l) / ml(l) * half_dlev(l)
// at wm[(l - 1) * stride] for l = 1 .. nlev+1: the per-level quotients are
// formed once per column instead of once per RK4 interpolation.
// HL, FD, RFD: half_lev, full_dlev and 1 / full_dlev in FP32 (index [k-1]),
// from the grid tables or a shared-memory copy of them.
//
// Every RK4 position z = z0 + c w lies on the side of z0 = HL[k-1] that the
// sign of w gives, so the level search (first layer l >= k with z <= HL[l]
// for w > 0, first l <= k-1 with HL[l-1] <= z otherwise) mostly stops at the
// layer next to z0, and the displacement mostly stays within one layer.  The
// two layers k-1 and k and their table values are loaded once; a position or
// displacement beyond them (or a NaN) takes the general search and walk,
// which also flags a departure outside the column.  Same operations on the
// same operands as the general path, so the same values.
__device__ __forceinline__ float cflz_of_f(const float *HL, const float *FD, const float *RFD, int nlev, const float *wm,
                                           int stride, int k, float dt_, bool &bad) {
  auto W = [&](int l) { return wm[(l - 1) * stride]; };   // l = 1 .. nlev+1
  auto locate = [&](float w, float z) {
    int l;
    if (w > 0) {
      for (l = k; l <= nlev; ++l)
        if (HL[l - 1] <= z && z <= HL[l]) break;
      if (l == nlev + 1) { bad = true; l = nlev; }
    } else {
      for (l = k - 1; l >= 1; --l)
        if (HL[l - 1] <= z && z <= HL[l]) break;
      if (l == 0) { bad = true; l = 1; }
    }
    return l;
  };
  auto interp = [&](int l, float z) { return ((HL[l] - z) * W(l) + (z - HL[l - 1]) * W(l + 1)) * RFD[l - 1]; };
  // layers k-1 (below z0 in eta) and k (above)
  const float h0 = HL[k - 2], h1 = HL[k - 1], h2 = HL[k];
  const float wkm = W(k - 1), wk = W(k), wkp = W(k + 1);
  const float r0 = RFD[k - 2], r1 = RFD[k - 1];
  auto at = [&](float w, float z) {   // wind at z of an RK4 stage moving with w
    if (w > 0) {
      if (z <= h2) return ((h2 - z) * wk + (z - h1) * wkp) * r1;   // layer k
    } else if (h0 <= z) {
      return ((h1 - z) * wkm + (z - h0) * wk) * r0;   // layer k-1
    }
    return interp(locate(w, z), z);
  };
  const float z0 = h1;
  const float w1 = wk;
  const float z1 = z0 + 0.5f * dt_ * w1;
  const float w2 = at(w1, z1);
  const float z2 = z0 + 0.5f * dt_ * w2;
  const float w3 = at(w2, z2);
  const float z3 = z0 + dt_ * w3;
  const float w4 = at(w3, z3);
  float deta = (w1 + 2.0f * w2 + 2.0f * w3 + w4) * (1.0f / 6.0f) * dt_;
  if (deta >= 0) {   // within layer k
    const float d = deta - FD[k - 1];
    if (d < 0) return (1.0f + d * r1) + 0.0f;
  } else {           // within layer k-1
    const float d = fabsf(deta) - FD[k - 2];
    if (d < 0) return -1.0f * ((1.0f + d * r0) + 0.0f);
  }
  int ks, ke, s;
  if (deta < 0) { ks = k - 1; ke = 1; s = -1; } else { ks = k; ke = nlev; s = 1; }
  const float sf = deta < 0 ? -1.0f : 1.0f;
  deta = fabsf(deta);
  float whole = 0;   // |l - ks| counted in FP32 (no integer conversions)
  for (int l = ks; s > 0 ? l <= ke : l >= ke; l += s, whole += 1.0f) {
    deta = deta - FD[l - 1];
    if (deta < 0) return sf * ((1.0f + deta * RFD[l - 1]) + whole);
  }
  return NAN;
}

// ---------------------------------------------------------------------------
// Polar filter of one latitude row (filter_mod.F90:25-163): Gaussian
// convolution with periodic wrap.  The row lives in shared memory; `ext`
// receives the row extended by hn points on each side.  Returns false when
// the row is not filtered (ngrid <= 1).  A is the accumulation type (FP64
// unless the caller asks for the FP32 pipeline).
// ---------------------------------------------------------------------------
// KB rows of the same latitude (KB levels of one row) filtered together: the
// weights are loaded once per tap for all of them.  row[kk * rs + i],
// ext[kk * es + t]; every row equals filter_row of that row alone.
template <int KB, class R, class A = double>
__device__ __forceinline__ bool filter_rows(const FilterDev &f, bool full_lat, int j, int nlon, R *row, int rs, R *ext,
                                            int es) {
  const int n = full_lat ? f.ntaps_full[j - 1] : f.ntaps_half[j - 1];
  if (n <= 1) return false;
  const int hn = (n - 1) / 2;
  const int off = full_lat ? f.off_full[j - 1] : f.off_half[j - 1];
  const A *w;
  if constexpr (std::is_same<A, float>::value) w = f.wgt_f + off; else w = f.wgt + off;
  __syncthreads();
  for (int kk = 0; kk < KB; ++kk)
    for (int t = threadIdx.x; t < nlon + 2 * hn; t += blockDim.x) {
      int i = t - hn + 1;
      i = i < 1 ? i + nlon : (i > nlon ? i - nlon : i);
      ext[kk * es + t] = row[kk * rs + i - 1];
    }
  __syncthreads();
  // three consecutive outputs per thread over a rolling window of ext: one
  // ext load per row and one weight load per tap for 3 KB sums (each sum in
  // tap order, as the one-output loop below forms it)
  const int nfull = nlon - nlon % 3;
  for (int b = 3 * threadIdx.x; b < nfull; b += 3 * blockDim.x) {
    A s0[KB], s1[KB], s2[KB], e0[KB], e1[KB];
#pragma unroll
    for (int kk = 0; kk < KB; ++kk) {
      s0[kk] = s1[kk] = s2[kk] = 0;
      e0[kk] = (A)ext[kk * es + b];
      e1[kk] = (A)ext[kk * es + b + 1];
    }
#pragma unroll 4
    for (int t = 0; t < n; ++t) {   // unrolled: the weights of four taps are requested together
      const A wt = w[t];
#pragma unroll
      for (int kk = 0; kk < KB; ++kk) {
        const A e2 = (A)ext[kk * es + b + t + 2];
        s0[kk] = s0[kk] + wt * e0[kk];
        s1[kk] = s1[kk] + wt * e1[kk];
        s2[kk] = s2[kk] + wt * e2;
        e0[kk] = e1[kk];
        e1[kk] = e2;
      }
    }
#pragma unroll
    for (int kk = 0; kk < KB; ++kk) {
      row[kk * rs + b] = (R)s0[kk];
      row[kk * rs + b + 1] = (R)s1[kk];
      row[kk * rs + b + 2] = (R)s2[kk];
    }
  }
  for (int i = nfull + threadIdx.x; i < nlon; i += blockDim.x)
    for (int kk = 0; kk < KB; ++kk) {
      A s = 0;
      for (int t = 0; t < n; ++t) s = s + w[t] * (A)ext[kk * es + i + t];
      row[kk * rs + i] = (R)s;
    }
  __syncthreads();
  return true;
}
template <class R, class A = double>
__device__ __forceinline__ bool filter_row(const FilterDev &f, bool full_lat, int j, int nlon, R *row, R *ext) {
  return filter_rows<1, R, A>(f, full_lat, j, nlon, row, 0, ext, 0);
}

// Vertical RK4 departure in eta and its Courant number
// (adv_batch_accum_we_lev, adv_batch_mod.F90:525-628).  we and ml hold the
// column's vertical mass flux and half-level mass, index [k-1].  T = double
// evaluates the reference's expressions in FP64; T = float runs the same
// steps on the FP32 pipeline (eta is O(1), so FP32 resolves it to ~1e-7).
template <class T>
__device__ __forceinline__ const T *eta_table(const DGrid &g, int which);
template <>
__device__ __forceinline__ const double *eta_table<double>(const DGrid &g, int which) {
  return which == 0 ? g.half_lev : which == 1 ? g.half_dlev : g.full_dlev;
}
template <>
__device__ __forceinline__ const float *eta_table<float>(const DGrid &g, int which) {
  return which == 0 ? g.half_lev_f : which == 1 ? g.half_dlev_f : g.full_dlev_f;
}

template <class T>
__device__ __forceinline__ T cflz_of(const DGrid &g, const T *we, const T *ml, int k, T dt_, bool &bad) {
  const int nlev = g.nlev;
  const T *HL = eta_table<T>(g, 0), *HD = eta_table<T>(g, 1), *FD = eta_table<T>(g, 2);   // [k-1]
  auto locate = [&](T w, T z) {
    int l;
    if (w > 0) {
      for (l = k; l <= nlev; ++l)
        if (HL[l - 1] <= z && z <= HL[l]) break;
      if (l == nlev + 1) { bad = true; l = nlev; }
    } else {
      for (l = k - 1; l >= 1; --l)
        if (HL[l - 1] <= z && z <= HL[l]) break;
      if (l == 0) { bad = true; l = 1; }
    }
    return l;
  };
  auto interp = [&](int l, T z) {
    return ((HL[l] - z) * we[l - 1] / ml[l - 1] * HD[l - 1] + (z - HL[l - 1]) * we[l] / ml[l] * HD[l]) / FD[l - 1];
  };
  T z0 = HL[k - 1];
  T w1 = we[k - 1] / ml[k - 1] * HD[k - 1];
  T z1 = z0 + dt_ / 2 * w1;
  T w2 = interp(locate(w1, z1), z1);
  T z2 = z0 + dt_ / 2 * w2;
  T w3 = interp(locate(w2, z2), z2);
  T z3 = z0 + dt_ * w3;
  T w4 = interp(locate(w3, z3), z3);
  T deta = (w1 + 2 * w2 + 2 * w3 + w4) / 6 * dt_;
  int ks, ke, s;
  if (deta < 0) { ks = k - 1; ke = 1; s = -1; } else { ks = k; ke = nlev; s = 1; }
  deta = fabs(deta);
  for (int l = ks; s > 0 ? l <= ke : l >= ke; l += s) {
    deta = deta - FD[l - 1];
    if (deta < 0) return s * ((1 + deta / FD[l - 1]) + abs(l - ks));
  }
  return (T)NAN;   // departure left the column: the reference keeps the previous value
}

}  // namespace gmc
