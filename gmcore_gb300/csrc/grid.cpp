// Host-side grid set-up: mesh metrics, hybrid levels, polar-filter weights,
// zonal-smoother weights and seeded synthetic initial states.
// Reference citations are given per routine; see grid.hpp.
#include "grid.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

#if defined(__x86_64__) || defined(__i386__)
#include <quadmath.h>
typedef __float128 quad;
static inline quad q_sqrt(quad x) { return sqrtq(x); }
static inline quad q_acos(quad x) { return acosq(x); }
static inline quad q_asin(quad x) { return asinq(x); }
static inline quad q_atan2(quad y, quad x) { return atan2q(y, x); }
static inline quad q_sin(quad x) { return sinq(x); }
#else
// aarch64 Linux: long double is IEEE binary128.
typedef long double quad;
static inline quad q_sqrt(quad x) { return sqrtl(x); }
static inline quad q_acos(quad x) { return acosl(x); }
static inline quad q_asin(quad x) { return asinl(x); }
static inline quad q_atan2(quad y, quad x) { return atan2l(y, x); }
static inline quad q_sin(quad x) { return sinl(x); }
#endif

namespace gmc {

namespace {

// ---------------------------------------------------------------------------
// Hybrid coefficient tables.  The reference writes these as default-kind
// (single precision) Fortran literals, so each value is the nearest float
// widened to double; the tables keep that rounding (hybrid_coord_test_mod.F90).
// ---------------------------------------------------------------------------
const float kTestL26A[27] = {
    0.002194067f, 0.004895209f, 0.009882418f, 0.01805201f, 0.02983724f, 0.04462334f,
    0.06160587f, 0.07851243f, 0.07731271f, 0.07590131f, 0.07424086f, 0.07228744f,
    0.06998933f, 0.06728574f, 0.06410509f, 0.06036322f, 0.05596111f, 0.05078225f,
    0.04468960f, 0.03752191f, 0.02908949f, 0.02084739f, 0.01334443f, 0.00708499f,
    0.00252136f, 0.00000000f, 0.00000000f};
const float kTestL26B[27] = {
    0.000000f, 0.000000f, 0.000000f, 0.000000f, 0.000000f, 0.000000f, 0.000000f,
    0.000000f, 0.01505309f, 0.03276228f, 0.05359622f, 0.07810627f, 0.1069411f,
    0.1408637f, 0.1807720f, 0.2277220f, 0.2829562f, 0.3479364f, 0.4243822f,
    0.5143168f, 0.6201202f, 0.7235355f, 0.8176768f, 0.8962153f, 0.9534761f,
    0.9851122f, 1.0000000f};
const float kWrfL32A[33] = {
    0.0000000000000000f, 0.0027008056640625f, 0.0076868347823620f, 0.0158526937798342f,
    0.0276367470939261f, 0.0414515552099706f, 0.0562277844155789f, 0.0724737972365225f,
    0.0893795253309864f, 0.1063548465048298f, 0.1254725257849640f, 0.1479642011314251f,
    0.1744233770857367f, 0.2054476619883455f, 0.2362396334209435f, 0.2617261684535087f,
    0.2783057827853432f, 0.2816243248017372f, 0.2683280168286641f, 0.2429473354807992f,
    0.2108099294331058f, 0.1759998110016148f, 0.1415334037742616f, 0.1095123294032484f,
    0.0812761592574764f, 0.0575423961814687f, 0.0385285881906738f, 0.0240694984015316f,
    0.0137226170696702f, 0.0068720184783044f, 0.0027973066609278f, 0.0007580797514921f,
    0.0000000000000000f};
const float kWrfL32B[33] = {
    0.0000000000000000f, 0.0000000000000000f, 0.0000000000000000f, 0.0000000000000000f,
    0.0000000000000000f, 0.0000000000000000f, 0.0000000000000000f, 0.0000000000000000f,
    0.0000000000000000f, 0.0000000000000000f, 0.0000000000000000f, 0.0000000000000000f,
    0.0000000000000000f, 0.0001056069805219f, 0.0059397906834944f, 0.0235374270991938f,
    0.0576439176162314f, 0.1139578493851603f, 0.1932313936022966f, 0.2808764820852269f,
    0.3715629284436812f, 0.4612091687348547f, 0.5467954414732804f, 0.6262219272258057f,
    0.6981497395977654f, 0.7618575996945027f, 0.8171268253424389f, 0.8641240158900223f,
    0.9032994538662682f, 0.9352560448161740f, 0.9607227915792738f, 0.9804356127137464f,
    1.0000000000000000f};
const float kWrfL64A[65] = {
    0.00000000e+00f, 1.56250000e-02f, 3.12500000e-02f, 4.68750000e-02f, 6.25000000e-02f,
    7.81250000e-02f, 9.37500000e-02f, 1.09375000e-01f, 1.25000000e-01f, 1.40625000e-01f,
    1.56250000e-01f, 1.71875000e-01f, 1.87500000e-01f, 2.03091502e-01f, 2.17556953e-01f,
    2.30408311e-01f, 2.41699219e-01f, 2.51483321e-01f, 2.59814262e-01f, 2.66745687e-01f,
    2.72331238e-01f, 2.76624560e-01f, 2.79679298e-01f, 2.81549096e-01f, 2.82287598e-01f,
    2.81948447e-01f, 2.80585289e-01f, 2.78251767e-01f, 2.75001526e-01f, 2.70888209e-01f,
    2.65965462e-01f, 2.60286927e-01f, 2.53906250e-01f, 2.46877074e-01f, 2.39253044e-01f,
    2.31087804e-01f, 2.22434998e-01f, 2.13348269e-01f, 2.03881264e-01f, 1.94087625e-01f,
    1.84020996e-01f, 1.73735023e-01f, 1.63283348e-01f, 1.52719617e-01f, 1.42097473e-01f,
    1.31470561e-01f, 1.20892525e-01f, 1.10417008e-01f, 1.00097656e-01f, 8.99881124e-02f,
    8.01420212e-02f, 7.06130266e-02f, 6.14547729e-02f, 5.27209044e-02f, 4.44650650e-02f,
    3.67408991e-02f, 2.96020508e-02f, 2.31021643e-02f, 1.72948837e-02f, 1.22338533e-02f,
    7.97271729e-03f, 4.56511974e-03f, 2.06470490e-03f, 5.25116920e-04f, 4.44089210e-16f};
const float kWrfL64B[65] = {
    0.00000000e+00f, 0.00000000e+00f, 0.00000000e+00f, 0.00000000e+00f, 0.00000000e+00f,
    0.00000000e+00f, 0.00000000e+00f, 0.00000000e+00f, 0.00000000e+00f, 0.00000000e+00f,
    0.00000000e+00f, 0.00000000e+00f, 0.00000000e+00f, 3.34978104e-05f, 1.19304657e-03f,
    3.96668911e-03f, 8.30078125e-03f, 1.41416788e-02f, 2.14357376e-02f, 3.01293135e-02f,
    4.01687622e-02f, 5.15004396e-02f, 6.40707016e-02f, 7.78259039e-02f, 9.27124023e-02f,
    1.08676553e-01f, 1.25664711e-01f, 1.43623233e-01f, 1.62498474e-01f, 1.82236791e-01f,
    2.02784538e-01f, 2.24088073e-01f, 2.46093750e-01f, 2.68747926e-01f, 2.91996956e-01f,
    3.15787196e-01f, 3.40065002e-01f, 3.64776731e-01f, 3.89868736e-01f, 4.15287375e-01f,
    4.40979004e-01f, 4.66889977e-01f, 4.92966652e-01f, 5.19155383e-01f, 5.45402527e-01f,
    5.71654439e-01f, 5.97857475e-01f, 6.23957992e-01f, 6.49902344e-01f, 6.75636888e-01f,
    7.01107979e-01f, 7.26261973e-01f, 7.51045227e-01f, 7.75404096e-01f, 7.99284935e-01f,
    8.22634101e-01f, 8.45397949e-01f, 8.67522836e-01f, 8.88955116e-01f, 9.09641147e-01f,
    9.29527283e-01f, 9.48559880e-01f, 9.66685295e-01f, 9.83849883e-01f, 1.00000000e+00f};

// ---------------------------------------------------------------------------
// Spherical geometry in binary128 (sphere_geometry_mod.F90:96-448).
// ---------------------------------------------------------------------------
struct V3 { quad x, y, z; };

V3 to_cartesian(double lon, double lat, double radius) {
  // cartesian_transform_1_r16: cos/sin evaluated in double, products in quad;
  // z = radius * sin(lat) is a double product widened afterwards.
  quad cos_lat = (quad)std::cos(lat);
  V3 p;
  p.x = (quad)radius * cos_lat * (quad)std::cos(lon);
  p.y = (quad)radius * cos_lat * (quad)std::sin(lon);
  p.z = (quad)(radius * std::sin(lat));
  return p;
}

V3 cross(const V3 &a, const V3 &b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
quad dot(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 unit(const V3 &a) {
  quad n = q_sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  if (n != 0) return V3{a.x / n, a.y / n, a.z / n};
  return a;
}

// Interior angle at b of the spherical polygon a-b-c (dihedral angle between
// the planes through the centre, a, b and b, c).
quad vertex_angle(const V3 &a, const V3 &b, const V3 &c, double pi2) {
  V3 nab = unit(cross(a, b));
  V3 nbc = unit(cross(b, c));
  quad d = dot(nab, nbc);
  if (d > 1) d = 1;
  if (d < -1) d = -1;
  quad ang = q_acos(-d);
  if (dot(cross(nab, nbc), a) < 0) ang = (quad)pi2 - ang;
  return ang;
}

// Spherical excess of a triangle times radius^2.
quad triangle_area(const V3 p[3], double radius, double pi, double pi2) {
  quad s = 0;
  for (int i = 0; i < 3; ++i) {
    const V3 &a = p[(i + 2) % 3], &b = p[i], &c = p[(i + 1) % 3];
    s += vertex_angle(a, b, c, pi2);
  }
  return (quad)(radius * radius) * (s - (quad)(1 * pi));
}

void to_lonlat(const V3 &p, double radius, double pi2, quad &lon, quad &lat) {
  lon = q_atan2(p.y, p.x);
  lat = q_asin(p.z / (quad)radius);
  if (lon < 0) lon = lon + (quad)pi2;
}

// Triangle whose last edge (p1-p2) follows a latitude circle instead of a
// great circle: great-circle area corrected by the lune between the two arcs
// (calc_area_with_last_small_arc, sphere_geometry_mod.F90:328-390).
quad small_arc_triangle_area(const V3 p[3], double radius, double pi, double pi2) {
  quad res = triangle_area(p, radius, pi, pi2);
  quad lon0, lat0, lon1, lat1, lon2, lat2;
  to_lonlat(p[0], radius, pi2, lon0, lat0);
  to_lonlat(p[1], radius, pi2, lon1, lat1);
  to_lonlat(p[2], radius, pi2, lon2, lat2);
  if (lat1 == 0) return res;
  quad dlon = lat0 > lat1 ? lon2 - lon1 : lon1 - lon2;
  if (dlon < 0) dlon = dlon + (quad)pi2;
  bool pole_side = (lat0 * lat1 >= 0) && ((lat0 < 0 ? -lat0 : lat0) > (lat1 < 0 ? -lat1 : lat1));
  V3 v[3];
  v[0].x = 0; v[0].y = 0;
  if (pole_side) { v[1] = p[1]; v[2] = p[2]; } else { v[1] = p[2]; v[2] = p[1]; }
  quad cap;
  quad r2 = (quad)(radius * radius);
  if (lat1 > 0) {
    v[0].z = (quad)radius;
    cap = r2 * dlon * ((quad)1 - q_sin(lat1));
  } else {
    v[0].z = -(quad)radius;
    cap = r2 * dlon * (q_sin(lat1) + (quad)1);
  }
  quad tri = triangle_area(v, radius, pi, pi2);
  quad lune = cap - tri;
  if (lune < 0 && -lune > (quad)1.0e-10) lune = 0;
  return pole_side ? res + lune : res - lune;
}

double gaussian_sum_normalise(std::vector<double> &w) {
  double s = 0;
  for (double x : w) s += x;
  for (double &x : w) x = x / s;
  return s;
}

// gaussian_weight (filter_types_mod.F90:31-47).
std::vector<double> gaussian_weights(double width, int ngrid, double coef_b, double pi2) {
  std::vector<double> w(ngrid);
  double s = coef_b * width / 2.0;
  for (int i = 1; i <= ngrid; ++i) {
    int x = i - (ngrid + 1) / 2;
    int x2 = -(x * x);
    w[i - 1] = std::exp((double)x2 / (2 * s * s)) / (s * std::sqrt(pi2));
  }
  gaussian_sum_normalise(w);
  return w;
}

double exp_two_values(double v1, double v2, double x0, double x1, double x) {
  // math_mod.F90:146-159
  double w = std::exp((x - x0) * (x - x0) * std::log(1.0e-3) / ((x1 - x0) * (x1 - x0)));
  return w * v1 + (1 - w) * v2;
}

}  // namespace

int Filter::max_taps() const {
  int m = 1;
  for (int n : ngrid_full) m = std::max(m, n);
  for (int n : ngrid_half) m = std::max(m, n);
  return m;
}

std::string validate_config(const gmc_config &c) {
  if (c.nlon < 8 || c.nlon % 2 != 0) return "nlon must be even and >= 8";
  if (c.nlat < 5) return "nlat must be >= 5";
  if (c.nlev < 1) return "nlev must be >= 1";
  if (!c.baroclinic && c.nlev != 1) return "shallow water needs nlev = 1";
  if (c.baroclinic) {
    if (c.vert_coord_template != GMC_VCOORD_TEST_L26 && c.vert_coord_template != GMC_VCOORD_WRF_L32 &&
        c.vert_coord_template != GMC_VCOORD_WRF_L64)
      return "unsupported vert_coord_template";
    if (c.nlev != c.vert_coord_template) return "nlev does not match the vertical template";
  }
  if (c.time_scheme < GMC_TIME_EULER || c.time_scheme > GMC_TIME_WRFRK3) return "bad time_scheme";
  if (c.ke_scheme != 1 && c.ke_scheme != 2) return "ke_scheme must be 1 or 2";
  if (c.pv_scheme != GMC_PV_MIDPOINT && c.pv_scheme != GMC_PV_UPWIND && c.pv_scheme != GMC_PV_TVD)
    return "pv_scheme must be midpoint, upwind or tvd";
  if (c.pv_scheme == GMC_PV_TVD && (c.tvd_limiter_type < GMC_TVD_NONE || c.tvd_limiter_type > GMC_TVD_MC))
    return "bad tvd_limiter_type";
  if (c.pv_scheme == GMC_PV_UPWIND && c.upwind_order_pv != 1 && c.upwind_order_pv != 3)
    return "upwind_order_pv must be 1 or 3";
  if (c.coriolis_scheme != 1 && c.coriolis_scheme != 2) return "coriolis_scheme must be 1 or 2";
  if (c.ffsl_flux_type != GMC_FLUX_PPM && c.ffsl_flux_type != GMC_FLUX_VAN_LEER) return "ffsl_flux_type must be ppm or van_leer";
  if (c.limiter_type < GMC_LIMITER_NONE || c.limiter_type > GMC_LIMITER_PD) return "bad limiter_type";
  if (!(c.dt_dyn > 0)) return "dt_dyn must be > 0";
  if (c.ntracer < 0 || c.ntracer > 64) return "ntracer must be in 0..64";
  if (c.ntracer > 0 && !c.baroclinic) return "tracers need the baroclinic model";
  if (c.precision != GMC_PREC_FP64 && c.precision != GMC_PREC_MIXED) return "bad precision";
  if (c.n_members < 1) return "n_members must be >= 1";
  if (c.use_div_damp && c.div_damp_order != 2 && c.div_damp_order != 4) return "div_damp_order must be 2 or 4";
  if (c.lon_halo_width < 1) return "lon_halo_width must be >= 1";
  if (c.forcing != GMC_FORCING_NONE && c.forcing != GMC_FORCING_HELD_SUAREZ) return "bad forcing";
  if (c.forcing == GMC_FORCING_HELD_SUAREZ && !c.baroclinic) return "held_suarez forcing needs the baroclinic model";
  if (c.use_smag_damp && !(c.smag_damp_coef >= 0)) return "smag_damp_coef must be >= 0";
  // device kernels index one field with 32-bit arithmetic
  if ((double)(c.nlev + 1) * c.nlat * c.nlon >= 2147483647.0) return "grid too large: (nlev+1)*nlat*nlon must be < 2^31";
  return "";
}

std::string Grid::build(const gmc_config &c) {
  std::string err = validate_config(c);
  if (!err.empty()) return err;
  cfg = c;
  nlon = c.nlon;
  nlat = c.nlat;
  nhalf = c.nlat - 1;
  nlev = c.nlev;
  pi = std::atan(1.0) * 4.0;
  pi2 = pi * 2;
  pi05 = pi * 0.5;
  deg = 180.0 / pi;
  const double radius = c.radius;
  const double inf = std::numeric_limits<double>::max();

  // --- longitudes (mesh_mod.F90:180-186) ---
  dlon = (pi2 - 0.0) / nlon;
  full_lon.resize(nlon + 2);
  half_lon.resize(nlon + 2);
  for (int i = 1; i <= nlon + 1; ++i) {
    full_lon[i - 1] = 0.0 + (i - 1) * dlon;
    half_lon[i - 1] = full_lon[i - 1] + 0.5 * dlon;
  }

  // --- latitudes (mesh_mod.F90:188-261) ---
  for (RowTable *t : {&full_lat, &full_lat_deg, &full_cos_lat, &full_sin_lat}) t->init(nlat, inf);
  for (RowTable *t : {&half_lat, &half_lat_deg, &half_cos_lat, &half_sin_lat}) t->init(nhalf, inf);
  double dlat0 = (pi05 - (-pi05)) / nhalf;
  std::vector<double> dlat(nhalf + 1, dlat0);
  full_lat[1] = -pi05;
  full_lat_deg[1] = -pi05 * deg;
  for (int j = 2; j <= nlat - 1; ++j) {
    full_lat[j] = full_lat[j - 1] + dlat[j - 1];
    if (std::fabs(full_lat[j]) < 1.0e-12) full_lat[j] = 0.0;
    full_lat_deg[j] = full_lat[j] * deg;
  }
  full_lat[nlat] = pi05;
  full_lat_deg[nlat] = pi05 * deg;
  for (int j = 1; j <= nhalf; ++j) {
    half_lat[j] = full_lat[j] + 0.5 * dlat[j];
    if (std::fabs(half_lat[j]) < 1.0e-12) half_lat[j] = 0.0;
    half_lat_deg[j] = half_lat[j] * deg;
  }
  // equatorial symmetry (mesh_mod.F90:225-237)
  for (int j = 1; j <= nlat; ++j)
    if (full_lat[j] > 0) {
      full_lat[j] = -full_lat[nlat - j + 1];
      full_lat_deg[j] = -full_lat_deg[nlat - j + 1];
    }
  for (int j = 1; j <= nhalf; ++j)
    if (half_lat[j] > 0) {
      half_lat[j] = -half_lat[nhalf - j + 1];
      half_lat_deg[j] = -half_lat_deg[nhalf - j + 1];
    }
  for (int j = 1; j <= nhalf; ++j) {
    half_cos_lat[j] = std::cos(half_lat[j]);
    half_sin_lat[j] = std::sin(half_lat[j]);
  }
  for (int j = 1; j <= nlat; ++j) {
    full_cos_lat[j] = std::cos(full_lat[j]);
    full_sin_lat[j] = std::sin(full_lat[j]);
  }
  full_cos_lat[1] = 0.0;
  full_sin_lat[1] = -1.0;
  full_cos_lat[nlat] = 0.0;
  full_sin_lat[nlat] = 1.0;

  // --- cell areas and the split of edge/vertex control volumes
  //     (mesh_mod.F90:269-377) ---
  for (RowTable *t : {&area_cell, &area_subcell1, &area_subcell2, &area_lon, &area_lon_west,
                      &area_lon_east, &area_lon_north, &area_lon_south, &de_lon, &le_lon})
    t->init(nlat, 0.0);
  for (RowTable *t : {&area_lat, &area_lat_west, &area_lat_east, &area_lat_north, &area_lat_south,
                      &area_vtx, &de_lat, &le_lat})
    t->init(nhalf, 0.0);
  const double r2 = radius * radius;
  for (int j = 1; j <= nlat; ++j) {
    if (j == 1) {
      area_cell[j] = r2 * dlon * (half_sin_lat[j] + 1.0);
      area_subcell2[j] = r2 * 0.5 * dlon * (half_sin_lat[j] + 1.0);
    } else if (j == nlat) {
      area_cell[j] = r2 * dlon * (1.0 - half_sin_lat[j - 1]);
      area_subcell1[j] = r2 * 0.5 * dlon * (1.0 - half_sin_lat[j - 1]);
    } else {
      area_cell[j] = r2 * dlon * (half_sin_lat[j] - half_sin_lat[j - 1]);
      area_subcell1[j] = r2 * 0.5 * dlon * (full_sin_lat[j] - half_sin_lat[j - 1]);
      area_subcell2[j] = r2 * 0.5 * dlon * (half_sin_lat[j] - full_sin_lat[j]);
      V3 t[3];
      t[0] = to_cartesian(full_lon[0], full_lat[j], radius);
      t[1] = to_cartesian(half_lon[0], half_lat[j - 1], radius);
      t[2] = to_cartesian(half_lon[0], half_lat[j], radius);
      area_lon_west[j] = (double)triangle_area(t, radius, pi, pi2);
      area_lon_east[j] = area_lon_west[j];
      area_lon[j] = area_lon_west[j] + area_lon_east[j];
      t[0] = to_cartesian(half_lon[0], half_lat[j], radius);
      t[1] = to_cartesian(full_lon[0], full_lat[j], radius);
      t[2] = to_cartesian(full_lon[1], full_lat[j], radius);
      area_lon_north[j] = (double)small_arc_triangle_area(t, radius, pi, pi2);
      t[0] = to_cartesian(half_lon[0], half_lat[j - 1], radius);
      t[1] = to_cartesian(full_lon[1], full_lat[j], radius);
      t[2] = to_cartesian(full_lon[0], full_lat[j], radius);
      area_lon_south[j] = (double)small_arc_triangle_area(t, radius, pi, pi2);
    }
  }
  for (int j = 1; j <= nhalf; ++j) {
    area_vtx[j] = r2 * dlon * (full_sin_lat[j + 1] - full_sin_lat[j]);
    V3 t[3];
    t[0] = to_cartesian(half_lon[0], half_lat[j], radius);
    t[1] = to_cartesian(full_lon[1], full_lat[j], radius);
    t[2] = to_cartesian(full_lon[1], full_lat[j + 1], radius);
    area_lat_west[j] = (double)triangle_area(t, radius, pi, pi2);
    area_lat_east[j] = area_lat_west[j];
    if (j == nhalf) {
      area_lat_north[j] = area_cell[j + 1];
    } else {
      t[0] = to_cartesian(full_lon[1], full_lat[j + 1], radius);
      t[1] = to_cartesian(half_lon[0], half_lat[j], radius);
      t[2] = to_cartesian(half_lon[1], half_lat[j], radius);
      area_lat_north[j] = (double)small_arc_triangle_area(t, radius, pi, pi2);
    }
    if (j == 1) {
      area_lat_south[j] = area_cell[j];
    } else {
      t[0] = to_cartesian(full_lon[1], full_lat[j], radius);
      t[1] = to_cartesian(half_lon[1], half_lat[j], radius);
      t[2] = to_cartesian(half_lon[0], half_lat[j], radius);
      area_lat_south[j] = (double)small_arc_triangle_area(t, radius, pi, pi2);
    }
    area_lat[j] = area_lat_north[j] + area_lat_south[j];
  }

  // --- edge lengths (mesh_mod.F90:379-395) ---
  for (int j = 2; j <= nlat - 1; ++j) {
    de_lon[j] = radius * full_cos_lat[j] * dlon;
    le_lon[j] = 2.0 * area_lon[j] / de_lon[j];
  }
  le_lon[1] = de_lon[1] = 0.0;
  le_lon[nlat] = de_lon[nlat] = 0.0;
  for (int j = 1; j <= nhalf; ++j) {
    le_lat[j] = radius * half_cos_lat[j] * dlon;
    de_lat[j] = 2.0 * area_lat[j] / le_lat[j];
  }

  // --- tangential-wind weights, 'classic' (mesh_mod.F90:417-427) ---
  for (RowTable *t : {&full_tangent_wgt1, &full_tangent_wgt2}) t->init(nlat, inf);
  for (RowTable *t : {&half_tangent_wgt1, &half_tangent_wgt2}) t->init(nhalf, inf);
  for (int j = 2; j <= nlat - 1; ++j) {
    full_tangent_wgt1[j] = le_lat[j - 1] / de_lon[j] * 0.25;
    full_tangent_wgt2[j] = le_lat[j] / de_lon[j] * 0.25;
  }
  for (int j = 1; j <= nhalf; ++j) {
    half_tangent_wgt1[j] = le_lon[j] / de_lat[j] * 0.25;
    half_tangent_wgt2[j] = le_lon[j + 1] / de_lat[j] * 0.25;
  }
  full_f.init(nlat, inf);
  half_f.init(nhalf, inf);
  for (int j = 1; j <= nlat; ++j) full_f[j] = 2.0 * c.omega * full_sin_lat[j];
  for (int j = 1; j <= nhalf; ++j) half_f[j] = 2.0 * c.omega * half_sin_lat[j];

  // --- vertical coordinate ---
  hyai.assign(nlev + 1, 0.0);
  hybi.assign(nlev + 1, 0.0);
  hyam.assign(nlev, 0.0);
  hybm.assign(nlev, 0.0);
  full_lev.assign(nlev, 0.0);
  half_lev.assign(nlev + 1, 0.0);
  full_dlev.assign(nlev, 0.0);
  half_dlev.assign(nlev + 1, 0.0);
  local_ptop = 0.0;
  ptop_nml = c.ptop;
  bool ptop_override = false;
  if (c.baroclinic) {
    const float *A = nullptr, *B = nullptr;
    switch (c.vert_coord_template) {
      case GMC_VCOORD_TEST_L26: A = kTestL26A; B = kTestL26B; ptop_override = true; break;
      case GMC_VCOORD_WRF_L32: A = kWrfL32A; B = kWrfL32B; local_ptop = c.ptop; break;
      case GMC_VCOORD_WRF_L64: A = kWrfL64A; B = kWrfL64B; local_ptop = c.ptop; break;
    }
    for (int k = 0; k <= nlev; ++k) {
      hyai[k] = (double)A[k];
      hybi[k] = (double)B[k];
    }
    for (int k = 0; k < nlev; ++k) {
      hyam[k] = 0.5 * (hyai[k] + hyai[k + 1]);
      hybm[k] = 0.5 * (hybi[k] + hybi[k + 1]);
    }
    if (ptop_override) ptop_nml = c.hybrid_coord_p0 * hyai[0];   // hybrid_coord_test_l26 :145
    for (int k = 0; k < nlev; ++k) full_lev[k] = hyam[k] + hybm[k];
    for (int k = 0; k <= nlev; ++k) half_lev[k] = hyai[k] + hybi[k];
    for (int k = 0; k < nlev; ++k) full_dlev[k] = half_lev[k + 1] - half_lev[k];
    for (int k = 1; k < nlev; ++k) half_dlev[k] = full_lev[k] - full_lev[k - 1];
    half_dlev[0] = full_lev[0] - half_lev[0];
    half_dlev[nlev] = half_lev[nlev] - full_lev[nlev - 1];
  } else {
    full_dlev[0] = 1.0;
  }

  // --- polar filters (filter_types_mod.F90:49-147) ---
  auto init_filter = [&](Filter &f, int type) {
    f.ngrid_full.assign(nlat, 0);
    f.ngrid_half.assign(nhalf, 0);
    f.width_full.assign(nlat, 0.0);
    f.width_half.assign(nhalf, 0.0);
    f.wgt_full.assign(nlat, {});
    f.wgt_half.assign(nhalf, {});
    const double dt = c.dt_dyn;
    if (c.max_wave_speed > 0) {
      for (int j = 2; j <= nlat - 1; ++j) {
        double dx = de_lon[j];
        if (dx > 0) {
          double cfl = c.max_wave_speed * dt / dx;
          double w = c.filter_coef_a * cfl / c.max_cfl *
                     (c.filter_coef_c * (std::tanh(90 - std::fabs(full_lat_deg[j])) - 1) + 1);
          int n = (int)std::ceil(w) + 2;
          if (n % 2 == 0) n = n + 1;
          f.width_full[j - 1] = w;
          f.ngrid_full[j - 1] = n;
        }
      }
      for (int j = 1; j <= nhalf; ++j) {
        double dx = le_lat[j];
        if (dx > 0) {
          double cfl = c.max_wave_speed * dt / dx;
          double w = c.filter_coef_a * cfl / c.max_cfl *
                     (c.filter_coef_c * (std::tanh(90 - std::fabs(half_lat_deg[j])) - 1) + 1);
          int n = (int)std::ceil(w) + 2;
          if (n % 2 == 0) n = n + 1;
          f.width_half[j - 1] = w;
          f.ngrid_half[j - 1] = n;
        }
      }
    }
    auto shrink = [](int &n, double w) {
      // Fortran real-to-integer assignment truncates.  A non-finite factor
      // (lat0 = 80 degrees makes exp_two_values divide by zero) leaves the
      // row unfiltered instead of producing a garbage tap count.
      double x = w * n;
      n = std::isfinite(x) && x < 1e6 ? (int)x : 1;
      if (n % 2 == 0) n = n + 1;
    };
    for (int j = 2; j <= nlat - 1; ++j) {
      int &n = f.ngrid_full[j - 1];
      if (n <= 1) continue;
      if (type == 1) {
        double w = c.filter_coef_d;
        shrink(n, w);
        f.width_full[j - 1] *= w;
      } else if (type == 2) {
        double lat0 = -full_lat_deg[2];
        double w = exp_two_values(c.filter_coef_e, c.filter_coef_d, lat0, 80.0, std::fabs(full_lat_deg[j]));
        shrink(n, w);
        f.width_full[j - 1] = w * f.width_full[j - 1];
      }
      f.wgt_full[j - 1] = gaussian_weights(f.width_full[j - 1], n, c.filter_coef_b, pi2);
    }
    for (int j = 1; j <= nhalf; ++j) {
      int &n = f.ngrid_half[j - 1];
      if (n <= 1) continue;
      if (type == 1) {
        double w = c.filter_coef_d;
        shrink(n, w);
        f.width_half[j - 1] *= w;
      } else if (type == 2) {
        double lat0 = -half_lat_deg[1];
        double w = exp_two_values(c.filter_coef_e, c.filter_coef_d, lat0, 80.0, std::fabs(half_lat_deg[j]));
        shrink(n, w);
        f.width_half[j - 1] = w * f.width_half[j - 1];
      }
      f.wgt_half[j - 1] = gaussian_weights(f.width_half[j - 1], n, c.filter_coef_b, pi2);
    }
  };
  init_filter(big, 0);
  init_filter(small1, 1);
  init_filter(small2, 2);

  // halo width rule (process_mod.F90:208-213)
  int max_hw = 2;
  for (int j = 1; j <= nhalf; ++j) max_hw = std::max(max_hw, (big.ngrid_half[j - 1] - 1) / 2);
  lon_halo_width = std::max(max_hw, c.lon_halo_width);

  // divergence damping coefficients (div_damp_mod.F90:41-76)
  div_c_lon.assign((size_t)nlev * nlat, 0.0);
  div_c_lat.assign((size_t)nlev * nhalf, 0.0);
  if (c.use_div_damp && c.div_damp_order == 4) {
    for (int k = 1; k <= nlev; ++k) {
      for (int j = 2; j <= nlat - 1; ++j)
        div_c_lon[(size_t)(k - 1) * nlat + (j - 1)] = c.div_damp_coef4 * (le_lon[j] * le_lon[j]) * (de_lon[j] * de_lon[j]);
      for (int j = 1; j <= nhalf; ++j)
        div_c_lat[(size_t)(k - 1) * nhalf + (j - 1)] = c.div_damp_coef4 * (le_lat[j] * le_lat[j]) * (de_lat[j] * de_lat[j]);
    }
  } else if (c.use_div_damp) {
    for (int k = 1; k <= nlev; ++k) {
      double amp = 1.0;
      if (c.baroclinic) {
        // vert_coord_calc_ph(k, p0) = hyam(k) (p0h - ptop_local) + hybm(k) (p0 - ptop_local) + ptop_local
        double ph = hyam[k - 1] * (c.hybrid_coord_p0 - local_ptop) + hybm[k - 1] * (c.p0 - local_ptop) + local_ptop;
        amp = std::max(1.0, 8 * (1 + std::tanh(std::log(ptop_nml / ph))));
      }
      for (int j = 2; j <= nlat - 1; ++j)
        div_c_lon[(size_t)(k - 1) * nlat + (j - 1)] =
            c.baroclinic ? c.div_damp_coef2 * amp * le_lon[j] * de_lon[j] : c.div_damp_coef2 * le_lon[j] * de_lon[j];
      for (int j = 1; j <= nhalf; ++j)
        div_c_lat[(size_t)(k - 1) * nhalf + (j - 1)] =
            c.baroclinic ? c.div_damp_coef2 * amp * le_lat[j] * de_lat[j] : c.div_damp_coef2 * le_lat[j] * de_lat[j];
    }
  }

  // zonal smoother weights (lon_damp_mod.F90:43-68)
  lon_damp_wgt_full.assign(nlat, 0.0);
  lon_damp_wgt_half.assign(nhalf, 0.0);
  {
    const double lat_cut = 80;
    double lat0 = -full_lat_deg[2];
    for (int j = 2; j <= nlat - 1; ++j) {
      double lat = std::fabs(full_lat_deg[j]);
      double w = std::exp((lat0 - lat) * (lat0 - lat) * std::log(1.0e-3) / ((lat0 - lat_cut) * (lat0 - lat_cut)));
      lon_damp_wgt_full[j - 1] = (w < 1.0e-6 || !std::isfinite(w)) ? 0.0 : w;
    }
    lat0 = -half_lat_deg[1];
    for (int j = 1; j <= nhalf; ++j) {
      double lat = std::fabs(half_lat_deg[j]);
      double w = std::exp((lat0 - lat) * (lat0 - lat) * std::log(1.0e-3) / ((lat0 - lat_cut) * (lat0 - lat_cut)));
      lon_damp_wgt_half[j - 1] = (w < 1.0e-6 || !std::isfinite(w)) ? 0.0 : w;
    }
  }
  return "";
}

const RowTable *Grid::metric(const std::string &n) const {
  struct E { const char *name; const RowTable *t; };
  const E tab[] = {
      {"full_lat", &full_lat}, {"half_lat", &half_lat}, {"full_lat_deg", &full_lat_deg},
      {"half_lat_deg", &half_lat_deg}, {"full_cos_lat", &full_cos_lat}, {"full_sin_lat", &full_sin_lat},
      {"half_cos_lat", &half_cos_lat}, {"half_sin_lat", &half_sin_lat}, {"area_cell", &area_cell},
      {"area_subcell1", &area_subcell1}, {"area_subcell2", &area_subcell2}, {"area_lon", &area_lon},
      {"area_lon_west", &area_lon_west}, {"area_lon_east", &area_lon_east},
      {"area_lon_north", &area_lon_north}, {"area_lon_south", &area_lon_south}, {"area_lat", &area_lat},
      {"area_lat_west", &area_lat_west}, {"area_lat_east", &area_lat_east},
      {"area_lat_north", &area_lat_north}, {"area_lat_south", &area_lat_south}, {"area_vtx", &area_vtx},
      {"de_lon", &de_lon}, {"le_lon", &le_lon}, {"de_lat", &de_lat}, {"le_lat", &le_lat},
      {"full_f", &full_f}, {"half_f", &half_f}, {"full_tangent_wgt1", &full_tangent_wgt1},
      {"full_tangent_wgt2", &full_tangent_wgt2}, {"half_tangent_wgt1", &half_tangent_wgt1},
      {"half_tangent_wgt2", &half_tangent_wgt2}};
  for (const E &e : tab)
    if (n == e.name) return e.t;
  return nullptr;
}

// ---------------------------------------------------------------------------
// Seeded synthetic initial states.
// ---------------------------------------------------------------------------
uint64_t SplitMix64::next() {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double SplitMix64::uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
double SplitMix64::normal() {
  double u1 = uniform(), u2 = uniform();
  if (u1 < 1e-300) u1 = 1e-300;
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
}

namespace {

// Fully normalised associated Legendre functions P_l^m(x), l,m <= 8.
void legendre(double x, double P[9][9]) {
  double s = std::sqrt(std::max(0.0, 1 - x * x));
  for (int l = 0; l < 9; ++l)
    for (int m = 0; m < 9; ++m) P[l][m] = 0;
  P[0][0] = 1;
  for (int m = 1; m <= 8; ++m) P[m][m] = std::sqrt((2.0 * m + 1) / (2.0 * m)) * s * P[m - 1][m - 1] * (m == 1 ? std::sqrt(2.0) : 1.0);
  for (int m = 0; m < 8; ++m) P[m + 1][m] = std::sqrt(2.0 * m + 3) * x * P[m][m];
  for (int m = 0; m <= 8; ++m)
    for (int l = m + 2; l <= 8; ++l) {
      double a = std::sqrt((4.0 * l * l - 1) / ((double)l * l - (double)m * m));
      double b = std::sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1));
      P[l][m] = a * (x * P[l - 1][m] - b * P[l - 2][m]);
    }
}

struct Harmonics {
  double a[9][9], b[9][9], scale = 1;
  double eval(double lon, double lat) const {
    double P[9][9];
    legendre(std::sin(lat), P);
    double s = 0;
    for (int l = 1; l <= 8; ++l)
      for (int m = 0; m <= l; ++m) s += (a[l][m] * std::cos(m * lon) + b[l][m] * std::sin(m * lon)) * P[l][m];
    return s * scale;
  }
};

double great_circle(double lon1, double lat1, double lon2, double lat2) {
  double c = std::sin(lat1) * std::sin(lat2) + std::cos(lat1) * std::cos(lat2) * std::cos(lon1 - lon2);
  c = std::min(1.0, std::max(-1.0, c));
  return std::acos(c);
}

}  // namespace

std::string make_ic(const Grid &g, int kind, uint64_t seed, double noise_k, double *u_lon,
                    double *v_lat, double *pt_or_gz, double *phs, double *gzs, double *q) {
  const gmc_config &c = g.cfg;
  const int nlon = g.nlon, nlat = g.nlat, nhalf = g.nhalf, nlev = g.nlev;
  const double pi = g.pi;
  SplitMix64 rng(seed);
  if (kind == 1) {
    if (c.baroclinic) return "kind 1 is the shallow-water state";
    // Free-surface height: 8000 m plus a random sum of spherical harmonics of
    // degree 1..8 rescaled to a 100 m maximum over the cell centres.
    Harmonics h;
    for (int l = 0; l < 9; ++l)
      for (int m = 0; m < 9; ++m) {
        h.a[l][m] = (m <= l && l >= 1) ? rng.normal() : 0.0;
        h.b[l][m] = (m <= l && l >= 1 && m > 0) ? rng.normal() : 0.0;
      }
    double amax = 0;
    for (int j = 1; j <= nlat; ++j)
      for (int i = 1; i <= nlon; ++i) amax = std::max(amax, std::fabs(h.eval(g.full_lon[i - 1], g.full_lat[j])));
    h.scale = 100.0 / amax;
    const double lon_c = rng.uniform() * 2 * pi;
    const double lat_c = (rng.uniform() * 2 - 1) * pi / 3;
    const double sigma = 20.0 * pi / 180.0;
    auto hill = [&](double lon, double lat) {
      double r = great_circle(lon, lat, lon_c, lat_c);
      return 2000.0 * std::exp(-(r * r) / (sigma * sigma));
    };
    auto eta = [&](double lon, double lat) { return 8000.0 + h.eval(lon, lat); };
    const double lat_taper = 5.0 * pi / 180.0;
    const double d = 1.0e-6;
    for (int j = 1; j <= nlat; ++j)
      for (int i = 1; i <= nlon; ++i) {
        size_t o = (size_t)(j - 1) * nlon + (i - 1);
        double lon = g.full_lon[i - 1], lat = g.full_lat[j];
        if (pt_or_gz) pt_or_gz[o] = c.g * eta(lon, lat);
        if (gzs) gzs[o] = c.g * hill(lon, lat);
      }
    // Geostrophic winds u = -(g/f) deta/dy, v = (g/f) deta/dx, tapered to zero
    // within a few degrees of the equator where f vanishes.
    auto geo_factor = [&](double lat) {
      if (std::fabs(lat) < 1.0e-10) return 0.0;
      double f = 2.0 * c.omega * std::sin(lat);
      double taper = 1.0 - std::exp(-(lat / lat_taper) * (lat / lat_taper));
      return c.g / f * taper;
    };
    if (u_lon)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double lon = g.half_lon[i - 1], lat = g.full_lat[j];
          double val = 0;
          if (j != 1 && j != nlat) {
            double dedy = (eta(lon, lat + d) - eta(lon, lat - d)) / (2 * d * c.radius);
            val = -geo_factor(lat) * dedy;
          }
          u_lon[(size_t)(j - 1) * nlon + (i - 1)] = val;
        }
    if (v_lat)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double lon = g.full_lon[i - 1], lat = g.half_lat[j];
          double dedx = (eta(lon + d, lat) - eta(lon - d, lat)) / (2 * d * c.radius * std::cos(lat));
          v_lat[(size_t)(j - 1) * nlon + (i - 1)] = geo_factor(lat) * dedx;
        }
    return "";
  }
  if (kind == 2) {
    if (!c.baroclinic) return "kind 2 is the baroclinic state";
    // Isothermal (300 K) atmosphere with a barotropic zonal jet
    // u = 35 sin^2(2 lat) m/s held by a surface pressure in gradient-wind
    // balance, (Rd T / a) dln(ps)/dlat = -(f u + u^2 tan(lat) / a), scaled to a
    // global mean of 1000 hPa; seeded N(0, noise_k) temperature noise per cell.
    const double kappa = c.Rd / c.cpd, T0 = 300.0, a = c.radius;
    auto jet = [](double lat) { double s = std::sin(2.0 * lat); return 35.0 * s * s; };
    auto lnps = [&](double lat) {   // integral from the south pole, Simpson rule
      const int n = 2000;
      double h = (lat + pi / 2) / n, acc = 0;
      for (int t = 0; t <= n; ++t) {
        double x = -pi / 2 + t * h;
        double u = jet(x);
        double f = 2.0 * c.omega * std::sin(x);
        double integrand = (std::fabs(std::cos(x)) < 1e-12) ? 0.0 : (f * u + u * u * std::tan(x) / a);
        double wgt = (t == 0 || t == n) ? 1 : (t % 2 ? 4 : 2);
        acc += wgt * integrand;
      }
      return -(a / (c.Rd * T0)) * acc * h / 3;
    };
    std::vector<double> ps_row(nlat + 1);
    double num = 0, den = 0;
    for (int j = 1; j <= nlat; ++j) {
      ps_row[j] = std::exp(lnps(g.full_lat[j]));
      num += ps_row[j] * g.area_cell[j];
      den += g.area_cell[j];
    }
    const double scale = 1.0e5 / (num / den);
    for (int j = 1; j <= nlat; ++j) ps_row[j] *= scale;
    for (int j = 1; j <= nlat; ++j)
      for (int i = 1; i <= nlon; ++i) {
        size_t o = (size_t)(j - 1) * nlon + (i - 1);
        if (phs) phs[o] = ps_row[j];
        if (gzs) gzs[o] = 0.0;
      }
    const double p0h = c.hybrid_coord_p0, pt_top = g.local_ptop;
    for (int k = 0; k < nlev; ++k)
      for (int j = 1; j <= nlat; ++j) {
        double pl0 = g.hyai[k] * (p0h - pt_top) + g.hybi[k] * (ps_row[j] - pt_top) + pt_top;
        double pl1 = g.hyai[k + 1] * (p0h - pt_top) + g.hybi[k + 1] * (ps_row[j] - pt_top) + pt_top;
        double ph = 0.5 * (pl0 + pl1);
        for (int i = 1; i <= nlon; ++i) {
          size_t o = ((size_t)k * nlat + (j - 1)) * nlon + (i - 1);
          double T = T0 + noise_k * rng.normal();
          if (pt_or_gz) pt_or_gz[o] = T * std::pow(c.p0 / ph, kappa);
          if (u_lon) u_lon[o] = (j == 1 || j == nlat) ? 0.0 : jet(g.full_lat[j]);
        }
      }
    if (v_lat)
      for (size_t o = 0; o < (size_t)nlev * nhalf * nlon; ++o) v_lat[o] = 0.0;
    if (q) {
      for (int t = 0; t < c.ntracer; ++t) {
        double lon_c = rng.uniform() * 2 * pi;
        double lat_c = (rng.uniform() * 2 - 1) * pi / 3;
        double sigma = (10.0 + 10.0 * rng.uniform()) * pi / 180.0;
        double kc = 0.25 * nlev + 0.5 * nlev * rng.uniform();
        double kw = std::max(1.0, nlev / 6.0);
        for (int k = 0; k < nlev; ++k)
          for (int j = 1; j <= nlat; ++j)
            for (int i = 1; i <= nlon; ++i) {
              double r = great_circle(g.full_lon[i - 1], g.full_lat[j], lon_c, lat_c) / sigma;
              double z = (k + 0.5 - kc) / kw;
              q[(((size_t)t * nlev + k) * nlat + (j - 1)) * nlon + (i - 1)] = std::exp(-r * r - z * z);
            }
      }
    }
    return "";
  }
  return "unknown initial-state kind";
}

}  // namespace gmc
