// Host-side grid set-up for the GMCORE latitude-longitude C-grid.
//
// Everything here runs once at context creation, on the host, in FP64 (the
// spherical-triangle areas in IEEE binary128).  It produces the 1-D metric
// tables, hybrid coefficients and polar-filter weights that the device step
// reads from constant/global memory.  The reference computes the same tables
// in its Fortran initialisation:
//   mesh metrics      src/dynamics/mesh_mod.F90:134-447
//   triangle areas    src/utils/sphere_geometry_mod.F90:302-448
//   vertical levels   src/dynamics/vert_coord/hybrid_coord_mod.F90:34-135,
//                     src/dynamics/vert_coord/vert_coord_mod.F90:84-101
//   polar filters     src/dynamics/filter_types_mod.F90:31-147
//   halo width rule   src/utils/process_mod.F90:208-213
//   zonal smoother    src/dynamics/damp/lon_damp_mod.F90:43-68
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "gmcore_gpu.h"

namespace gmc {

// Row tables indexed by latitude.  Full latitudes use j = 1..nlat and half
// latitudes j = 1..nlat-1 (the reference's Fortran indices); slot 0 and the
// slot past the last row hold the values the reference keeps in its halo
// (0 for lengths and areas), so stencils that touch j-1 or j+1 at the ends
// read what the reference reads.
struct RowTable {
  std::vector<double> v;   // index j + 1 (so v[0] is j = -1)
  double &operator[](int j) { return v[j + 1]; }
  double operator[](int j) const { return v[j + 1]; }
  void init(int n, double fill) { v.assign(n + 4, fill); }
};

struct Filter {
  // Per-row tap counts and normalised Gaussian weights
  // (filter_types_mod.F90:31-47, 67-145).  Rows with ngrid <= 1 are copied.
  std::vector<int> ngrid_full;                 // j = 1..nlat   -> [j-1]
  std::vector<int> ngrid_half;                 // j = 1..nlat-1 -> [j-1]
  std::vector<std::vector<double>> wgt_full;   // [j-1][0..n-1]
  std::vector<std::vector<double>> wgt_half;
  std::vector<double> width_full, width_half;
  int max_taps() const;
};

struct Grid {
  gmc_config cfg;
  int nlon, nlat, nhalf, nlev;
  int lon_halo_width;   // process_mod.F90:208-213
  double pi, pi2, pi05, deg, dlon;

  std::vector<double> full_lon, half_lon;   // i = 1..nlon -> [i-1]
  RowTable full_lat, half_lat, full_lat_deg, half_lat_deg;
  RowTable full_cos_lat, full_sin_lat, half_cos_lat, half_sin_lat;
  RowTable area_cell, area_subcell1, area_subcell2;
  RowTable area_lon, area_lon_west, area_lon_east, area_lon_north, area_lon_south;
  RowTable area_lat, area_lat_west, area_lat_east, area_lat_north, area_lat_south;
  RowTable area_vtx;
  RowTable de_lon, le_lon, de_lat, le_lat;
  RowTable full_f, half_f;
  RowTable full_tangent_wgt1, full_tangent_wgt2, half_tangent_wgt1, half_tangent_wgt2;

  // Vertical coordinate (hybrid sigma-p).  Arrays are 1-based in the
  // reference; here [k-1].
  std::vector<double> hyai, hybi, hyam, hybm;     // nlev+1, nlev+1, nlev, nlev
  std::vector<double> full_lev, half_lev;         // eta
  std::vector<double> full_dlev, half_dlev;
  double local_ptop = 0.0;
  double ptop_nml = 0.0;   // namelist ptop after the vertical template (test_l* set it to p0 hyai(1))

  // Divergence-damping coefficients c_lon(j,k), c_lat(j,k) of order 2
  // (div_damp_mod.F90:41-64), [(k-1) * nlat + (j-1)] and [(k-1) * nhalf + (j-1)].
  std::vector<double> div_c_lon, div_c_lat;

  Filter big, small1, small2;
  std::vector<double> lon_damp_wgt_full;   // lon_damp_mod.F90:55-60, [j-1]
  std::vector<double> lon_damp_wgt_half;   // [j-1]

  // Returns an empty string on success, else a message.
  std::string build(const gmc_config &c);
  const RowTable *metric(const std::string &name) const;
};

// SplitMix64 counter-based generator (public-domain algorithm by S. Vigna):
// seeded synthetic inputs are bit-identical on every machine.
struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next();
  double uniform();          // [0, 1)
  double normal();           // Box-Muller
};

std::string make_ic(const Grid &g, int kind, uint64_t seed, double noise_k,
                    double *u_lon, double *v_lat, double *pt_or_gz, double *phs,
                    double *gzs, double *q);

std::string validate_config(const gmc_config &c);

}  // namespace gmc
