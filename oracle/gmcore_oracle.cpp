// ORACLE -- test infrastructure only.
//
// CPU FP64 restatement of the GMCORE dynamics step (the reference path
// time_integrate, src/dynamics/gmcore_mod.F90:577-591) used as the parity
// checker for the GPU library and as the timed CPU baseline.  It is never
// linked into, called from or shipped with the product library.
//
// It keeps the reference's own index space: every field is an array with
// Fortran lower bounds (longitude halo = lon_halo_width, latitude halo 2,
// level halo 2 on full levels), and halo exchange reproduces the single-rank
// behaviour of fill_halo (src/utils/parallel_mod.F90:318-418, 464-565 with the
// subarrays of src/utils/halo_mod.F90:46-267): periodic west/east copies over
// the interior rows, pole rows mirrored across the pole with the interior
// columns rotated by nlon/2 and the longitude-halo columns left unrotated.
// Loop order and arithmetic order follow the Fortran statements so that the
// parity build (-O2 -fno-fast-math -ffp-contract=off) evaluates the same
// expressions.  Values the reference leaves uninitialised (the halo of a
// filter's work row) are set to NaN here so any read of them shows up.
//
// Parity status: the reference cannot be compiled (no Fortran compiler, MPI
// or netCDF, and its git submodules are empty), so this restatement is pinned
// by the reference's own known answers -- area identities of
// debug_check_areas, mass conservation of diagnose, the steady geostrophic
// flow test -- and not by outputs of the reference binary: parity unpinned
// against the binary itself.
//
// Mesh metrics, polar-filter weights and hybrid coefficients are inputs of
// the step; they come from the host set-up code (gmcore_gb300/csrc/grid.cpp).

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "grid.hpp"

namespace orc {

static const double kNaN = std::numeric_limits<double>::quiet_NaN();

// Fortran-style array with explicit bounds, column-major.
struct Arr {
  std::vector<double> d;
  int lb0 = 0, ub0 = -1, lb1 = 0, ub1 = -1, lb2 = 0, ub2 = -1;
  long n0 = 0, n1 = 0;
  void alloc(int l0, int u0, int l1, int u1, int l2, int u2) {
    lb0 = l0; ub0 = u0; lb1 = l1; ub1 = u1; lb2 = l2; ub2 = u2;
    n0 = u0 - l0 + 1; n1 = u1 - l1 + 1;
    d.assign((size_t)n0 * n1 * (u2 - l2 + 1), 0.0);
  }
  bool ok() const { return !d.empty(); }
  inline double &operator()(int i, int j, int k) {
    return d[(size_t)(i - lb0) + (size_t)n0 * ((size_t)(j - lb1) + (size_t)n1 * (size_t)(k - lb2))];
  }
  inline double operator()(int i, int j, int k) const {
    return d[(size_t)(i - lb0) + (size_t)n0 * ((size_t)(j - lb1) + (size_t)n1 * (size_t)(k - lb2))];
  }
};

static inline double fsign(double a, double b) { return std::copysign(std::fabs(a), b); }
static inline double fmin3(double a, double b, double c) { return std::fmin(std::fmin(a, b), c); }
static inline double fmax3(double a, double b, double c) { return std::fmax(std::fmax(a, b), c); }

struct Error {
  int code = 0;
  std::string msg;
  void set(int c, const std::string &m) {
#pragma omp critical(orc_error)
    {
      if (code == 0) { code = c; msg = m; }
    }
  }
};

// ---------------------------------------------------------------------------
struct Mesh {
  const gmc::Grid *g = nullptr;
  int nlon, nlat, nhalf, nlev, hx;
  // bounds (mesh_common_init, mesh_mod.F90:586-609)
  int lon_lb, lon_ub;            // full and half lon share bounds
  int flat_lb, flat_ub, hlat_lb, hlat_ub;
  int flev_lb, flev_ub, hlev_lb, hlev_ub;
  double dlon;
  void init(const gmc::Grid *grid) {
    g = grid;
    nlon = g->nlon; nlat = g->nlat; nhalf = g->nhalf; nlev = g->nlev; hx = g->lon_halo_width;
    lon_lb = 1 - hx; lon_ub = nlon + hx;
    flat_lb = -1; flat_ub = nlat + 2; hlat_lb = -1; hlat_ub = nhalf + 2;
    flev_lb = -1; flev_ub = nlev + 2; hlev_lb = 1; hlev_ub = nlev + 1;
    dlon = g->dlon;
  }
  // half_lon(i) for any i in the halo range (mesh_mod.F90:181-186)
  double half_lon(int i) const { double f = 0.0 + (i - 1) * dlon; return f + 0.5 * dlon; }
};

enum Loc { CELL, LON, LAT, VTX };

struct Fields {
  const Mesh *m;
  void cell3(Arr &a) { a.alloc(m->lon_lb, m->lon_ub, m->flat_lb, m->flat_ub, m->flev_lb, m->flev_ub); }
  void lon3(Arr &a) { cell3(a); }
  void lat3(Arr &a) { a.alloc(m->lon_lb, m->lon_ub, m->hlat_lb, m->hlat_ub, m->flev_lb, m->flev_ub); }
  void vtx3(Arr &a) { lat3(a); }
  void lev3(Arr &a) { a.alloc(m->lon_lb, m->lon_ub, m->flat_lb, m->flat_ub, m->hlev_lb, m->hlev_ub); }
  void levlon3(Arr &a) { lev3(a); }
  void levlat3(Arr &a) { a.alloc(m->lon_lb, m->lon_ub, m->hlat_lb, m->hlat_ub, m->hlev_lb, m->hlev_ub); }
  void cell2(Arr &a) { a.alloc(m->lon_lb, m->lon_ub, m->flat_lb, m->flat_ub, 1, 1); }
};

struct State {
  Arr u_lon, v_lon, u_f, u_lat, v_lat, v_f, we_lev, we_lev_lon, we_lev_lat, gz, gz_lev, m, m_vtx, m_lon,
      m_lat, m_lev, mfx_lon, mfy_lon, mfy_lat, mfx_lat, pv, pv_lon, pv_lat, ke, pt, ptf_lon, ptf_lat,
      ptf_lev, t, ph, ph_lev, ph_exn_lev, phs, phs_f, vor, gz_f, div, div2;
  Arr smag_t, smag_s, kmh_lon, kmh_lat, smag_dudt, smag_dvdt;   // smag_damp_run working arrays
};

struct Tend {
  Arr du, dv, dgz, dpt, dphs, qhv, qhu, dkedlon, dkedlat, dmfdlon, dmfdlat, dptfdlon, dptfdlat, dptfdlev,
      pgf_lon, pgf_lat, wedudlev, wedvdlev;
  bool update_u = false, update_v = false, update_gz = false, update_pt = false, update_phs = false;
  void reset_flags() { update_u = update_v = update_gz = update_pt = update_phs = false; }
};

struct Batch {
  bool dynamic = false;
  int nstep = 0, uv_step = 0, we_step = 0, mf_step = 0, old_idx = 0, new_idx = 1;
  double dt = 0;
  Arr old_m, mfx, mfy, m_lev, u, v, we, cflx, cfly, cflz, divx, divy, qx, qy, qlx, qly, dqx, dqy, q6x, q6y;
  std::vector<Arr> q[2];
  Arr qmf_lon, qmf_lat, qmf_lev;
};

// ---------------------------------------------------------------------------
struct Model {
  gmc::Grid grid;
  Mesh mesh;
  gmc_config cfg;
  bool baroclinic, hydrostatic;
  double Rd_o_cpd;
  State state[3];
  Tend tend[3];
  Arr gzs;
  Batch mass;          // adv_batch_mass (dynamic)
  Batch tracers;       // one tracer batch (static)
  bool has_tracers = false;
  int old_i = 0, new_i = 1;
  long time_step = 0;
  double alert_last_time = 0, curr_time = 0;   // tracer alert (time_mod.F90:210-291)
  Error err;

  const gmc::Grid &G() const { return grid; }

  // ------------------------------------------------------------------------
  // fill_halo (parallel_mod.F90:464-565) for one rank that owns both poles.
  void fill_halo(Arr &a, bool full_lat, bool west = true, bool east = true, bool south = true,
                 bool north = true) {
    const int nlon = mesh.nlon, hx = mesh.hx;
    const int nrow = full_lat ? mesh.nlat : mesh.nhalf;
    // West/east: rows full_lat 1..nlat, or half_lat 1..nhalf+1 (halo_mod.F90:95-106).
    const int we_j0 = 1, we_j1 = full_lat ? mesh.nlat : mesh.nhalf + 1;
    for (int k = a.lb2; k <= a.ub2; ++k) {
      if (west)
        for (int j = we_j0; j <= we_j1; ++j)
          for (int i = 1 - hx; i <= 0; ++i) a(i, j, k) = a(i + nlon, j, k);
      if (east)
        for (int j = we_j0; j <= we_j1; ++j)
          for (int i = nlon + 1; i <= nlon + hx; ++i) a(i, j, k) = a(i - nlon, j, k);
    }
    const int half = nlon / 2;
    // Pole rows: copy the two rows next to the pole into the halo rows (all
    // columns), then rewrite the interior columns of the halo rows in reverse
    // row order with a half-ring rotation.
    auto pole = [&](int r1, int r2, int h1, int h2, bool reverse_to_h2_first) {
      for (int k = a.lb2; k <= a.ub2; ++k) {
        for (int i = a.lb0; i <= a.ub0; ++i) {
          a(i, h1, k) = a(i, r1, k);
          a(i, h2, k) = a(i, r2, k);
        }
        std::vector<double> t1(nlon + 1), t2(nlon + 1);
        for (int i = 1; i <= nlon; ++i) { t1[i] = a(i, h1, k); t2[i] = a(i, h2, k); }
        // south: row 0 <- t1 rotated, row -1 <- t2 rotated (h1=-1,h2=0);
        // north: row h1 <- t2 rotated, row h2 <- t1 rotated.
        for (int i = 1; i <= nlon; ++i) {
          int s = i <= half ? i + half : i - half;
          if (reverse_to_h2_first) {
            a(i, h2, k) = t1[s];
            a(i, h1, k) = t2[s];
          } else {
            a(i, h1, k) = t2[s];
            a(i, h2, k) = t1[s];
          }
        }
      }
    };
    if (south) {
      if (full_lat) pole(2, 3, -1, 0, true); else pole(1, 2, -1, 0, true);
    }
    if (north) {
      if (full_lat) pole(nrow - 2, nrow - 1, nrow + 1, nrow + 2, false);
      else pole(nrow - 1, nrow, nrow + 1, nrow + 2, false);
    }
  }

  // zonal_sum over i = 1..nlon (parallel_mod.F90:741-764, one rank)
  template <class F>
  double ring(F f) {
    double s = 0;
    for (int i = 1; i <= mesh.nlon; ++i) s = s + f(i);
    return s;
  }

  // ------------------------------------------------------------------------
  // Polar filters (filter_mod.F90:25-163).  x is filtered into y (or in place
  // when y == nullptr) over rows of the requested latitude kind.
  void filter(const gmc::Filter &f, Arr &x, Arr *y, bool full_lat, int k0, int k1) {
    const int nlon = mesh.nlon;
    const int nrow = full_lat ? mesh.nlat : mesh.nhalf;
#pragma omp parallel for schedule(dynamic)
    for (int k = k0; k <= k1; ++k) {
      std::vector<double> tmp(x.n0);
      for (int j = 1; j <= nrow; ++j) {
        int n = full_lat ? f.ngrid_full[j - 1] : f.ngrid_half[j - 1];
        if (n > 1) {
          const std::vector<double> &w = full_lat ? f.wgt_full[j - 1] : f.wgt_half[j - 1];
          int hn = (n - 1) / 2;
          for (size_t t = 0; t < tmp.size(); ++t) tmp[t] = kNaN;
          for (int i = 1; i <= nlon; ++i) {
            double s = 0;
            for (int t = 0; t < n; ++t) s = s + w[t] * x(i - hn + t, j, k);
            tmp[i - x.lb0] = s;
          }
          Arr &dst = y ? *y : x;
          for (int i = x.lb0; i <= x.ub0; ++i) dst(i, j, k) = tmp[i - x.lb0];
        } else if (y) {
          for (int i = x.lb0; i <= x.ub0; ++i) (*y)(i, j, k) = x(i, j, k);
        }
      }
    }
  }

  // ------------------------------------------------------------------------
  void alloc_state(State &s) {
    Fields F{&mesh};
    F.lon3(s.u_lon); F.lon3(s.v_lon); F.lon3(s.u_f);
    F.lat3(s.u_lat); F.lat3(s.v_lat); F.lat3(s.v_f);
    F.lev3(s.we_lev); F.levlon3(s.we_lev_lon); F.levlat3(s.we_lev_lat);
    F.cell3(s.gz); F.lev3(s.gz_lev); F.cell3(s.m); F.vtx3(s.m_vtx); F.lon3(s.m_lon); F.lat3(s.m_lat);
    F.lev3(s.m_lev); F.lon3(s.mfx_lon); F.lon3(s.mfy_lon); F.lat3(s.mfy_lat); F.lat3(s.mfx_lat);
    F.vtx3(s.pv); F.lon3(s.pv_lon); F.lat3(s.pv_lat); F.cell3(s.ke); F.cell3(s.pt);
    F.lon3(s.ptf_lon); F.lat3(s.ptf_lat); F.lev3(s.ptf_lev); F.cell3(s.t); F.cell3(s.ph);
    F.lev3(s.ph_lev); F.lev3(s.ph_exn_lev); F.cell2(s.phs); F.cell2(s.phs_f); F.vtx3(s.vor); F.cell3(s.div);
    F.cell3(s.div2);   // zero at allocation, pole rows never written (allocator_mod.F90:198)
    if (cfg.use_smag_damp) {   // state_mod.F90:185-191, zero at allocation
      F.cell3(s.smag_t); F.vtx3(s.smag_s); F.lon3(s.kmh_lon); F.lat3(s.kmh_lat);
      F.lon3(s.smag_dudt); F.lat3(s.smag_dvdt);
    }
    if (!baroclinic) F.cell3(s.gz_f);
  }
  void alloc_tend(Tend &t) {
    Fields F{&mesh};
    F.lon3(t.du); F.lat3(t.dv); F.cell3(t.dgz); F.cell3(t.dpt); F.cell2(t.dphs); F.lon3(t.qhv);
    F.lat3(t.qhu); F.lon3(t.dkedlon); F.lat3(t.dkedlat); F.cell3(t.dmfdlon); F.cell3(t.dmfdlat);
    F.cell3(t.dptfdlon); F.cell3(t.dptfdlat); F.cell3(t.dptfdlev); F.lon3(t.pgf_lon); F.lat3(t.pgf_lat);
    F.lon3(t.wedudlev); F.lat3(t.wedvdlev);
  }
  void alloc_batch(Batch &b, double dt, bool dynamic, int ntr) {
    Fields F{&mesh};
    b.dt = dt;
    b.dynamic = dynamic;
    b.nstep = (int)(dt / cfg.dt_dyn);
    b.uv_step = b.we_step = b.mf_step = 0;
    F.cell3(b.old_m); F.lon3(b.mfx); F.lat3(b.mfy); F.lev3(b.m_lev); F.lon3(b.u); F.lat3(b.v);
    F.lev3(b.we); F.lon3(b.cflx); F.lat3(b.cfly); F.lev3(b.cflz); F.cell3(b.divx); F.cell3(b.divy);
    F.cell3(b.qx); F.cell3(b.qy); F.cell3(b.qlx); F.cell3(b.qly); F.cell3(b.dqx); F.cell3(b.dqy);
    F.cell3(b.q6x); F.cell3(b.q6y);
    if (ntr > 0) {
      for (int s = 0; s < 2; ++s) {
        b.q[s].resize(ntr);
        for (int l = 0; l < ntr; ++l) F.cell3(b.q[s][l]);
      }
      F.lon3(b.qmf_lon); F.lat3(b.qmf_lat); F.lev3(b.qmf_lev);
    }
  }

  std::string init(const gmc_config &c) {
    gmc_config cc = c;
    if (!cc.baroclinic) cc.ke_scheme = 1;   // parse_namelist (namelist_mod.F90:229-233)
    if (!(cc.dt_adv > 0)) cc.dt_adv = cc.dt_dyn;
    std::string e = grid.build(cc);
    if (!e.empty()) return e;
    cfg = cc;
    mesh.init(&grid);
    baroclinic = cfg.baroclinic != 0;
    hydrostatic = baroclinic;
    Rd_o_cpd = cfg.Rd / cfg.cpd;
    for (int s = 0; s < 3; ++s) alloc_state(state[s]);
    for (int s = 0; s < 3; ++s) alloc_tend(tend[s]);
    Fields F{&mesh};
    F.cell2(gzs);
    alloc_batch(mass, cfg.dt_dyn, true, 0);
    has_tracers = baroclinic && cfg.ntracer > 0;
    if (has_tracers) alloc_batch(tracers, cfg.dt_adv, false, cfg.ntracer);
    old_i = 0; new_i = 1;
    time_step = 0;
    curr_time = 0;
    alert_last_time = -cfg.dt_adv;
    return "";
  }

  // ========================================================================
  // Operators (operators_mod.F90)
  // ========================================================================
  double ph_lev_of(int k, double phs) const {
    // hybrid_coord_calc_ph_lev (hybrid_coord_mod.F90:155-162)
    const double p0 = cfg.hybrid_coord_p0, pt = grid.local_ptop;
    return grid.hyai[k - 1] * (p0 - pt) + grid.hybi[k - 1] * (phs - pt) + pt;
  }

  void calc_ph(State &s) {   // operators_mod.F90:136-168
    const int nlon = mesh.nlon, nlat = mesh.nlat, nlev = mesh.nlev;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev + 1; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          s.ph_lev(i, j, k) = ph_lev_of(k, s.phs_f(i, j, 1));
          s.ph_exn_lev(i, j, k) = std::pow(s.ph_lev(i, j, k), Rd_o_cpd);
        }
    fill_halo(s.ph_exn_lev, true, false, true, false, true);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) s.ph(i, j, k) = 0.5 * (s.ph_lev(i, j, k) + s.ph_lev(i, j, k + 1));
    fill_halo(s.ph, true);
  }

  void calc_t(State &s) {   // operators_mod.F90:170-190, formula_mod.F90:24-31
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= mesh.nlev; ++k)
      for (int j = 1; j <= mesh.nlat; ++j)
        for (int i = 1; i <= mesh.nlon; ++i)
          s.t(i, j, k) = s.pt(i, j, k) * std::pow(s.ph(i, j, k) / cfg.p0, Rd_o_cpd);
  }

  void calc_m(State &s) {   // operators_mod.F90:471-543
    const int nlon = mesh.nlon, nlat = mesh.nlat, nlev = mesh.nlev, nhalf = mesh.nhalf;
    if (baroclinic) {
      #pragma omp parallel for schedule(static)
      for (int k = 1; k <= nlev; ++k)
        for (int j = 1; j <= nlat; ++j)
          for (int i = 1; i <= nlon; ++i) {
            s.m(i, j, k) = s.ph_lev(i, j, k + 1) - s.ph_lev(i, j, k);
            if (s.m(i, j, k) <= 0) err.set(GMC_ENONMONO, "The pressure levels are not monotonic!");
          }
      #pragma omp parallel for schedule(static)
      for (int k = 2; k <= nlev; ++k)
        for (int j = 1; j <= nlat; ++j)
          for (int i = 1; i <= nlon; ++i) s.m_lev(i, j, k) = s.ph(i, j, k) - s.ph(i, j, k - 1);
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          s.m_lev(i, j, 1) = s.ph(i, j, 1) - s.ph_lev(i, j, 1);
          s.m_lev(i, j, nlev + 1) = s.ph_lev(i, j, nlev + 1) - s.ph(i, j, nlev);
        }
      fill_halo(s.m_lev, true);
    } else {
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) s.m(i, j, 1) = (s.gz(i, j, 1) - gzs(i, j, 1)) / cfg.g;
    }
    fill_halo(s.m, true);
    const gmc::Grid &g = G();
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) s.m_lon(i, j, k) = (s.m(i, j, k) + s.m(i + 1, j, k)) * 0.5;
    fill_halo(s.m_lon, true);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) s.m_lat(i, j, k) = (s.m(i, j, k) + s.m(i, j + 1, k)) * 0.5;
    fill_halo(s.m_lat, false);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i)
          s.m_vtx(i, j, k) = ((s.m(i, j, k) + s.m(i + 1, j, k)) * g.area_subcell2[j] +
                              (s.m(i, j + 1, k) + s.m(i + 1, j + 1, k)) * g.area_subcell1[j + 1]) /
                             g.area_vtx[j];
  }

  // adv_batch_accum_uv_cell (adv_batch_mod.F90:218-377)
  void accum_uv_cell(Batch &b, Arr &u, Arr &v, double dt_) {
    const int nlon = mesh.nlon, nlat = mesh.nlat, nhalf = mesh.nhalf, nlev = mesh.nlev;
    const gmc::Grid &g = G();
    const double radius = cfg.radius;
    if (b.uv_step == 0) {
      b.u.d = u.d; b.v.d = v.d;
      if (!b.dynamic) b.uv_step = b.uv_step + 1;
    } else if (b.uv_step == b.nstep) {
      for (size_t n = 0; n < b.u.d.size(); ++n) b.u.d[n] = (b.u.d[n] + u.d[n]) / (b.nstep + 1);
      for (size_t n = 0; n < b.v.d.size(); ++n) b.v.d[n] = (b.v.d[n] + v.d[n]) / (b.nstep + 1);
      b.uv_step = 0;
    } else {
      for (size_t n = 0; n < b.u.d.size(); ++n) b.u.d[n] = b.u.d[n] + u.d[n];
      for (size_t n = 0; n < b.v.d.size(); ++n) b.v.d[n] = b.v.d[n] + v.d[n];
      b.uv_step = b.uv_step + 1;
    }
    if (b.uv_step != 0) return;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      for (int j = 2; j <= nlat - 1; ++j) {
        double dx = g.de_lon[j];
        double cl = g.full_cos_lat[j];
        for (int i = 1; i <= nlon; ++i) {
          double x0 = radius * mesh.half_lon(i) * cl;
          double u1 = b.u(i, j, k);
          double x1 = x0 + dt_ / 2 * u1;
          int l = (int)std::floor(i + (x1 - x0) / dx);
          double u2 = ((radius * mesh.half_lon(l + 1) * cl - x1) * b.u(l, j, k) +
                       (x1 - radius * mesh.half_lon(l) * cl) * b.u(l + 1, j, k)) / dx;
          double x2 = x0 + dt_ / 2 * u2;
          l = (int)std::floor(i + (x2 - x0) / dx);
          double u3 = ((radius * mesh.half_lon(l + 1) * cl - x2) * b.u(l, j, k) +
                       (x2 - radius * mesh.half_lon(l) * cl) * b.u(l + 1, j, k)) / dx;
          double x3 = x0 + dt_ * u3;
          l = (int)std::floor(i + (x3 - x0) / dx);
          double u4 = ((radius * mesh.half_lon(l + 1) * cl - x3) * b.u(l, j, k) +
                       (x3 - radius * mesh.half_lon(l) * cl) * b.u(l + 1, j, k)) / dx;
          b.cflx(i, j, k) = (u1 + 2 * u2 + 2 * u3 + u4) / 6 * dt_ / dx;
          if (std::fabs(b.cflx(i, j, k)) > mesh.hx) err.set(GMC_ECFL, "cflx exceeds mesh%lon_halo_width");
        }
      }
      for (int j = 1; j <= nhalf; ++j) {
        double dy = g.de_lat[j];
        for (int i = 1; i <= nlon; ++i) {
          double y0 = radius * g.half_lat[j];
          double v1 = b.v(i, j, k);
          double y1 = y0 + dt_ / 2 * v1;
          int l = (int)std::floor(j + (y1 - y0) / dy);
          double v2 = (l < 1 || l > nhalf - 1)
                          ? v1
                          : ((radius * g.half_lat[l + 1] - y1) * b.v(i, l, k) +
                             (y1 - radius * g.half_lat[l]) * b.v(i, l + 1, k)) / dy;
          double y2 = y0 + dt_ / 2 * v2;
          l = (int)std::floor(j + (y2 - y0) / dy);
          double v3 = (l < 1 || l > nhalf - 1)
                          ? v1
                          : ((radius * g.half_lat[l + 1] - y2) * b.v(i, l, k) +
                             (y2 - radius * g.half_lat[l]) * b.v(i, l + 1, k)) / dy;
          double y3 = y0 + dt_ * v3;
          l = (int)std::floor(j + (y3 - y0) / dy);
          double v4 = (l < 1 || l > nhalf - 1)
                          ? v1
                          : ((radius * g.half_lat[l + 1] - y3) * b.v(i, l, k) +
                             (y3 - radius * g.half_lat[l]) * b.v(i, l + 1, k)) / dy;
          b.cfly(i, j, k) = (v1 + 2 * v2 + 2 * v3 + v4) / 6 * dt_ / dy;
          if (std::fabs(b.cfly(i, j, k)) > 1) err.set(GMC_ECFL, "cfly exceeds 1");
        }
      }
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) {
          b.divx(i, j, k) = (b.u(i, j, k) - b.u(i - 1, j, k)) * g.le_lon[j] / g.area_cell[j];
          b.divy(i, j, k) = (b.v(i, j, k) * g.le_lat[j] - b.v(i, j - 1, k) * g.le_lat[j - 1]) / g.area_cell[j];
        }
    }
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      double p = ring([&](int i) { return b.v(i, 1, k); });
      p = p * g.le_lat[1] / nlon / g.area_cell[1];
      for (int i = 1; i <= nlon; ++i) b.divy(i, 1, k) = p;
      p = ring([&](int i) { return -b.v(i, nhalf, k); });
      p = p * g.le_lat[nhalf] / nlon / g.area_cell[nlat];
      for (int i = 1; i <= nlon; ++i) b.divy(i, nlat, k) = p;
    }
  }

  // adv_batch_accum_mf_cell (adv_batch_mod.F90:379-403)
  void accum_mf_cell(Batch &b, Arr &mfx, Arr &mfy) {
    if (b.mf_step == 0) {
      b.mfx.d = mfx.d; b.mfy.d = mfy.d;
      if (!b.dynamic) b.mf_step = b.mf_step + 1;
    } else if (b.mf_step == b.nstep) {
      for (size_t n = 0; n < b.mfx.d.size(); ++n) b.mfx.d[n] = (b.mfx.d[n] + mfx.d[n]) / (b.nstep + 1);
      for (size_t n = 0; n < b.mfy.d.size(); ++n) b.mfy.d[n] = (b.mfy.d[n] + mfy.d[n]) / (b.nstep + 1);
      b.mf_step = 0;
    } else {
      for (size_t n = 0; n < b.mfx.d.size(); ++n) b.mfx.d[n] = b.mfx.d[n] + mfx.d[n];
      for (size_t n = 0; n < b.mfy.d.size(); ++n) b.mfy.d[n] = b.mfy.d[n] + mfy.d[n];
      b.mf_step = b.mf_step + 1;
    }
  }

  // adv_batch_accum_we_lev (adv_batch_mod.F90:493-632)
  void accum_we_lev(Batch &b, Arr &we, Arr &m_lev, double dt_) {
    const int nlon = mesh.nlon, nlat = mesh.nlat, nlev = mesh.nlev;
    const std::vector<double> &hl = grid.half_lev, &hd = grid.half_dlev, &fd = grid.full_dlev;
    // 1-based accessors
    auto HL = [&](int k) { return hl[k - 1]; };
    auto HD = [&](int k) { return hd[k - 1]; };
    auto FD = [&](int k) { return fd[k - 1]; };
    if (b.we_step == 0) {
      b.we.d = we.d; b.m_lev.d = m_lev.d;
      if (!b.dynamic) b.we_step = b.we_step + 1;
    } else if (b.we_step == b.nstep) {
      for (size_t n = 0; n < b.we.d.size(); ++n) b.we.d[n] = (b.we.d[n] + we.d[n]) / (b.nstep + 1);
      for (size_t n = 0; n < b.m_lev.d.size(); ++n) b.m_lev.d[n] = (b.m_lev.d[n] + m_lev.d[n]) / (b.nstep + 1);
      b.we_step = 0;
    } else {
      for (size_t n = 0; n < b.we.d.size(); ++n) b.we.d[n] = b.we.d[n] + we.d[n];
      for (size_t n = 0; n < b.m_lev.d.size(); ++n) b.m_lev.d[n] = b.m_lev.d[n] + m_lev.d[n];
      b.we_step = b.we_step + 1;
    }
    if (b.we_step != 0) return;
    #pragma omp parallel for schedule(static)
    for (int k = 2; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          auto W = [&](int l) { return b.we(i, j, l) / b.m_lev(i, j, l) * HD(l); };
          auto locate = [&](double w, double z) {
            int l;
            if (w > 0) {
              for (l = k; l <= nlev; ++l)
                if (HL(l) <= z && z <= HL(l + 1)) break;
              if (l == nlev + 1) { err.set(GMC_ECFL, "cflz exceeds range"); l = nlev; }
            } else {
              for (l = k - 1; l >= 1; --l)
                if (HL(l) <= z && z <= HL(l + 1)) break;
              if (l == 0) { err.set(GMC_ECFL, "cflz exceeds range"); l = 1; }
            }
            return l;
          };
          auto interp = [&](int l, double z) {
            return ((HL(l + 1) - z) * b.we(i, j, l) / b.m_lev(i, j, l) * HD(l) +
                    (z - HL(l)) * b.we(i, j, l + 1) / b.m_lev(i, j, l + 1) * HD(l + 1)) / FD(l);
          };
          double z0 = HL(k);
          double w1 = W(k);
          double z1 = z0 + dt_ / 2 * w1;
          double w2 = interp(locate(w1, z1), z1);
          double z2 = z0 + dt_ / 2 * w2;
          double w3 = interp(locate(w2, z2), z2);
          double z3 = z0 + dt_ * w3;
          double w4 = interp(locate(w3, z3), z3);
          double deta = (w1 + 2 * w2 + 2 * w3 + w4) / 6 * dt_;
          int ks, ke, s;
          if (deta < 0) { ks = k - 1; ke = 1; s = -1; } else { ks = k; ke = nlev; s = 1; }
          deta = std::fabs(deta);
          for (int l = ks; s > 0 ? l <= ke : l >= ke; l += s) {
            deta = deta - FD(l);
            if (deta < 0) {
              b.cflz(i, j, k) = s * ((1 + deta / FD(l)) + std::abs(l - ks));
              break;
            }
          }
        }
  }

  void calc_we_lev(State &s, Tend &t, double dt) {   // operators_mod.F90:192-232
    const int nlon = mesh.nlon, nlat = mesh.nlat, nlev = mesh.nlev;
    const gmc::Grid &g = G();
    #pragma omp parallel for schedule(static)
    for (int k = 2; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double mf = 0.0;
          for (int l = 1; l <= k - 1; ++l) mf = mf + t.dmfdlon(i, j, l) + t.dmfdlat(i, j, l);
          s.we_lev(i, j, k) = -(g.hybi[k - 1] * t.dphs(i, j, 1)) - mf;
        }
    for (int j = s.we_lev.lb1; j <= s.we_lev.ub1; ++j)
      for (int i = s.we_lev.lb0; i <= s.we_lev.ub0; ++i) {
        s.we_lev(i, j, 1) = 0.0;
        s.we_lev(i, j, nlev + 1) = 0.0;
      }
    fill_halo(s.we_lev, true);
    accum_we_lev(mass, s.we_lev, s.m_lev, dt);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev + 1; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i)
          s.we_lev_lon(i, j, k) = (g.area_lon_west[j] * s.we_lev(i, j, k) + g.area_lon_east[j] * s.we_lev(i + 1, j, k)) /
                                  g.area_lon[j];
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev + 1; ++k)
      for (int j = 1; j <= mesh.nhalf; ++j)
        for (int i = 1; i <= nlon; ++i)
          s.we_lev_lat(i, j, k) = (g.area_lat_north[j] * s.we_lev(i, j + 1, k) + g.area_lat_south[j] * s.we_lev(i, j, k)) /
                                  g.area_lat[j];
  }

  void calc_ke(State &s) {   // operators_mod.F90:234-352
    const int nlon = mesh.nlon, nlat = mesh.nlat, nlev = mesh.nlev, nhalf = mesh.nhalf;
    const gmc::Grid &g = G();
    Arr &u = s.u_f, &v = s.v_f, &ke = s.ke;
    auto sq = [](double x) { return x * x; };
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon + 1; ++i)
          ke(i, j, k) = (g.area_lon_west[j] * sq(u(i - 1, j, k)) + g.area_lon_east[j] * sq(u(i, j, k)) +
                         g.area_lat_north[j - 1] * sq(v(i, j - 1, k)) + g.area_lat_south[j] * sq(v(i, j, k))) /
                        g.area_cell[j];
    if (cfg.ke_scheme == 2) {
      const double w = cfg.ke_cell_wgt;
      #pragma omp parallel for schedule(static)
      for (int k = 1; k <= nlev; ++k)
        for (int j = 2; j <= nlat - 1; ++j)
          for (int i = 1; i <= nlon + 1; ++i) {
            double k1 = (g.area_lat_east[j] * sq(v(i - 1, j, k)) + g.area_lat_west[j] * sq(v(i, j, k)) +
                         g.area_lon_north[j] * sq(u(i - 1, j, k)) + g.area_lon_south[j + 1] * sq(u(i - 1, j + 1, k))) /
                        g.area_vtx[j];
            double k2 = (g.area_lat_east[j - 1] * sq(v(i - 1, j - 1, k)) + g.area_lat_west[j - 1] * sq(v(i, j - 1, k)) +
                         g.area_lon_north[j - 1] * sq(u(i - 1, j - 1, k)) + g.area_lon_south[j] * sq(u(i - 1, j, k))) /
                        g.area_vtx[j - 1];
            double k3 = (g.area_lat_east[j - 1] * sq(v(i, j - 1, k)) + g.area_lat_west[j - 1] * sq(v(i + 1, j - 1, k)) +
                         g.area_lon_north[j - 1] * sq(u(i, j - 1, k)) + g.area_lon_south[j] * sq(u(i, j, k))) /
                        g.area_vtx[j - 1];
            double k4 = (g.area_lat_east[j] * sq(v(i, j, k)) + g.area_lat_west[j] * sq(v(i + 1, j, k)) +
                         g.area_lon_north[j] * sq(u(i, j, k)) + g.area_lon_south[j + 1] * sq(u(i, j + 1, k))) /
                        g.area_vtx[j];
            ke(i, j, k) = (1.0 - w) * ((k1 + k4) * g.area_subcell2[j] + (k2 + k3) * g.area_subcell1[j]) / g.area_cell[j] +
                          w * ke(i, j, k);
          }
    }
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      double p = ring([&](int i) { return v(i, 1, k) * v(i, 1, k); });
      p = p / nlon;
      for (int i = 1; i <= nlon; ++i) ke(i, 1, k) = p;
      p = ring([&](int i) { return v(i, nhalf, k) * v(i, nhalf, k); });
      p = p / nlon;
      for (int i = 1; i <= nlon; ++i) ke(i, nlat, k) = p;
    }
  }

  void calc_mf(State &s, double dt) {   // operators_mod.F90:545-610
    const int nlon = mesh.nlon, nlat = mesh.nlat, nlev = mesh.nlev, nhalf = mesh.nhalf;
    const gmc::Grid &g = G();
    if (baroclinic) accum_uv_cell(mass, s.u_f, s.v_f, dt);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 0; i <= nlon; ++i) s.mfx_lon(i, j, k) = s.m_lon(i, j, k) * s.u_f(i, j, k);
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon + 1; ++i) s.mfy_lat(i, j, k) = s.m_lat(i, j, k) * s.v_f(i, j, k);
    if (baroclinic) accum_mf_cell(mass, s.mfx_lon, s.mfy_lat);
    calc_u_lat(s);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) {
          s.mfy_lon(i, j, k) = g.full_tangent_wgt1[j] * (s.mfy_lat(i, j - 1, k) + s.mfy_lat(i + 1, j - 1, k)) +
                               g.full_tangent_wgt2[j] * (s.mfy_lat(i, j, k) + s.mfy_lat(i + 1, j, k));
          s.v_lon(i, j, k) = s.mfy_lon(i, j, k) / s.m_lon(i, j, k);
        }
    fill_halo(s.v_lon, true);
  }

  // tangential mass flux and wind on the half rows (calc_mf, operators_mod.F90:585-597)
  void calc_u_lat(State &s) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf;
    const gmc::Grid &g = G();
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) {
          s.mfx_lat(i, j, k) = g.half_tangent_wgt1[j] * (s.mfx_lon(i - 1, j, k) + s.mfx_lon(i, j, k)) +
                               g.half_tangent_wgt2[j] * (s.mfx_lon(i - 1, j + 1, k) + s.mfx_lon(i, j + 1, k));
          s.u_lat(i, j, k) = s.mfx_lat(i, j, k) / s.m_lat(i, j, k);
        }
    fill_halo(s.u_lat, false);
  }

  void calc_pv(State &s) {   // calc_vor + calc_pv, operators_mod.F90:612-703
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf;
    const gmc::Grid &g = G();
    calc_vor(s);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) s.pv(i, j, k) = (s.vor(i, j, k) + g.half_f[j]) / s.m_vtx(i, j, k);
    fill_halo(s.pv, false);
  }

  void calc_vor(State &s) {   // operators_mod.F90:612-680
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf;
    const gmc::Grid &g = G();
    Arr &u = s.u_f, &v = s.v_f, &vor = s.vor;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 0; i <= nlon; ++i)
          vor(i, j, k) = (u(i, j, k) * g.de_lon[j] - u(i, j + 1, k) * g.de_lon[j + 1] + v(i + 1, j, k) * g.de_lat[j] -
                          v(i, j, k) * g.de_lat[j]) / g.area_vtx[j];
    if (cfg.pv_pole_stokes) {
      #pragma omp parallel for schedule(static)
      for (int k = 1; k <= nlev; ++k) {
        double p = ring([&](int i) { return -s.u_lat(i, 1, k) * g.le_lat[1]; });
        p = p / nlon / g.area_cell[1];
        for (int i = 1; i <= nlon; ++i) vor(i, 1, k) = p;
        p = ring([&](int i) { return s.u_lat(i, nhalf, k) * g.le_lat[nhalf]; });
        p = p / nlon / g.area_cell[nhalf + 1];
        for (int i = 1; i <= nlon; ++i) vor(i, nhalf, k) = p;
      }
    }
  }

  // The fields a history record holds beside the state (history_mod.F90:519-580
  // writes state%ph, t, gz / g, vor and div): recomputed on a copy of
  // state(old) by calc_ph, calc_m, calc_t, calc_gz_lev, the zonal and
  // tangential mass fluxes of calc_mf (without its batch accumulation),
  // calc_vor and calc_div.
  State output_state() {
    State d = state[old_i];
    const int nlon = mesh.nlon, nlat = mesh.nlat, nlev = mesh.nlev;
    if (baroclinic) calc_ph(d);
    calc_m(d);
    if (baroclinic) {
      calc_t(d);
      calc_gz_lev(d);
    }
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 0; i <= nlon; ++i) d.mfx_lon(i, j, k) = d.m_lon(i, j, k) * d.u_f(i, j, k);
    calc_u_lat(d);
    calc_vor(d);
    calc_div(d);
    return d;
  }

  static double upwind1(double dir, double wgt, double f1, double f2) {
    const double c11 = 0.5, c12 = -0.5;
    return c11 * (f2 + f1) + c12 * (f2 - f1) * wgt * dir;
  }
  static double upwind3(double dir, double wgt, double f1, double f2, double f3, double f4) {
    const double c31 = 7.0 / 12.0, c32 = -1.0 / 12.0, c33 = 1.0 / 12.0;
    return c31 * (f3 + f2) + c32 * (f4 + f1) + c33 * (f4 - f1 - 3 * (f3 - f2)) * wgt * dir;
  }

  // tvd (tvd_mod.F90:44-60) with the flux limiters of :62-84; eps is the
  // default-kind literal 1.0e-6 widened to double.
  double tvd(double cfl, double fm1, double f, double fp1, double fp2) const {
    const double eps = (double)1.0e-6f;
    double r;
    if (cfl > 0)
      r = (f - fm1 + eps) / (fp1 - f + eps);
    else
      r = (fp2 - fp1 + eps) / (fp1 - f + eps);
    double C;
    switch (cfg.tvd_limiter_type) {
      case GMC_TVD_NONE: C = 1; break;
      case GMC_TVD_MC: C = std::fmax(0.0, std::fmin(std::fmin(2.0 * r, 0.5 * (1 + r)), 2.0)); break;
      default: C = (r + std::fabs(r)) / (1 + std::fabs(r)); break;
    }
    return 0.5 * (fp1 + f - ((1 - C) * fsign(1.0, cfl) + cfl * C) * (fp1 - f));
  }

  void interp_pv(State &s, double dt) {   // operators_mod.F90:705-832
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const double eps = std::numeric_limits<double>::epsilon();
    Arr &pv = s.pv;
    if (cfg.pv_scheme == GMC_PV_TVD) {   // interp_pv_tvd :797-832
      const gmc::Grid &g = G();
      #pragma omp parallel for schedule(static)
      for (int k = 1; k <= nlev; ++k) {
        for (int j = 2; j <= nlat - 1; ++j)
          for (int i = 1; i <= nlon; ++i) {
            double cfl = s.v_lon(i, j, k) * dt / g.le_lon[j];
            s.pv_lon(i, j, k) = tvd(cfl, pv(i, j - 2, k), pv(i, j - 1, k), pv(i, j, k), pv(i, j + 1, k));
          }
        for (int j = 1; j <= nhalf; ++j)
          for (int i = 1; i <= nlon; ++i) {
            double cfl = s.u_lat(i, j, k) * dt / g.le_lat[j];
            s.pv_lat(i, j, k) = tvd(cfl, pv(i - 2, j, k), pv(i - 1, j, k), pv(i, j, k), pv(i + 1, j, k));
          }
      }
      fill_halo(s.pv_lon, true, true, true, false, true);
      fill_halo(s.pv_lat, false, true, true, true, false);
      return;
    }
    if (cfg.pv_scheme == GMC_PV_MIDPOINT) {
      #pragma omp parallel for schedule(static)
      for (int k = 1; k <= nlev; ++k)
        for (int j = 1; j <= nhalf; ++j)
          for (int i = 1; i <= nlon; ++i) s.pv_lat(i, j, k) = 0.5 * (pv(i - 1, j, k) + pv(i, j, k));
      fill_halo(s.pv_lat, false, true, true, true, false);
      #pragma omp parallel for schedule(static)
      for (int k = 1; k <= nlev; ++k)
        for (int j = 2; j <= nlat - 1; ++j)
          for (int i = 1; i <= nlon; ++i) s.pv_lon(i, j, k) = 0.5 * (pv(i, j, k) + pv(i, j - 1, k));
      fill_halo(s.pv_lon, true, true, true, false, true);
      return;
    }
    Arr &un = s.u_f, &vn = s.v_f, &ut = s.u_lat, &vt = s.v_lon;
    const double wgt = cfg.upwind_wgt_pv;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double b = std::fabs(vt(i, j, k)) / (std::sqrt(un(i, j, k) * un(i, j, k) + vt(i, j, k) * vt(i, j, k)) + eps);
          double dir = fsign(1.0, vt(i, j, k));
          double up = cfg.upwind_order_pv == 3
                          ? upwind3(dir, wgt, pv(i, j - 2, k), pv(i, j - 1, k), pv(i, j, k), pv(i, j + 1, k))
                          : upwind1(dir, wgt, pv(i, j - 1, k), pv(i, j, k));
          s.pv_lon(i, j, k) = b * up + (1 - b) * 0.5 * (pv(i, j - 1, k) + pv(i, j, k));
        }
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double b = std::fabs(ut(i, j, k)) / (std::sqrt(ut(i, j, k) * ut(i, j, k) + vn(i, j, k) * vn(i, j, k)) + eps);
          double dir = fsign(1.0, ut(i, j, k));
          double up = cfg.upwind_order_pv == 3
                          ? upwind3(dir, wgt, pv(i - 2, j, k), pv(i - 1, j, k), pv(i, j, k), pv(i + 1, j, k))
                          : upwind1(dir, wgt, pv(i - 1, j, k), pv(i, j, k));
          s.pv_lat(i, j, k) = b * up + (1 - b) * 0.5 * (pv(i - 1, j, k) + pv(i, j, k));
        }
    }
    fill_halo(s.pv_lon, true, true, true, false, true);
    fill_halo(s.pv_lat, false, true, true, true, false);
  }

  void calc_gz_lev(State &s) {   // operators_mod.F90:433-469
    const int nlon = mesh.nlon, nlat = mesh.nlat, nlev = mesh.nlev;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double dgz = 0.0;
          for (int l = k; l <= nlev; ++l)
            dgz = dgz + cfg.Rd * s.t(i, j, l) * std::log(s.ph_lev(i, j, l + 1) / s.ph_lev(i, j, l));
          s.gz_lev(i, j, k) = gzs(i, j, 1) + dgz;
        }
    fill_halo(s.gz_lev, true);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) s.gz(i, j, k) = 0.5 * (s.gz_lev(i, j, k) + s.gz_lev(i, j, k + 1));
  }

  void calc_coriolis(State &s, Tend &t) {   // operators_mod.F90:846-906
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const gmc::Grid &g = G();
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) {
          if (cfg.coriolis_scheme == 1)
            t.qhu(i, j, k) = (g.half_tangent_wgt1[j] * (s.mfx_lon(i - 1, j, k) * (s.pv_lat(i, j, k) + s.pv_lon(i - 1, j, k)) +
                                                        s.mfx_lon(i, j, k) * (s.pv_lat(i, j, k) + s.pv_lon(i, j, k))) +
                              g.half_tangent_wgt2[j] * (s.mfx_lon(i - 1, j + 1, k) * (s.pv_lat(i, j, k) + s.pv_lon(i - 1, j + 1, k)) +
                                                        s.mfx_lon(i, j + 1, k) * (s.pv_lat(i, j, k) + s.pv_lon(i, j + 1, k)))) *
                             0.5;
          else
            t.qhu(i, j, k) = s.mfx_lat(i, j, k) * s.pv_lat(i, j, k);
        }
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) {
          if (cfg.coriolis_scheme == 1)
            t.qhv(i, j, k) = (g.full_tangent_wgt1[j] * (s.mfy_lat(i, j - 1, k) * (s.pv_lon(i, j, k) + s.pv_lat(i, j - 1, k)) +
                                                        s.mfy_lat(i + 1, j - 1, k) * (s.pv_lon(i, j, k) + s.pv_lat(i + 1, j - 1, k))) +
                              g.full_tangent_wgt2[j] * (s.mfy_lat(i, j, k) * (s.pv_lon(i, j, k) + s.pv_lat(i, j, k)) +
                                                        s.mfy_lat(i + 1, j, k) * (s.pv_lon(i, j, k) + s.pv_lat(i + 1, j, k)))) *
                             0.5;
          else
            t.qhv(i, j, k) = s.mfy_lon(i, j, k) * s.pv_lon(i, j, k);
        }
  }

  void calc_grad_ke(State &s, Tend &t) {   // operators_mod.F90:908-937
    const gmc::Grid &g = G();
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= mesh.nlev; ++k) {
      for (int j = 2; j <= mesh.nlat - 1; ++j)
        for (int i = 1; i <= mesh.nlon; ++i) t.dkedlon(i, j, k) = (s.ke(i + 1, j, k) - s.ke(i, j, k)) / g.de_lon[j];
      for (int j = 1; j <= mesh.nhalf; ++j)
        for (int i = 1; i <= mesh.nlon; ++i) t.dkedlat(i, j, k) = (s.ke(i, j + 1, k) - s.ke(i, j, k)) / g.de_lat[j];
    }
  }

  // divergence of an edge flux pair with pole ring sums (the pattern of
  // calc_grad_mf, operators_mod.F90:939-1006, and calc_grad_ptf :1034-1082)
  void flux_div(Arr &fx, Arr &fy, Arr &dx, Arr &dy) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const gmc::Grid &g = G();
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) dx(i, j, k) = (fx(i, j, k) - fx(i - 1, j, k)) * g.le_lon[j] / g.area_cell[j];
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i)
          dy(i, j, k) = (fy(i, j, k) * g.le_lat[j] - fy(i, j - 1, k) * g.le_lat[j - 1]) / g.area_cell[j];
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      double p = ring([&](int i) { return fy(i, 1, k); });
      p = p * g.le_lat[1] / nlon / g.area_cell[1];
      for (int i = 1; i <= nlon; ++i) dy(i, 1, k) = p;
      p = ring([&](int i) { return -fy(i, nhalf, k); });
      p = p * g.le_lat[nhalf] / nlon / g.area_cell[nlat];
      for (int i = 1; i <= nlon; ++i) dy(i, nlat, k) = p;
    }
  }

  void calc_dphsdt(Tend &t) {   // operators_mod.F90:1120-1143
    std::fill(t.dphs.d.begin(), t.dphs.d.end(), 0.0);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= mesh.nlat; ++j)
      for (int k = 1; k <= mesh.nlev; ++k)
        for (int i = 1; i <= mesh.nlon; ++i)
          t.dphs(i, j, 1) = t.dphs(i, j, 1) - t.dmfdlon(i, j, k) - t.dmfdlat(i, j, k);
  }

  void calc_wedudlev_wedvdlev(State &s, Tend &t) {   // operators_mod.F90:1145-1216
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    Arr &u = s.u_f, &v = s.v_f;
    #pragma omp parallel for schedule(static)
    for (int k = 2; k <= nlev - 1; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i)
          t.wedudlev(i, j, k) = (s.we_lev_lon(i, j, k + 1) * (u(i, j, k + 1) - u(i, j, k)) +
                                 s.we_lev_lon(i, j, k) * (u(i, j, k) - u(i, j, k - 1))) / s.m_lon(i, j, k) / 2.0;
    for (int j = 2; j <= nlat - 1; ++j)
      for (int i = 1; i <= nlon; ++i) {
        t.wedudlev(i, j, 1) = (s.we_lev_lon(i, j, 2) * (u(i, j, 2) - u(i, j, 1))) / s.m_lon(i, j, 1) / 2.0;
        t.wedudlev(i, j, nlev) = (s.we_lev_lon(i, j, nlev) * (u(i, j, nlev) - u(i, j, nlev - 1))) / s.m_lon(i, j, nlev) / 2.0;
      }
    #pragma omp parallel for schedule(static)
    for (int k = 2; k <= nlev - 1; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i)
          t.wedvdlev(i, j, k) = (s.we_lev_lat(i, j, k + 1) * (v(i, j, k + 1) - v(i, j, k)) +
                                 s.we_lev_lat(i, j, k) * (v(i, j, k) - v(i, j, k - 1))) / s.m_lat(i, j, k) / 2.0;
    for (int j = 1; j <= nhalf; ++j)
      for (int i = 1; i <= nlon; ++i) {
        t.wedvdlev(i, j, 1) = (s.we_lev_lat(i, j, 2) * (v(i, j, 2) - v(i, j, 1))) / s.m_lat(i, j, 1) / 2.0;
        t.wedvdlev(i, j, nlev) = (s.we_lev_lat(i, j, nlev) * (v(i, j, nlev) - v(i, j, nlev - 1))) / s.m_lat(i, j, nlev) / 2.0;
      }
  }

  // ========================================================================
  // FFSL (ffsl_mod.F90)
  // ========================================================================
  double slope(double fm1, double f, double fp1) const {
    double df = (fp1 - fm1) * 0.5;
    switch (cfg.limiter_type) {
      case GMC_LIMITER_NONE: return df;
      case GMC_LIMITER_PD: return fsign(std::fmin(std::fabs(df), 2 * f), df);
      default: {
        double dmin = 2 * (f - fmin3(fm1, f, fp1));
        double dmax = 2 * (fmax3(fm1, f, fp1) - f);
        return fsign(fmin3(std::fabs(df), dmin, dmax), df);
      }
    }
  }
  void ppm(double fm2, double fm1, double f, double fp1, double fp2, double &fl, double &df, double &f6) const {
    double dfl = slope(fm2, fm1, f);
    df = slope(fm1, f, fp1);
    double dfr = slope(f, fp1, fp2);
    fl = 0.5 * (fm1 + f) + (dfl - df) / 6.0;
    double fr = 0.5 * (fp1 + f) + (df - dfr) / 6.0;
    fl = f - fsign(std::fmin(std::fabs(df), std::fabs(fl - f)), df);
    fr = f + fsign(std::fmin(std::fabs(df), std::fabs(fr - f)), df);
    f6 = 6 * f - 3 * (fl + fr);
    df = fr - fl;
  }

  // hflx_ppm_cell (ffsl_mod.F90:778-881)
  void hflx_ppm_cell(Batch &b, Arr &u, Arr &v, Arr &mx, Arr &my, Arr &mfx, Arr &mfy) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    Arr &mlx = b.qlx, &mly = b.qly, &dmx = b.dqx, &dmy = b.dqy, &m6x = b.q6x, &m6y = b.q6y;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          ppm(mx(i - 2, j, k), mx(i - 1, j, k), mx(i, j, k), mx(i + 1, j, k), mx(i + 2, j, k), mlx(i, j, k), dmx(i, j, k), m6x(i, j, k));
          ppm(my(i, j - 2, k), my(i, j - 1, k), my(i, j, k), my(i, j + 1, k), my(i, j + 2, k), mly(i, j, k), dmy(i, j, k), m6y(i, j, k));
        }
    fill_halo(mlx, true, true, true, false, false);
    fill_halo(dmx, true, true, true, false, false);
    fill_halo(m6x, true, true, true, false, false);
    fill_halo(mly, true, false, false, true, true);
    fill_halo(dmy, true, false, false, true, true);
    fill_halo(m6y, true, false, false, true, true);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double c = b.cflx(i, j, k);
          int ci = (int)c;   // int() truncates toward zero
          double cf = c - ci;
          if (c > 0) {
            int iu = i - ci;
            double s1 = 1 - cf, s2 = 1;
            double ds1 = s2 - s1, ds2 = s2 * s2 - s1 * s1, ds3 = s2 * s2 * s2 - s1 * s1 * s1;
            double sum = 0;
            for (int l = i + 1 - ci; l <= i; ++l) sum = sum + mx(l, j, k);
            mfx(i, j, k) = u(i, j, k) * (sum + mlx(iu, j, k) * ds1 + 0.5 * dmx(iu, j, k) * ds2 +
                                         m6x(iu, j, k) * (ds2 / 2.0 - ds3 / 3.0)) / c;
          } else if (c < 0) {
            int iu = i - ci + 1;
            double s1 = 0, s2 = -cf;
            double ds1 = s2 - s1, ds2 = s2 * s2 - s1 * s1, ds3 = s2 * s2 * s2 - s1 * s1 * s1;
            double sum = 0;
            for (int l = i + 1; l <= i - ci; ++l) sum = sum + mx(l, j, k);
            mfx(i, j, k) = -u(i, j, k) * (sum + mlx(iu, j, k) * ds1 + 0.5 * dmx(iu, j, k) * ds2 +
                                          m6x(iu, j, k) * (ds2 / 2.0 - ds3 / 3.0)) / c;
          } else {
            mfx(i, j, k) = 0;
          }
        }
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double c = b.cfly(i, j, k);
          if (c > 0) {
            int ju = j;
            double s1 = 1 - c, s2 = 1;
            double ds1 = s2 - s1, ds2 = s2 * s2 - s1 * s1, ds3 = s2 * s2 * s2 - s1 * s1 * s1;
            mfy(i, j, k) = v(i, j, k) * (mly(i, ju, k) * ds1 + 0.5 * dmy(i, ju, k) * ds2 + m6y(i, ju, k) * (ds2 / 2.0 - ds3 / 3.0)) / c;
          } else if (c < 0) {
            int ju = j + 1;
            double s1 = 0, s2 = -c;
            double ds1 = s2 - s1, ds2 = s2 * s2 - s1 * s1, ds3 = s2 * s2 * s2 - s1 * s1 * s1;
            mfy(i, j, k) = -v(i, j, k) * (mly(i, ju, k) * ds1 + 0.5 * dmy(i, ju, k) * ds2 + m6y(i, ju, k) * (ds2 / 2.0 - ds3 / 3.0)) / c;
          } else {
            mfy(i, j, k) = 0;
          }
        }
    }
  }

  // vflx_ppm_cell (ffsl_mod.F90:883-941)
  void vflx_ppm_cell(Batch &b, Arr &w, Arr &m, Arr &mfz) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nlat = mesh.nlat;
    Arr &mlz = b.qlx, &dmz = b.dqx, &m6z = b.q6x;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i)
          ppm(m(i, j, k - 2), m(i, j, k - 1), m(i, j, k), m(i, j, k + 1), m(i, j, k + 2), mlz(i, j, k), dmz(i, j, k), m6z(i, j, k));
    #pragma omp parallel for schedule(static)
    for (int k = 2; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double c = b.cflz(i, j, k);
          int ci = (int)c;
          double cf = c - ci;
          if (c > 0) {
            int ku = k - ci - 1;
            double s1 = 1 - cf, s2 = 1;
            double ds1 = s2 - s1, ds2 = s2 * s2 - s1 * s1, ds3 = s2 * s2 * s2 - s1 * s1 * s1;
            double sum = 0;
            for (int l = k - ci; l <= k - 1; ++l) sum = sum + m(i, j, l);
            mfz(i, j, k) = w(i, j, k) * (sum + mlz(i, j, ku) * ds1 + 0.5 * dmz(i, j, ku) * ds2 +
                                         m6z(i, j, ku) * (ds2 / 2.0 - ds3 / 3.0)) / c;
          } else if (c < 0) {
            int ku = k - ci;
            double s1 = 0, s2 = -cf;
            double ds1 = s2 - s1, ds2 = s2 * s2 - s1 * s1, ds3 = s2 * s2 * s2 - s1 * s1 * s1;
            double sum = 0;
            for (int l = k; l <= k - ci - 1; ++l) sum = sum + m(i, j, l);
            mfz(i, j, k) = -w(i, j, k) * (sum + mlz(i, j, ku) * ds1 + 0.5 * dmz(i, j, ku) * ds2 +
                                          m6z(i, j, ku) * (ds2 / 2.0 - ds3 / 3.0)) / c;
          } else {
            mfz(i, j, k) = 0;
          }
        }
  }

  // hflx_van_leer_cell (ffsl_mod.F90:556-616)
  void hflx_van_leer_cell(Batch &b, Arr &u, Arr &v, Arr &mx, Arr &my, Arr &mfx, Arr &mfy) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double c = b.cflx(i, j, k);
          int ci = (int)c;
          double cf = c - ci;
          if (c > 0) {
            int iu = i - ci;
            double dm = slope(mx(iu - 1, j, k), mx(iu, j, k), mx(iu + 1, j, k));
            double sum = 0;
            for (int l = i + 1 - ci; l <= i; ++l) sum = sum + mx(l, j, k);
            mfx(i, j, k) = u(i, j, k) * (cf * (mx(iu, j, k) + dm * 0.5 * (1 - cf)) + sum) / c;
          } else if (c < 0) {
            int iu = i - ci + 1;
            double dm = slope(mx(iu - 1, j, k), mx(iu, j, k), mx(iu + 1, j, k));
            double sum = 0;
            for (int l = i + 1; l <= i - ci; ++l) sum = sum + mx(l, j, k);
            mfx(i, j, k) = u(i, j, k) * (cf * (mx(iu, j, k) - dm * 0.5 * (1 + cf)) - sum) / c;
          } else {
            mfx(i, j, k) = 0;
          }
        }
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double cf = b.cfly(i, j, k);
          int ju = cf > 0 ? j : j + 1;
          double dm = slope(my(i, ju - 1, k), my(i, ju, k), my(i, ju + 1, k));
          mfy(i, j, k) = v(i, j, k) * (my(i, ju, k) + dm * 0.5 * (fsign(1.0, cf) - cf));
        }
    }
  }

  // vflx_van_leer_cell (ffsl_mod.F90:618-658)
  void vflx_van_leer_cell(Batch &b, Arr &w, Arr &m, Arr &mfz) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nlat = mesh.nlat;
    #pragma omp parallel for schedule(static)
    for (int k = 2; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          double c = b.cflz(i, j, k);
          int ci = (int)c;
          double cf = c - ci;
          if (c > 0) {
            int ku = k - ci - 1;
            double dm = slope(m(i, j, ku - 1), m(i, j, ku), m(i, j, ku + 1));
            double sum = 0;
            for (int l = k - ci; l <= k - 1; ++l) sum = sum + m(i, j, l);
            mfz(i, j, k) = w(i, j, k) * (cf * (m(i, j, ku) + dm * 0.5 * (1 - cf)) + sum) / c;
          } else if (c < 0) {
            int ku = k - ci;
            double dm = slope(m(i, j, ku - 1), m(i, j, ku), m(i, j, ku + 1));
            double sum = 0;
            for (int l = k; l <= k - ci - 1; ++l) sum = sum + m(i, j, l);
            mfz(i, j, k) = w(i, j, k) * (cf * (m(i, j, ku) - dm * 0.5 * (1 + cf)) - sum) / c;
          } else {
            mfz(i, j, k) = 0;
          }
        }
  }

  // the hflx_cell / vflx_cell procedure pointers (ffsl_mod.F90:114-142)
  void hflx_cell(Batch &b, Arr &u, Arr &v, Arr &mx, Arr &my, Arr &mfx, Arr &mfy) {
    if (cfg.ffsl_flux_type == GMC_FLUX_VAN_LEER) hflx_van_leer_cell(b, u, v, mx, my, mfx, mfy);
    else hflx_ppm_cell(b, u, v, mx, my, mfx, mfy);
  }
  void vflx_cell(Batch &b, Arr &w, Arr &m, Arr &mfz) {
    if (cfg.ffsl_flux_type == GMC_FLUX_VAN_LEER) vflx_van_leer_cell(b, w, m, mfz);
    else vflx_ppm_cell(b, w, m, mfz);
  }

  // ffsl_calc_tracer_hflx_cell (ffsl_mod.F90:318-413)
  void tracer_hflx_cell(Batch &b, Arr &q, Arr &qmfx, Arr &qmfy, double dt_) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const gmc::Grid &g = G();
    Arr &qx = b.qx, &qy = b.qy;
    hflx_cell(b, b.u, b.v, q, q, qmfx, qmfy);
    fill_halo(qmfx, true, true, true, false, false);
    fill_halo(qmfy, false, false, false, true, true);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) {
          qx(i, j, k) = q(i, j, k) - 0.5 * ((qmfx(i, j, k) - qmfx(i - 1, j, k)) * g.le_lon[j] / g.area_cell[j] -
                                            b.divx(i, j, k) * q(i, j, k)) * dt_;
          qy(i, j, k) = q(i, j, k) - 0.5 * ((qmfy(i, j, k) * g.le_lat[j] - qmfy(i, j - 1, k) * g.le_lat[j - 1]) / g.area_cell[j] -
                                            b.divy(i, j, k) * q(i, j, k)) * dt_;
        }
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      double p = ring([&](int i) { return qmfy(i, 1, k); });
      p = p * g.le_lat[1] / nlon / g.area_cell[1];
      for (int i = 1; i <= nlon; ++i) {
        qx(i, 1, k) = q(i, 1, k);
        qy(i, 1, k) = q(i, 1, k) - 0.5 * (p - b.divy(i, 1, k) * q(i, 1, k)) * dt_;
      }
      p = ring([&](int i) { return qmfy(i, nhalf, k); });
      p = p * g.le_lat[nhalf] / nlon / g.area_cell[nlat];
      for (int i = 1; i <= nlon; ++i) {
        qx(i, nlat, k) = q(i, nlat, k);
        qy(i, nlat, k) = q(i, nlat, k) + 0.5 * (p - b.divy(i, nlat, k) * q(i, nlat, k)) * dt_;
      }
    }
    fill_halo(qx, true, false, false, true, true);
    fill_halo(qy, true, true, true, false, false);
    hflx_cell(b, b.mfx, b.mfy, qy, qx, qmfx, qmfy);
  }

  void calc_grad_ptf(State &s, Tend &t, double dt) {   // operators_mod.F90:1008-1118
    const int nlev = mesh.nlev;
    tracer_hflx_cell(mass, s.pt, s.ptf_lon, s.ptf_lat, dt);
    fill_halo(s.ptf_lon, true, true, false, false, false);
    fill_halo(s.ptf_lat, false, false, false, true, false);
    flux_div(s.ptf_lon, s.ptf_lat, t.dptfdlon, t.dptfdlat);
    Arr &pt = s.pt;
    for (int k = 0; k >= -1; --k)
      for (int j = pt.lb1; j <= pt.ub1; ++j)
        for (int i = pt.lb0; i <= pt.ub0; ++i) pt(i, j, k) = 2 * pt(i, j, k + 1) - pt(i, j, k + 2);
    for (int k = nlev + 1; k <= nlev + 2; ++k)
      for (int j = pt.lb1; j <= pt.ub1; ++j)
        for (int i = pt.lb0; i <= pt.ub0; ++i) pt(i, j, k) = 2 * pt(i, j, k - 1) - pt(i, j, k - 2);
    vflx_cell(mass, mass.we, pt, s.ptf_lev);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= mesh.nlat; ++j)
        for (int i = 1; i <= mesh.nlon; ++i) t.dptfdlev(i, j, k) = s.ptf_lev(i, j, k + 1) - s.ptf_lev(i, j, k);
  }

  void pgf_run(State &s, Tend &t) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const gmc::Grid &g = G();
    if (hydrostatic) {   // pgf_lin97_run (pgf_lin97_mod.F90:20-105)
      Arr &pe = s.ph_exn_lev, &gz = s.gz_lev;
      #pragma omp parallel for schedule(static)
      for (int k = 1; k <= nlev; ++k) {
        for (int j = 2; j <= nlat - 1; ++j)
          for (int i = 1; i <= nlon; ++i) {
            double dph1 = pe(i + 1, j, k + 1) - pe(i, j, k);
            double dph2 = pe(i, j, k + 1) - pe(i + 1, j, k);
            double dgz1 = gz(i, j, k + 1) - gz(i + 1, j, k);
            double dgz2 = gz(i, j, k) - gz(i + 1, j, k + 1);
            t.pgf_lon(i, j, k) = -(dph1 * dgz1 + dph2 * dgz2) / g.de_lon[j] / (dph1 + dph2);
          }
        for (int j = 1; j <= nhalf; ++j)
          for (int i = 1; i <= nlon; ++i) {
            double dph1 = pe(i, j + 1, k + 1) - pe(i, j, k);
            double dph2 = pe(i, j, k + 1) - pe(i, j + 1, k);
            double dgz1 = gz(i, j, k + 1) - gz(i, j + 1, k);
            double dgz2 = gz(i, j, k) - gz(i, j + 1, k + 1);
            t.pgf_lat(i, j, k) = -(dph1 * dgz1 + dph2 * dgz2) / g.de_lat[j] / (dph1 + dph2);
          }
      }
    } else {   // pgf_swm_run (pgf_swm_mod.F90:18-46)
      Arr &gz = s.gz_f;
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) t.pgf_lon(i, j, 1) = (gz(i + 1, j, 1) - gz(i, j, 1)) / g.de_lon[j];
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) t.pgf_lat(i, j, 1) = (gz(i, j + 1, 1) - gz(i, j, 1)) / g.de_lat[j];
    }
  }

  // ========================================================================
  // space_operators (gmcore_mod.F90:343-575), forward/backward passes
  // ========================================================================
  void operators_prepare_fwd(State &s, double dt) {
    calc_mf(s, dt);
    calc_ke(s);
    calc_pv(s);
    interp_pv(s, dt);
  }
  void operators_prepare_bwd(State &s) {
    if (hydrostatic) {
      calc_ph(s);
      calc_t(s);
      calc_gz_lev(s);
    }
    calc_m(s);
  }

  void space_operators_fwd(State &star, Tend &t1, double dt) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    t1.reset_flags();
    operators_prepare_fwd(star, dt);
    flux_div(star.mfx_lon, star.mfy_lat, t1.dmfdlon, t1.dmfdlat);   // calc_grad_mf
    if (hydrostatic) {
      calc_dphsdt(t1);
      calc_we_lev(star, t1, dt);
      calc_wedudlev_wedvdlev(star, t1);
      calc_grad_ptf(star, t1, dt);
    }
    calc_coriolis(star, t1);
    calc_grad_ke(star, t1);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i)
          t1.du(i, j, k) = hydrostatic ? t1.qhv(i, j, k) - t1.dkedlon(i, j, k) - t1.wedudlev(i, j, k)
                                       : t1.qhv(i, j, k) - t1.dkedlon(i, j, k);
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i)
          t1.dv(i, j, k) = hydrostatic ? -t1.qhu(i, j, k) - t1.dkedlat(i, j, k) - t1.wedvdlev(i, j, k)
                                       : -t1.qhu(i, j, k) - t1.dkedlat(i, j, k);
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          if (hydrostatic)
            t1.dpt(i, j, k) = -t1.dptfdlon(i, j, k) - t1.dptfdlat(i, j, k) - t1.dptfdlev(i, j, k);
          else
            t1.dgz(i, j, k) = -(t1.dmfdlon(i, j, k) + t1.dmfdlat(i, j, k)) * cfg.g;
        }
    }
    if (hydrostatic) { t1.update_phs = true; t1.update_pt = true; } else { t1.update_gz = true; }
  }

  void space_operators_bwd(State &nw, Tend &t1, Tend &t2) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    t1.reset_flags();
    operators_prepare_bwd(nw);
    pgf_run(nw, t1);
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) t1.du(i, j, k) = t2.du(i, j, k) - t1.pgf_lon(i, j, k);
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) t1.dv(i, j, k) = t2.dv(i, j, k) - t1.pgf_lat(i, j, k);
    }
    t1.update_u = true;
    t1.update_v = true;
  }

  // update_state (time_schemes_mod.F90:120-242)
  void update_state(Tend &t, State &o, State &n, double dt) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    if (baroclinic) {
      if (t.update_phs) {
        for (int j = 1; j <= nlat; ++j)
          for (int i = 1; i <= nlon; ++i) n.phs(i, j, 1) = o.phs(i, j, 1) + dt * t.dphs(i, j, 1);
        fill_halo(n.phs, true, true, true, false, false);
        filter(grid.big, n.phs, &n.phs_f, true, 1, 1);
        fill_halo(n.phs, true);
        calc_ph(n);
        calc_m(n);
      }
      if (t.update_pt) {
        #pragma omp parallel for schedule(static)
        for (int k = 1; k <= nlev; ++k)
          for (int j = 1; j <= nlat; ++j)
            for (int i = 1; i <= nlon; ++i) n.pt(i, j, k) = o.pt(i, j, k) * o.m(i, j, k) + dt * t.dpt(i, j, k);
        fill_halo(n.pt, true, true, true, false, false);
        filter(grid.small1, n.pt, nullptr, true, 1, nlev);
        #pragma omp parallel for schedule(static)
        for (int k = 1; k <= nlev; ++k)
          for (int j = 1; j <= nlat; ++j)
            for (int i = 1; i <= nlon; ++i) n.pt(i, j, k) = n.pt(i, j, k) / n.m(i, j, k);
        fill_halo(n.pt, true);
      }
    } else if (t.update_gz) {
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) n.gz(i, j, 1) = o.gz(i, j, 1) + dt * t.dgz(i, j, 1);
      fill_halo(n.gz, true, true, true, false, false);
      filter(grid.big, n.gz, &n.gz_f, true, 1, 1);
      fill_halo(n.gz_f, true);
      filter(grid.small1, n.gz, nullptr, true, 1, 1);
      fill_halo(n.gz, true);
    }
    if (t.update_u && t.update_v) {
      #pragma omp parallel for schedule(static)
      for (int k = 1; k <= nlev; ++k)
        for (int j = 2; j <= nlat - 1; ++j)
          for (int i = 1; i <= nlon; ++i) n.u_lon(i, j, k) = o.u_lon(i, j, k) + dt * t.du(i, j, k);
      for (int k = 1; k <= nlev; ++k)
        for (int j = 1; j <= nhalf; ++j)
          for (int i = 1; i <= nlon; ++i) n.v_lat(i, j, k) = o.v_lat(i, j, k) + dt * t.dv(i, j, k);
      if (baroclinic) {
        fill_halo(n.u_lon, true, true, true, false, false);
        filter(grid.small2, n.u_lon, nullptr, true, 1, nlev);
        fill_halo(n.u_lon, true);
        fill_halo(n.v_lat, false, true, true, false, false);
        filter(grid.small2, n.v_lat, nullptr, false, 1, nlev);
        fill_halo(n.v_lat, false);
      }
      fill_halo(n.u_lon, true);
      fill_halo(n.v_lat, false);
      const double wgt = 0.6;
      Arr &v = n.v_lat;
      for (int k = v.lb2; k <= v.ub2; ++k)
        for (int i = v.lb0; i <= v.ub0; ++i) {
          v(i, 1, k) = (1 - wgt) * v(i, 1, k) + wgt * v(i, 2, k);
          v(i, nhalf, k) = (1 - wgt) * v(i, nhalf, k) + wgt * v(i, nhalf - 1, k);
        }
      fill_halo(n.v_lat, false, false, false, true, true);
      filter(grid.big, n.u_lon, &n.u_f, true, 1, nlev);
      filter(grid.big, n.v_lat, &n.v_f, false, 1, nlev);
      fill_halo(n.u_f, true);
      fill_halo(n.v_f, false);
    }
  }

  void step_fb(int o, int s, int n, int t1, int t2, double dt) {   // step_forward_backward
    space_operators_fwd(state[s], tend[t1], dt);
    update_state(tend[t1], state[o], state[n], dt);
    space_operators_bwd(state[n], tend[t2], tend[t1]);
    update_state(tend[t2], state[o], state[n], dt);
  }

  // calc_div, order-2 branch (operators_mod.F90:354-412)
  void calc_div(State &s) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const gmc::Grid &g = G();
    Arr &u = s.u_f, &v = s.v_f, &div = s.div;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i)
          div(i, j, k) = ((u(i, j, k) * g.le_lon[j] - u(i - 1, j, k) * g.le_lon[j]) +
                          (v(i, j, k) * g.le_lat[j] - v(i, j - 1, k) * g.le_lat[j - 1])) / g.area_cell[j];
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      double p = ring([&](int i) { return v(i, 1, k); });
      p = p * g.le_lat[1] / nlon / g.area_cell[1];
      for (int i = 1; i <= nlon; ++i) div(i, 1, k) = p;
      p = ring([&](int i) { return -v(i, nhalf, k); });
      p = p * g.le_lat[nhalf] / nlon / g.area_cell[nlat];
      for (int i = 1; i <= nlon; ++i) div(i, nlat, k) = p;
    }
    if (cfg.div_damp_order != 4) {
      fill_halo(div, true, false, true, false, true);
      return;
    }
    fill_halo(div, true);
    Arr &div2 = s.div2;   // operators_mod.F90:412-425
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i)
          div2(i, j, k) = (div(i + 1, j, k) - 2 * div(i, j, k) + div(i - 1, j, k)) / (g.de_lon[j] * g.de_lon[j]) +
                          ((div(i, j + 1, k) - div(i, j, k)) * g.half_cos_lat[j] / g.de_lat[j] -
                           (div(i, j, k) - div(i, j - 1, k)) * g.half_cos_lat[j - 1] / g.de_lat[j - 1]) /
                              g.le_lon[j] / g.full_cos_lat[j];
    fill_halo(div2, true, false, true, false, true);
  }

  // div_damp_run (div_damp_mod.F90:89-139)
  void div_damp_run(State &s) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const gmc::Grid &g = G();
    calc_div(s);
    if (cfg.div_damp_order == 4) {
      Arr &div2 = s.div2;
      #pragma omp parallel for schedule(static)
      for (int k = 1; k <= nlev; ++k)
        for (int j = 2; j <= nlat - 1; ++j)
          for (int i = 1; i <= nlon; ++i)
            s.u_lon(i, j, k) = s.u_lon(i, j, k) -
                               g.div_c_lon[(size_t)(k - 1) * nlat + (j - 1)] * (div2(i + 1, j, k) - div2(i, j, k)) / g.de_lon[j];
      #pragma omp parallel for schedule(static)
      for (int k = 1; k <= nlev; ++k)
        for (int j = 1; j <= nhalf; ++j)
          for (int i = 1; i <= nlon; ++i)
            s.v_lat(i, j, k) = s.v_lat(i, j, k) -
                               g.div_c_lat[(size_t)(k - 1) * nhalf + (j - 1)] * (div2(i, j + 1, k) - div2(i, j, k)) / g.de_lat[j];
      fill_halo(s.u_lon, true);
      fill_halo(s.v_lat, false);
      return;
    }
    Arr &div = s.div;
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i)
          s.u_lon(i, j, k) = s.u_lon(i, j, k) +
                             g.div_c_lon[(size_t)(k - 1) * nlat + (j - 1)] * (div(i + 1, j, k) - div(i, j, k)) / g.de_lon[j];
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i)
          s.v_lat(i, j, k) = s.v_lat(i, j, k) +
                             g.div_c_lat[(size_t)(k - 1) * nhalf + (j - 1)] * (div(i, j + 1, k) - div(i, j, k)) / g.de_lat[j];
    fill_halo(s.u_lon, true);
    fill_halo(s.v_lat, false);
  }

  // ========================================================================
  // adv_run (adv_mod.F90:152-312) for the single tracer batch
  // ========================================================================
  void accum_wind(Batch &b, State &s) {   // adv_accum_wind (adv_mod.F90:420-455)
    accum_uv_cell(b, s.u_f, s.v_f, b.dt);
    accum_mf_cell(b, s.mfx_lon, s.mfy_lat);
    if (mesh.nlev > 1) accum_we_lev(b, s.we_lev, s.m_lev, b.dt);
  }

  void lon_damp_on_cell(Arr &f) {   // lon_damp_on_cell_3d order 2 (lon_damp_mod.F90:158-241)
    const int nlon = mesh.nlon;
    std::vector<double> gw(nlon + 2);
    for (int k = 1; k <= mesh.nlev; ++k)
      for (int j = 2; j <= mesh.nlat - 1; ++j) {
        double wgt = grid.lon_damp_wgt_full[j - 1];
        if (wgt == 0) continue;
        const double c = 0.25;   // 0.5**2
        for (int i = 1; i <= nlon; ++i)
          gw[i] = wgt * (f(i, j, k) + c * (f(i - 1, j, k) - 2.0 * f(i, j, k) + f(i + 1, j, k))) + (1 - wgt) * f(i, j, k);
        for (int i = 1; i <= nlon; ++i) f(i, j, k) = gw[i];
      }
    fill_halo(f, true);
  }

  // Negative fixer along longitude (adv_mod.F90:236-258): sequential in i,
  // borrowing from i-1 and i+1, which at the row ends are the longitude halo.
  void zonal_fixer(Arr &qn, const Arr &m) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nlat = mesh.nlat;
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          if (qn(i, j, k) < 0) {
            double qm0 = qn(i, j, k) * m(i, j, k);
            double qm1 = qn(i - 1, j, k) * m(i - 1, j, k);
            double qm2 = qn(i + 1, j, k) * m(i + 1, j, k);
            double qm0_half = 0.5 * qm0;
            if (qm1 >= qm0_half && qm2 >= qm0_half) {
              qn(i - 1, j, k) = (qm1 - qm0_half) / m(i - 1, j, k);
              qn(i + 1, j, k) = (qm2 - qm0_half) / m(i + 1, j, k);
            } else if (qm1 > qm0) {
              qn(i - 1, j, k) = (qm1 - qm0) / m(i - 1, j, k);
            } else if (qm2 > qm0) {
              qn(i + 1, j, k) = (qm2 - qm0) / m(i + 1, j, k);
            } else {
              err.set(GMC_ENEGTRACER, "Negative tracer!");
            }
            qn(i, j, k) = 0;
          }
        }
  }

  // Negative fixer along the column (adv_mod.F90:275-297).
  void vertical_fixer(Arr &qn, const Arr &m) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nlat = mesh.nlat;
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          if (qn(i, j, k) < 0) {
            double qm0 = qn(i, j, k) * m(i, j, k);
            double qm1 = k > 1 ? qn(i, j, k - 1) * m(i, j, k - 1) : 0.0;
            double qm2 = k < nlev ? qn(i, j, k + 1) * m(i, j, k + 1) : 0.0;
            double qm0_half = 0.5 * qm0;
            if (qm1 >= qm0_half && qm2 >= qm0_half) {
              if (qm1 > 0) qn(i, j, k - 1) = (qm1 - qm0_half) / m(i, j, k - 1);
              if (qm2 > 0) qn(i, j, k + 1) = (qm2 - qm0_half) / m(i, j, k + 1);
            } else if (qm1 > qm0) {
              if (qm1 > 0) qn(i, j, k - 1) = (qm1 - qm0) / m(i, j, k - 1);
            } else if (qm2 > qm0) {
              if (qm2 > 0) qn(i, j, k + 1) = (qm2 - qm0) / m(i, j, k + 1);
            } else {
              err.set(GMC_ENEGTRACER, "Negative tracer!");
            }
            qn(i, j, k) = 0;
          }
        }
  }

  void adv_run(State &s) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const gmc::Grid &g = G();
    if (!has_tracers) return;
    Batch &b = tracers;
    accum_wind(b, s);
    // time_is_alerted(name) .and. time_step > 0 (time_mod.F90:270-291)
    bool ring_now = alert_last_time + b.dt <= curr_time + 1e-9 * b.dt;
    if (ring_now) alert_ringing = true;
    const double dt_adv = cfg.dt_adv;
    if (ring_now && time_step > 0) {
      for (int l = 0; l < cfg.ntracer; ++l) {
        Arr &qo = b.q[b.old_idx][l], &qn = b.q[b.new_idx][l];
        tracer_hflx_cell(b, qo, b.qmf_lon, b.qmf_lat, b.dt);
        fill_halo(b.qmf_lon, true, true, false, false, false);
        fill_halo(b.qmf_lat, false, false, false, true, false);
        for (int k = 1; k <= nlev; ++k)
          for (int j = 2; j <= nlat - 1; ++j)
            for (int i = 1; i <= nlon; ++i)
              qn(i, j, k) = b.old_m(i, j, k) * qo(i, j, k) -
                            ((b.qmf_lon(i, j, k) - b.qmf_lon(i - 1, j, k)) * g.le_lon[j] +
                             (b.qmf_lat(i, j, k) * g.le_lat[j] - b.qmf_lat(i, j - 1, k) * g.le_lat[j - 1])) /
                                g.area_cell[j] * dt_adv;
        for (int k = 1; k <= nlev; ++k) {
          double p = ring([&](int i) { return b.qmf_lat(i, 1, k); });
          p = p * g.le_lat[1] / nlon / g.area_cell[1] * dt_adv;
          for (int i = 1; i <= nlon; ++i) qn(i, 1, k) = b.old_m(i, 1, k) * qo(i, 1, k) - p;
          p = ring([&](int i) { return b.qmf_lat(i, nhalf, k); });
          p = p * g.le_lat[nhalf] / nlon / g.area_cell[nlat] * dt_adv;
          for (int i = 1; i <= nlon; ++i) qn(i, nlat, k) = b.old_m(i, nlat, k) * qo(i, nlat, k) + p;
        }
        for (int k = 1; k <= nlev; ++k)
          for (int j = 1; j <= nlat; ++j)
            for (int i = 1; i <= nlon; ++i) qn(i, j, k) = qn(i, j, k) / s.m(i, j, k);
        zonal_fixer(qn, s.m);
        for (int k = qn.lb2; k <= 0; ++k)
          for (int j = qn.lb1; j <= qn.ub1; ++j)
            for (int i = qn.lb0; i <= qn.ub0; ++i) qn(i, j, k) = qn(i, j, 1);
        for (int k = nlev + 1; k <= qn.ub2; ++k)
          for (int j = qn.lb1; j <= qn.ub1; ++j)
            for (int i = qn.lb0; i <= qn.ub0; ++i) qn(i, j, k) = qn(i, j, nlev);
        vflx_cell(b, b.we, qn, b.qmf_lev);
        for (int k = 1; k <= nlev; ++k)
          for (int j = 1; j <= nlat; ++j)
            for (int i = 1; i <= nlon; ++i)
              qn(i, j, k) = qn(i, j, k) - ((b.qmf_lev(i, j, k + 1) - b.qmf_lev(i, j, k)) * dt_adv) / s.m(i, j, k);
        vertical_fixer(qn, s.m);
        fill_halo(qn, true, true, true, false, false);
        for (int it = 0; it < 3; ++it) lon_damp_on_cell(qn);
        fill_halo(qn, true);
      }
      std::swap(b.old_idx, b.new_idx);
    }
    b.old_m.d = s.m.d;
  }
  bool alert_ringing = false;

  // ========================================================================
  // gmcore_run prologue and time loop
  // ========================================================================
  void prepare() {
    State &s = state[old_i];
    if (baroclinic)
      for (int t = 0; t < 3; ++t)
        for (int j = gzs.lb1; j <= gzs.ub1; ++j)
          for (int i = gzs.lb0; i <= gzs.ub0; ++i) state[t].gz_lev(i, j, mesh.nlev + 1) = gzs(i, j, 1);
    filter(grid.big, s.u_lon, &s.u_f, true, 1, mesh.nlev);
    fill_halo(s.u_f, true);
    filter(grid.big, s.v_lat, &s.v_f, false, 1, mesh.nlev);
    fill_halo(s.v_f, false);
    if (baroclinic) {
      filter(grid.big, s.phs, &s.phs_f, true, 1, 1);
      fill_halo(s.phs_f, true);
    } else {
      filter(grid.big, s.gz, &s.gz_f, true, 1, 1);
      fill_halo(s.gz_f, true);
    }
    if (has_tracers) {
      tracers.old_m.d = s.m.d;
      accum_wind(tracers, s);
    }
    // operators_prepare_1 (operators_mod.F90:73-94)
    if (baroclinic) calc_ph(s);
    calc_m(s);
    if (baroclinic) calc_t(s);
    calc_mf(s, cfg.dt_dyn);
    calc_ke(s);
    calc_pv(s);
    interp_pv(s, cfg.dt_dyn);
    if (hydrostatic) calc_gz_lev(s);
  }

  // debug_check_space_operators (debug_mod.F90:113-220): inner products of
  // the forward-pass tendencies of state(old) that the C-grid scheme keeps
  // near zero.  out = {ip_cf, |cf|, ip_ke, |ke|, ip_mf, |mf|, ip_ptf, |ptf|},
  // each divided by 4 pi radius^2 (the |.| entries sum absolute terms, for scale).
  void space_identities(double out[8]) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const gmc::Grid &g = G();
    State &s = state[old_i];
    Tend &t = tend[0];
    space_operators_fwd(s, t, cfg.dt_dyn);
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    auto add = [&](int q, double x) { v[q] += x; v[q + 1] += std::fabs(x); };
    for (int k = 1; k <= nlev; ++k) {
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) {
          add(0, t.qhv(i, j, k) * s.mfx_lon(i, j, k) * g.area_lon[j]);
          add(2, t.dkedlon(i, j, k) * s.mfx_lon(i, j, k) * g.area_lon[j] * 2);
        }
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) {
          add(0, -t.qhu(i, j, k) * s.mfy_lat(i, j, k) * g.area_lat[j]);
          add(2, t.dkedlat(i, j, k) * s.mfy_lat(i, j, k) * g.area_lat[j] * 2);
        }
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) {
          add(2, (t.dmfdlon(i, j, k) + t.dmfdlat(i, j, k)) * s.ke(i, j, k) * g.area_cell[j]);
          add(4, (t.dmfdlon(i, j, k) + t.dmfdlat(i, j, k)) * g.area_cell[j]);
          if (hydrostatic) add(6, (t.dptfdlon(i, j, k) + t.dptfdlat(i, j, k) + t.dptfdlev(i, j, k)) * g.area_cell[j]);
        }
    }
    const double pi = std::atan(1.0) * 4.0, a = 4 * pi * cfg.radius * cfg.radius;
    for (int q = 0; q < 8; ++q) out[q] = v[q] / a;
  }

  // smag_damp_run (smag_damp_mod.F90:52-190); decay_from_top = 1 (:36)
  void smag_damp_run(State &s, double dt) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const gmc::Grid &g = G();
    Arr &u = s.u_lon, &v = s.v_lat, &st = s.smag_t, &ss = s.smag_s, &kl = s.kmh_lon, &kt = s.kmh_lat;
    Arr &du = s.smag_dudt, &dv = s.smag_dvdt;
    const double coef = cfg.smag_damp_coef, decay = 1.0;
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i)
          st(i, j, k) = (u(i, j, k) - u(i - 1, j, k)) / g.de_lon[j] -
                        (v(i, j, k) * g.half_cos_lat[j] - v(i, j - 1, k) * g.half_cos_lat[j - 1]) / g.le_lon[j] /
                            g.full_cos_lat[j];
    fill_halo(st, true, false, true, false, true);
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i)
          ss(i, j, k) = (v(i + 1, j, k) - v(i, j, k)) / g.le_lat[j] +
                        (u(i, j + 1, k) * g.full_cos_lat[j + 1] - u(i, j, k) * g.full_cos_lat[j]) / g.de_lat[j] /
                            g.half_cos_lat[j];
    fill_halo(ss, false, true, false, true, false);
    auto sq = [](double x) { return x * x; };
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j) {
        const double ls2 = coef / (1 / sq(g.de_lon[j]) + 1 / sq(g.le_lon[j])) * decay;
        for (int i = 1; i <= nlon; ++i)
          kl(i, j, k) = ls2 * std::sqrt(0.5 * (sq(st(i, j, k)) + sq(st(i + 1, j, k))) +
                                        0.5 * (sq(ss(i, j, k)) + sq(ss(i, j - 1, k))));
      }
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j) {
        const double ls2 = coef / (1 / sq(g.le_lat[j]) + 1 / sq(g.de_lat[j])) * decay;
        for (int i = 1; i <= nlon; ++i)
          kt(i, j, k) = ls2 * std::sqrt(0.5 * (sq(st(i, j, k)) + sq(st(i, j + 1, k))) +
                                        0.5 * (sq(ss(i, j, k)) + sq(ss(i - 1, j, k))));
      }
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i)
          du(i, j, k) = kl(i, j, k) * ((u(i - 1, j, k) - 2 * u(i, j, k) + u(i + 1, j, k)) / sq(g.de_lon[j]) +
                                       ((u(i, j + 1, k) - u(i, j, k)) / g.de_lat[j] * g.half_cos_lat[j] -
                                        (u(i, j, k) - u(i, j - 1, k)) / g.de_lat[j - 1] * g.half_cos_lat[j - 1]) /
                                           g.le_lon[j] / g.full_cos_lat[j]);
    for (int k = 1; k <= nlev; ++k)
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) u(i, j, k) = u(i, j, k) + dt * du(i, j, k);
    fill_halo(u, true);
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j) {
        const bool edge = j == 1 || j == nhalf;
        for (int i = 1; i <= nlon; ++i) {
          double t = (v(i - 1, j, k) - 2 * v(i, j, k) + v(i + 1, j, k)) / sq(g.le_lat[j]);
          if (!edge)
            t = t + ((v(i, j + 1, k) - v(i, j, k)) / g.le_lon[j + 1] * g.full_cos_lat[j + 1] -
                     (v(i, j, k) - v(i, j - 1, k)) / g.le_lon[j] * g.full_cos_lat[j]) /
                        g.de_lat[j] / g.half_cos_lat[j];
          dv(i, j, k) = kt(i, j, k) * t;
        }
      }
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) v(i, j, k) = v(i, j, k) + dt * dv(i, j, k);
    fill_halo(v, false);
  }

  // held_suarez_test_apply_forcing (held_suarez_test_mod.F90:74-112) on the
  // new state, whose ph and t the last stage's backward pass left
  void held_suarez_forcing(State &s, double dt) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const gmc::Grid &g = G();
    const double sig_b = 0.7, kf = 1.0 / 86400.0, ka = 0.025 / 86400.0, ks = 0.25 / 86400.0;
    const double dt_lat = 60.0, dpt_lev = 10.0, p0 = 1.0e5;
    for (int k = 1; k <= nlev; ++k) {
      const double kv = kf * std::max(0.0, (g.full_lev[k - 1] - sig_b) / (1.0 - sig_b));
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) s.u_lon(i, j, k) = s.u_lon(i, j, k) - dt * kv * s.u_lon(i, j, k);
    }
    fill_halo(s.u_lon, true);
    for (int k = 1; k <= nlev; ++k) {
      const double kv = kf * std::max(0.0, (g.full_lev[k - 1] - sig_b) / (1.0 - sig_b));
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) s.v_lat(i, j, k) = s.v_lat(i, j, k) - dt * kv * s.v_lat(i, j, k);
    }
    fill_halo(s.v_lat, false);
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j) {
        const double c = g.full_cos_lat[j], sn = g.full_sin_lat[j];
        const double c2 = c * c, c4 = c2 * c2;   // cos**2, cos**4
        const double kt = ka + (ks - ka) * std::max(0.0, (g.full_lev[k - 1] - sig_b) / (1.0 - sig_b)) * c4;
        for (int i = 1; i <= nlon; ++i) {
          const double p_p0 = s.ph(i, j, k) / p0;
          const double teq = std::max(200.0, (315.0 - dt_lat * (sn * sn) - dpt_lev * std::log(p_p0) * c2) *
                                                 std::pow(p_p0, Rd_o_cpd));
          s.pt(i, j, k) = s.pt(i, j, k) - dt * kt * s.pt(i, j, k) * (1.0 - teq / s.t(i, j, k));
        }
      }
    fill_halo(s.pt, true);
  }

  void time_integrate() {
    const double dt = cfg.dt_dyn;
    const int o = old_i, n = new_i, t3 = 3 - o - n;
    switch (cfg.time_scheme) {
      case GMC_TIME_EULER:
        step_fb(o, o, n, o, n, dt);
        break;
      case GMC_TIME_PC2:
        step_fb(o, o, n, o, n, dt / 2.0);
        step_fb(o, n, t3, o, n, dt / 2.0);
        step_fb(o, t3, n, o, n, dt);
        break;
      default:
        step_fb(o, o, n, o, n, dt / 3.0);
        step_fb(o, n, t3, o, n, dt / 2.0);
        step_fb(o, t3, n, o, n, dt);
        break;
    }
    if (cfg.forcing == GMC_FORCING_HELD_SUAREZ) held_suarez_forcing(state[n], dt);   // test_forcing_run (gmcore_mod.F90:586)
    if (cfg.use_div_damp) div_damp_run(state[n]);   // damp_run (damp_mod.F90:49-63)
    if (cfg.use_smag_damp) smag_damp_run(state[n], dt);
    adv_run(state[n]);
    // time_advance (time_mod.F90:128-159)
    if (alert_ringing) { alert_last_time = curr_time; alert_ringing = false; }
    std::swap(old_i, new_i);
    time_step += 1;
    curr_time += dt;
  }

  // diagnose (gmcore_mod.F90:213-341)
  void diagnose(double out[8]) {
    const int nlon = mesh.nlon, nlev = mesh.nlev, nhalf = mesh.nhalf, nlat = mesh.nlat;
    const gmc::Grid &g = G();
    State &s = state[old_i];
    double tm = 0, te_ke = 0, te_ie = 0, te_pe = 0, tav = 0, tpe = 0, tpt = 0;
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) tm = tm + s.m(i, j, k) * g.area_cell[j];
    for (int k = 1; k <= nlev; ++k) {
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i) te_ke = te_ke + s.mfx_lon(i, j, k) * 0.5 * s.u_lon(i, j, k) * g.area_lon[j] * 2;
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) te_ke = te_ke + s.mfy_lat(i, j, k) * 0.5 * s.v_lat(i, j, k) * g.area_lat[j] * 2;
    }
    if (baroclinic) {
      for (int k = 1; k <= nlev; ++k)
        for (int j = 1; j <= nlat; ++j)
          for (int i = 1; i <= nlon; ++i) te_ie = te_ie + s.m(i, j, k) * cfg.cpd * s.t(i, j, k) * g.area_cell[j];
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) te_pe = te_pe + gzs(i, j, 1) * s.phs(i, j, 1) * g.area_cell[j];
    } else {
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i)
          te_pe = te_pe + (s.m(i, j, 1) * s.m(i, j, 1) * cfg.g * 0.5 + s.m(i, j, 1) * gzs(i, j, 1)) * g.area_cell[j];
    }
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i) tav = tav + s.pv(i, j, k) * g.area_vtx[j];
    for (int k = 1; k <= nlev; ++k) {
      for (int j = 2; j <= nlat - 1; ++j)
        for (int i = 1; i <= nlon; ++i)
          tpe = tpe + s.m_lon(i, j, k) * (s.pv_lon(i, j, k) * s.pv_lon(i, j, k)) * 0.5 * g.area_lon[j];
      for (int j = 1; j <= nhalf; ++j)
        for (int i = 1; i <= nlon; ++i)
          tpe = tpe + s.m_lat(i, j, k) * (s.pv_lat(i, j, k) * s.pv_lat(i, j, k)) * 0.5 * g.area_lat[j];
    }
    if (baroclinic)
      for (int k = 1; k <= nlev; ++k)
        for (int j = 1; j <= nlat; ++j)
          for (int i = 1; i <= nlon; ++i) tpt = tpt + s.m(i, j, k) * s.pt(i, j, k) * g.area_cell[j];
    out[0] = tm; out[1] = te_ke + te_ie + te_pe; out[2] = te_ke; out[3] = te_ie; out[4] = te_pe;
    out[5] = tav; out[6] = tpe; out[7] = tpt;
  }
};

}  // namespace orc

// ---------------------------------------------------------------------------
// C interface for the test harness (ctypes).
// Exchange layout: interior points only, C order [k][j][i].
// ---------------------------------------------------------------------------
extern "C" {

void *orc_create(const gmc_config *cfg, char *errbuf, int errlen) {
  orc::Model *m = new orc::Model();
  std::string e = m->init(*cfg);
  if (!e.empty()) {
    if (errbuf && errlen > 0) snprintf(errbuf, errlen, "%s", e.c_str());
    delete m;
    return nullptr;
  }
  return m;
}

void orc_destroy(void *h) { delete (orc::Model *)h; }

// The seeded synthetic initial state of a benchmark configuration, from the
// oracle's own build of the host set-up code (so that a CPU-only caller, such
// as the timed CPU baseline, needs no other library).  Arguments as
// gmc_make_ic: kind 1 shallow water, kind 2 baroclinic; interior arrays in C
// order [k][j][i]; a null pointer skips that field.
int orc_make_ic(const gmc_config *cfg, int kind, uint64_t seed, double noise_k, double *u_lon, double *v_lat,
                double *pt_or_gz, double *phs, double *gzs, double *q) {
  if (!cfg) return GMC_EINVAL;
  gmc_config cc = *cfg;
  if (!cc.baroclinic) cc.ke_scheme = 1;
  if (!(cc.dt_adv > 0)) cc.dt_adv = cc.dt_dyn;
  gmc::Grid g;
  if (!g.build(cc).empty()) return GMC_EINVAL;
  return gmc::make_ic(g, kind, seed, noise_k, u_lon, v_lat, pt_or_gz, phs, gzs, q).empty() ? GMC_OK : GMC_EINVAL;
}

int orc_lon_halo_width(void *h) { return ((orc::Model *)h)->mesh.hx; }

static orc::Arr *orc_field(orc::Model *m, orc::State &s, const char *name, int &nrow, int &k0, int &k1) {
  const int nlat = m->mesh.nlat, nhalf = m->mesh.nhalf, nlev = m->mesh.nlev;
  std::string n(name);
  nrow = nlat; k0 = 1; k1 = nlev;
  struct E { const char *name; orc::Arr *a; int lat; int lev; };   // lat: 0 full 1 half; lev: 0 full 1 half 2 two-d
  E tab[] = {{"u_lon", &s.u_lon, 0, 0}, {"v_lat", &s.v_lat, 1, 0}, {"u_f", &s.u_f, 0, 0}, {"v_f", &s.v_f, 1, 0},
             {"pt", &s.pt, 0, 0}, {"gz", &s.gz, 0, 0}, {"gz_f", &s.gz_f, 0, 0}, {"phs", &s.phs, 0, 2},
             {"phs_f", &s.phs_f, 0, 2}, {"gzs", &m->gzs, 0, 2}, {"m", &s.m, 0, 0}, {"t", &s.t, 0, 0},
             {"pv", &s.pv, 1, 0}, {"ke", &s.ke, 0, 0}, {"pv_lon", &s.pv_lon, 0, 0}, {"pv_lat", &s.pv_lat, 1, 0},
             {"mfx_lon", &s.mfx_lon, 0, 0}, {"mfy_lat", &s.mfy_lat, 1, 0}, {"u_lat", &s.u_lat, 1, 0},
             {"v_lon", &s.v_lon, 0, 0}, {"we_lev", &s.we_lev, 0, 1}, {"m_lev", &s.m_lev, 0, 1},
             {"gz_lev", &s.gz_lev, 0, 1}, {"ph_lev", &s.ph_lev, 0, 1}, {"ph_exn_lev", &s.ph_exn_lev, 0, 1},
             {"vor", &s.vor, 1, 0}};
  for (E &e : tab)
    if (n == e.name) {
      if (!e.a->ok()) return nullptr;
      nrow = e.lat ? nhalf : nlat;
      if (e.lev == 1) { k0 = 1; k1 = nlev + 1; }
      if (e.lev == 2) { k0 = 1; k1 = 1; }
      return e.a;
    }
  return nullptr;
}

int orc_set_field(void *h, const char *name, const double *src) {
  orc::Model *m = (orc::Model *)h;
  orc::State &s = m->state[m->old_i];
  int nrow, k0, k1;
  orc::Arr *a = orc_field(m, s, name, nrow, k0, k1);
  if (!a) return GMC_EINVAL;
  const int nlon = m->mesh.nlon;
  size_t o = 0;
  for (int k = k0; k <= k1; ++k)
    for (int j = 1; j <= nrow; ++j)
      for (int i = 1; i <= nlon; ++i) (*a)(i, j, k) = src[o++];
  // set_ic routines fill all halos after assigning the interior
  m->fill_halo(*a, nrow == m->mesh.nlat);
  return GMC_OK;
}

int orc_get_field(void *h, const char *name, double *dst) {
  orc::Model *m = (orc::Model *)h;
  orc::State &s = m->state[m->old_i];
  int nrow, k0, k1;
  orc::Arr *a = orc_field(m, s, name, nrow, k0, k1);
  if (!a) return GMC_EINVAL;
  const int nlon = m->mesh.nlon;
  size_t o = 0;
  for (int k = k0; k <= k1; ++k)
    for (int j = 1; j <= nrow; ++j)
      for (int i = 1; i <= nlon; ++i) dst[o++] = (*a)(i, j, k);
  return GMC_OK;
}

int orc_set_tracer(void *h, int l, const double *src) {
  orc::Model *m = (orc::Model *)h;
  if (!m->has_tracers || l < 0 || l >= m->cfg.ntracer) return GMC_EINVAL;
  const int nlon = m->mesh.nlon, nlat = m->mesh.nlat, nlev = m->mesh.nlev;
  // Both time levels start from the initial mixing ratio (the reference
  // leaves the second level uninitialised, adv_mod.F90:390).
  for (int s = 0; s < 2; ++s) {
    orc::Arr &q = m->tracers.q[s][l];
    #pragma omp parallel for schedule(static)
    for (int k = 1; k <= nlev; ++k) {
      size_t o = (size_t)(k - 1) * nlat * nlon;   // each level from its own offset
      for (int j = 1; j <= nlat; ++j)
        for (int i = 1; i <= nlon; ++i) q(i, j, k) = src[o++];
    }
    m->fill_halo(q, true);
  }
  return GMC_OK;
}

int orc_get_tracer(void *h, int l, double *dst) {
  orc::Model *m = (orc::Model *)h;
  if (!m->has_tracers || l < 0 || l >= m->cfg.ntracer) return GMC_EINVAL;
  const int nlon = m->mesh.nlon, nlat = m->mesh.nlat, nlev = m->mesh.nlev;
  orc::Arr &q = m->tracers.q[m->tracers.old_idx][l];
  #pragma omp parallel for schedule(static)
  for (int k = 1; k <= nlev; ++k) {
    size_t o = (size_t)(k - 1) * nlat * nlon;
    for (int j = 1; j <= nlat; ++j)
      for (int i = 1; i <= nlon; ++i) dst[o++] = q(i, j, k);
  }
  return GMC_OK;
}

int orc_prepare(void *h, char *errbuf, int errlen) {
  orc::Model *m = (orc::Model *)h;
  m->prepare();
  if (m->err.code && errbuf) snprintf(errbuf, errlen, "%s", m->err.msg.c_str());
  return m->err.code;
}

int orc_step(void *h, int nsteps, char *errbuf, int errlen) {
  orc::Model *m = (orc::Model *)h;
  for (int n = 0; n < nsteps && m->err.code == 0; ++n) m->time_integrate();
  if (m->err.code && errbuf) snprintf(errbuf, errlen, "%s", m->err.msg.c_str());
  return m->err.code;
}

int orc_space_identities(void *h, double *out) {
  ((orc::Model *)h)->space_identities(out);
  return 0;
}

// One pass of the space operators on state(old), for the known-answer tests:
// pass 0 the forward pass (space_operators_fwd) into tend[0]; pass 1 the
// backward pass's prepare (calc_ph, calc_t, calc_gz_lev, calc_m) and the
// pressure-gradient force into tend[1]; pass 2 the divergence damping of
// u_lon, v_lat (div_damp_run, div_damp_mod.F90:89-139).
int orc_run_pass(void *h, int pass) {
  orc::Model *m = (orc::Model *)h;
  orc::State &s = m->state[m->old_i];
  if (pass == 0) {
    m->space_operators_fwd(s, m->tend[0], m->cfg.dt_dyn);
  } else if (pass == 1) {
    m->operators_prepare_bwd(s);
    m->pgf_run(s, m->tend[1]);
  } else if (pass == 2) {
    m->div_damp_run(s);
  } else {
    return GMC_EINVAL;
  }
  return m->err.code;
}

// A tendency of tend[pass] by name, interior-only [k][j][i] (dphs: [j][i]).
int orc_get_tend(void *h, int pass, const char *name, double *dst) {
  orc::Model *m = (orc::Model *)h;
  if (pass < 0 || pass > 1) return GMC_EINVAL;
  orc::Tend &t = m->tend[pass];
  const int nlat = m->mesh.nlat, nhalf = m->mesh.nhalf, nlev = m->mesh.nlev;
  struct T { const char *name; orc::Arr *a; int nrow, nk; };
  const T tab[] = {{"du", &t.du, nlat, nlev},           {"dv", &t.dv, nhalf, nlev},
                   {"dgz", &t.dgz, nlat, nlev},         {"dpt", &t.dpt, nlat, nlev},
                   {"dphs", &t.dphs, nlat, 1},          {"qhu", &t.qhu, nhalf, nlev},
                   {"qhv", &t.qhv, nlat, nlev},         {"dkedlon", &t.dkedlon, nlat, nlev},
                   {"dkedlat", &t.dkedlat, nhalf, nlev}, {"dmfdlon", &t.dmfdlon, nlat, nlev},
                   {"dmfdlat", &t.dmfdlat, nlat, nlev}, {"dptfdlon", &t.dptfdlon, nlat, nlev},
                   {"dptfdlat", &t.dptfdlat, nlat, nlev}, {"dptfdlev", &t.dptfdlev, nlat, nlev},
                   {"pgf_lon", &t.pgf_lon, nlat, nlev}, {"pgf_lat", &t.pgf_lat, nhalf, nlev},
                   {"wedudlev", &t.wedudlev, nlat, nlev}, {"wedvdlev", &t.wedvdlev, nhalf, nlev}};
  for (const T &e : tab) {
    if (std::strcmp(name, e.name)) continue;
    size_t o = 0;
    for (int k = 1; k <= e.nk; ++k)
      for (int j = 1; j <= e.nrow; ++j)
        for (int i = 1; i <= m->mesh.nlon; ++i) dst[o++] = (*e.a)(i, j, k);
    return GMC_OK;
  }
  return GMC_EINVAL;
}

// A field of the dynamic mass batch (adv_batch_mass) as the last pass left it,
// interior-only [k][j][i]: the winds u, v it holds, the Courant numbers cflx,
// cfly and the axis divergences divx, divy (adv_batch_mod.F90:218-377); on
// half levels the vertical mass flux we, the half-level mass m_lev and the
// vertical Courant number cflz (:493-632); the FFSL intermediates qx, qy of
// the last horizontal flux (ffsl_mod.F90:353-406).
static int get_batch_field(orc::Model *m, orc::Batch &b, const char *name, double *dst) {
  const int nlat = m->mesh.nlat, nhalf = m->mesh.nhalf, nlev = m->mesh.nlev;
  struct T { const char *name; orc::Arr *a; int nrow, nk; };
  const T tab[] = {{"u", &b.u, nlat, nlev},          {"v", &b.v, nhalf, nlev},
                   {"mfx", &b.mfx, nlat, nlev},      {"mfy", &b.mfy, nhalf, nlev},
                   {"cflx", &b.cflx, nlat, nlev},    {"cfly", &b.cfly, nhalf, nlev},
                   {"divx", &b.divx, nlat, nlev},    {"divy", &b.divy, nlat, nlev},
                   {"we", &b.we, nlat, nlev + 1},    {"m_lev", &b.m_lev, nlat, nlev + 1},
                   {"cflz", &b.cflz, nlat, nlev + 1}, {"qx", &b.qx, nlat, nlev},
                   {"qy", &b.qy, nlat, nlev},        {"old_m", &b.old_m, nlat, nlev}};
  for (const T &e : tab) {
    if (std::strcmp(name, e.name)) continue;
    size_t o = 0;
    for (int k = 1; k <= e.nk; ++k)
      for (int j = 1; j <= e.nrow; ++j)
        for (int i = 1; i <= m->mesh.nlon; ++i) dst[o++] = (*e.a)(i, j, k);
    return GMC_OK;
  }
  return GMC_EINVAL;
}

int orc_get_batch(void *h, const char *name, double *dst) {
  orc::Model *m = (orc::Model *)h;
  return get_batch_field(m, m->mass, name, dst);
}

// The same fields of the static tracer batch (adv_mod.F90:152-312), with its
// previous layer mass old_m.
int orc_get_tracer_batch(void *h, const char *name, double *dst) {
  orc::Model *m = (orc::Model *)h;
  if (!m->has_tracers) return GMC_EINVAL;
  return get_batch_field(m, m->tracers, name, dst);
}

// Tracer l of time level lev (0 the batch's old level, 1 its new level) with
// two longitude-halo columns on each side as the level holds them now,
// [k][j][nlon + 4] from i = -1.
int orc_get_tracer_level(void *h, int l, int lev, double *dst) {
  orc::Model *m = (orc::Model *)h;
  if (!m->has_tracers || l < 0 || l >= m->cfg.ntracer || lev < 0 || lev > 1) return GMC_EINVAL;
  orc::Batch &b = m->tracers;
  orc::Arr &q = b.q[lev == 0 ? b.old_idx : b.new_idx][l];
  size_t o = 0;
  for (int k = 1; k <= m->mesh.nlev; ++k)
    for (int j = 1; j <= m->mesh.nlat; ++j)
      for (int i = -1; i <= m->mesh.nlon + 2; ++i) dst[o++] = q(i, j, k);
  return GMC_OK;
}

// One piece of the tracer step applied to a given cell field, for the
// known-answer tests: which 0 the zonal negative fixer, 1 the vertical
// negative fixer (with layer masses m), 2 three passes of the order-2 zonal
// smoother.  q (in/out) and m interior-only [k][j][i]; their halos are filled
// from the interior before the call, and what a fixer writes into a halo
// cell is dropped, as the reference's next fill_halo drops it.
int orc_tracer_piece(void *h, int which, double *q, const double *mass) {
  orc::Model *m = (orc::Model *)h;
  const int nlon = m->mesh.nlon, nlat = m->mesh.nlat, nlev = m->mesh.nlev;
  orc::Fields F{&m->mesh};
  orc::Arr qa, ma;
  F.cell3(qa);
  F.cell3(ma);
  size_t o = 0;
  for (int k = 1; k <= nlev; ++k)
    for (int j = 1; j <= nlat; ++j)
      for (int i = 1; i <= nlon; ++i, ++o) {
        qa(i, j, k) = q[o];
        ma(i, j, k) = mass[o];
      }
  m->fill_halo(qa, true);
  m->fill_halo(ma, true);
  m->err = {};
  if (which == 0) {
    m->zonal_fixer(qa, ma);
  } else if (which == 1) {
    m->vertical_fixer(qa, ma);
  } else if (which == 2) {
    for (int it = 0; it < 3; ++it) m->lon_damp_on_cell(qa);
  } else {
    return GMC_EINVAL;
  }
  o = 0;
  for (int k = 1; k <= nlev; ++k)
    for (int j = 1; j <= nlat; ++j)
      for (int i = 1; i <= nlon; ++i) q[o++] = qa(i, j, k);
  return m->err.code;
}

int orc_diagnose(void *h, double *out) {
  ((orc::Model *)h)->diagnose(out);
  return GMC_OK;
}

// History diagnostics of state(old), interior-only [k][j][i] (null: skipped):
// ph, t, z = gz / g and div at cells, vor at vertices (half rows).  Shallow
// water: z = gz / g of the state, div and vor; ph and t unused.
int orc_output_diag(void *h, double *ph, double *t, double *z, double *div, double *vor) {
  orc::Model *m = (orc::Model *)h;
  orc::State d = m->output_state();
  const int nlon = m->mesh.nlon, nlat = m->mesh.nlat, nhalf = m->mesh.nhalf, nlev = m->mesh.nlev;
  const double g = m->cfg.g;
  size_t o = 0, ov = 0;
  for (int k = 1; k <= nlev; ++k)
    for (int j = 1; j <= nlat; ++j)
      for (int i = 1; i <= nlon; ++i, ++o) {
        if (m->baroclinic) {
          if (ph) ph[o] = d.ph(i, j, k);
          if (t) t[o] = d.t(i, j, k);
        }
        if (z) z[o] = d.gz(i, j, k) / g;
        if (div) div[o] = d.div(i, j, k);
      }
  for (int k = 1; k <= nlev; ++k)
    for (int j = 1; j <= nhalf; ++j)
      for (int i = 1; i <= nlon; ++i, ++ov)
        if (vor) vor[ov] = d.vor(i, j, k);
  return GMC_OK;
}

// One horizontal FFSL flux (ffsl_calc_tracer_hflx_cell) of field q with the
// given batch fields; inputs and outputs interior-only [k][j][i].
int orc_ffsl_hflx(void *h, const double *q, const double *u, const double *v, const double *mfx, const double *mfy,
                  const double *cflx, const double *cfly, const double *divx, const double *divy, double dt,
                  double *qmfx, double *qmfy) {
  orc::Model *m = (orc::Model *)h;
  const int nlon = m->mesh.nlon, nlat = m->mesh.nlat, nhalf = m->mesh.nhalf, nlev = m->mesh.nlev;
  orc::Fields F{&m->mesh};
  orc::Batch b;
  m->alloc_batch(b, dt, true, 0);
  orc::Arr qa, fx, fy;
  F.cell3(qa); F.lon3(fx); F.lat3(fy);
  auto load = [&](orc::Arr &a, const double *src, int nrow, bool full) {
    size_t o = 0;
    for (int k = 1; k <= nlev; ++k)
      for (int j = 1; j <= nrow; ++j)
        for (int i = 1; i <= nlon; ++i) a(i, j, k) = src[o++];
    m->fill_halo(a, full);
  };
  load(qa, q, nlat, true); load(b.u, u, nlat, true); load(b.v, v, nhalf, false);
  load(b.mfx, mfx, nlat, true); load(b.mfy, mfy, nhalf, false);
  load(b.cflx, cflx, nlat, true); load(b.cfly, cfly, nhalf, false);
  load(b.divx, divx, nlat, true); load(b.divy, divy, nlat, true);
  m->tracer_hflx_cell(b, qa, fx, fy, dt);
  size_t o = 0;
  for (int k = 1; k <= nlev; ++k)
    for (int j = 1; j <= nlat; ++j)
      for (int i = 1; i <= nlon; ++i) qmfx[o++] = fx(i, j, k);
  o = 0;
  for (int k = 1; k <= nlev; ++k)
    for (int j = 1; j <= nhalf; ++j)
      for (int i = 1; i <= nlon; ++i) qmfy[o++] = fy(i, j, k);
  return m->err.code;
}

// Mesh/filter queries for the known-answer tests.  Besides the per-row
// tables, the vertical coordinate: the hybrid coefficients hyai, hybi (the
// template's tables) and hyam, hybm, and the eta levels full_lev = hyam + hybm,
// half_lev = hyai + hybi (hybrid_coord_mod.F90:121-132); the divergence-damping
// coefficients c_lon, c_lat by level (div_damp_mod.F90:27-80, [k][j]); the
// zonal smoother's weights (lon_damp_mod.F90:43-68).
int orc_metric(void *h, const char *name, double *out, int n) {
  orc::Model *m = (orc::Model *)h;
  const gmc::Grid &g = m->grid;
  struct V { const char *name; const std::vector<double> *v; };
  const V vecs[] = {{"full_lev", &g.full_lev},
                    {"half_lev", &g.half_lev},
                    {"hyai", &g.hyai},
                    {"hybi", &g.hybi},
                    {"hyam", &g.hyam},
                    {"hybm", &g.hybm},
                    {"div_c_lon", &g.div_c_lon},
                    {"div_c_lat", &g.div_c_lat},
                    {"lon_damp_wgt_full", &g.lon_damp_wgt_full},
                    {"lon_damp_wgt_half", &g.lon_damp_wgt_half}};
  const std::vector<double> *lev = nullptr;
  for (const V &e : vecs)
    if (!std::strcmp(name, e.name)) lev = e.v;
  if (lev) {
    if (n != (int)lev->size()) return GMC_EINVAL;
    for (int k = 0; k < n; ++k) out[k] = (*lev)[k];
    return GMC_OK;
  }
  const gmc::RowTable *t = m->grid.metric(name);
  if (!t) return GMC_EINVAL;
  for (int j = 1; j <= n; ++j) out[j - 1] = (*t)[j];
  return GMC_OK;
}

// Normalised weights of one polar-filter row (which: 0 big, 1 small1,
// 2 small2; lat: 0 full, 1 half latitudes; j 1-based); n must equal the
// row's tap count.
int orc_filter_weights(void *h, int which, int lat, int j, double *out, int n) {
  orc::Model *m = (orc::Model *)h;
  const gmc::Filter &f = which == 0 ? m->grid.big : which == 1 ? m->grid.small1 : m->grid.small2;
  const std::vector<std::vector<double>> &w = lat ? f.wgt_half : f.wgt_full;
  if (j < 1 || j > (int)w.size() || n != (int)w[j - 1].size()) return GMC_EINVAL;
  for (int t = 0; t < n; ++t) out[t] = w[j - 1][t];
  return GMC_OK;
}

int orc_filter_taps(void *h, int which, int lat, int *out) {
  orc::Model *m = (orc::Model *)h;
  const gmc::Filter &f = which == 0 ? m->grid.big : which == 1 ? m->grid.small1 : m->grid.small2;
  const std::vector<int> &v = lat ? f.ngrid_half : f.ngrid_full;
  for (size_t j = 0; j < v.size(); ++j) out[j] = v[j];
  return GMC_OK;
}

}  // extern "C"
