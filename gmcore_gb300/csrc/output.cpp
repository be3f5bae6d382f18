// History and restart file layouts (see output.hpp).
//
// Names, dimensions, long names and units follow the reference's
// fiona_add_dim / fiona_add_var calls.  Variables the reference declares with
// dtype='r8' are 64-bit; the ones it declares without a type (tm, ph, vor,
// div and the shallow-water zs) are 32-bit, fiona's default type.  The time
// axis is "<units> since <start time>" with the elapsed time in those units
// (the reference passes the history interval's unit and its start time to
// fiona_init).  Restart files also carry the tracers (64-bit, named as in the
// history files), which the reference's restart omits.
#include "output.hpp"

#include <cmath>
#include <cstdio>

#include "ncfile.hpp"

namespace gmc {
namespace out {

namespace {

using nc::Att;
using nc::Header;
using nc::Var;

Att text(const std::string &name, const std::string &v) {
  Att a;
  a.name = name;
  a.type = nc::CHAR;
  a.text = v;
  return a;
}
Att num(const std::string &name, double v) {
  Att a;
  a.name = name;
  a.type = nc::DOUBLE;
  a.num = {v};
  return a;
}

// Dimension ids of the layout built below.
struct Dims {
  int time = -1, lon = -1, lat = -1, ilon = -1, ilat = -1, lev = -1, ilev = -1;
};

Dims add_dims(Header &h, const Grid &g) {
  Dims d;
  auto add = [&](const char *name, uint64_t len) {
    h.dims.push_back({name, len});
    return (int)h.dims.size() - 1;
  };
  d.time = add("time", 0);
  d.lon = add("lon", (uint64_t)g.nlon);
  d.lat = add("lat", (uint64_t)g.nlat);
  d.ilon = add("ilon", (uint64_t)g.nlon);
  d.ilat = add("ilat", (uint64_t)g.nhalf);
  if (g.cfg.baroclinic) {
    d.lev = add("lev", (uint64_t)g.nlev);
    d.ilev = add("ilev", (uint64_t)g.nlev + 1);
  }
  return d;
}

void add_var(Header &h, const std::string &name, std::vector<int> dims, nc::Type type, const std::string &long_name,
             const std::string &units) {
  Var v;
  v.name = name;
  v.dims = std::move(dims);
  v.type = type;
  v.atts = {text("long_name", long_name), text("units", units)};
  h.vars.push_back(std::move(v));
}

// Coordinate variables (add_var=.true. of each dimension).
void add_coords(Header &h, const Dims &d, const Opts &o) {
  add_var(h, "time", {d.time}, nc::DOUBLE, "time", o.time_units + " since " + o.start_time);
  add_var(h, "lon", {d.lon}, nc::DOUBLE, "longitude", "degrees_east");
  add_var(h, "lat", {d.lat}, nc::DOUBLE, "latitude", "degrees_north");
  add_var(h, "ilon", {d.ilon}, nc::DOUBLE, "half longitude", "degrees_east");
  add_var(h, "ilat", {d.ilat}, nc::DOUBLE, "half latitude", "degrees_north");
  if (d.lev >= 0) {
    add_var(h, "lev", {d.lev}, nc::DOUBLE, "full level", "1");
    add_var(h, "ilev", {d.ilev}, nc::DOUBLE, "half level", "1");
  }
}

std::string put_coords(nc::File &f, const Grid &g) {
  std::vector<double> a((size_t)std::max(g.nlon, g.nlat + 1) + (size_t)g.nlev + 2);
  std::string e;
  for (int i = 0; i < g.nlon; ++i) a[(size_t)i] = g.full_lon[(size_t)i] * g.deg;
  if (!(e = f.put("lon", 0, a.data())).empty()) return e;
  for (int i = 0; i < g.nlon; ++i) a[(size_t)i] = g.half_lon[(size_t)i] * g.deg;
  if (!(e = f.put("ilon", 0, a.data())).empty()) return e;
  for (int j = 1; j <= g.nlat; ++j) a[(size_t)j - 1] = g.full_lat_deg[j];
  if (!(e = f.put("lat", 0, a.data())).empty()) return e;
  for (int j = 1; j <= g.nhalf; ++j) a[(size_t)j - 1] = g.half_lat_deg[j];
  if (!(e = f.put("ilat", 0, a.data())).empty()) return e;
  if (g.cfg.baroclinic) {
    if (!(e = f.put("lev", 0, g.full_lev.data())).empty()) return e;
    if (!(e = f.put("ilev", 0, g.half_lev.data())).empty()) return e;
  }
  return "";
}

std::string tracer_check(const Grid &g, const Opts &o, size_t given) {
  if (given != 0 && given != (size_t)g.cfg.ntracer) return "tracer array count differs from ntracer";
  if (o.tracer_names.size() != (size_t)g.cfg.ntracer) return "tracer name count differs from ntracer";
  return "";
}

// Seconds per unit of a time axis "<unit> since ..." (fiona's units).
bool unit_of(const std::string &units, std::string &unit, double &sec) {
  const size_t sp = units.find(' ');
  unit = units.substr(0, sp);
  if (unit == "days") sec = 86400;
  else if (unit == "hours") sec = 3600;
  else if (unit == "minutes") sec = 60;
  else if (unit == "seconds") sec = 1;
  else return false;
  return true;
}

}  // namespace

std::string parse_opts(const gmc_file_opts *o, int ntracer, Opts &out) {
  out = Opts();
  if (o && o->time_units && !unit_of(o->time_units, out.time_units, out.unit_seconds))
    return std::string("time_units must be days, hours, minutes or seconds, not '") + o->time_units + "'";
  if (o && o->start_time) out.start_time = o->start_time;
  if (o && o->restart_interval) out.restart_interval = o->restart_interval;
  if (o && o->tracer_names) {
    std::string s = o->tracer_names, cur;
    for (size_t k = 0; k <= s.size(); ++k) {
      if (k == s.size() || s[k] == ',') {
        if (cur.empty()) return "empty tracer name in tracer_names";
        out.tracer_names.push_back(cur);
        cur.clear();
      } else if (s[k] != ' ') {
        cur += s[k];
      }
    }
    if ((int)out.tracer_names.size() != ntracer)
      return "tracer_names lists " + std::to_string(out.tracer_names.size()) + " names for " +
             std::to_string(ntracer) + " tracers";
  } else {
    for (int l = 0; l < ntracer; ++l) out.tracer_names.push_back("q" + std::to_string(l + 1));
  }
  return "";
}

std::string write_restart(const Grid &g, const std::string &path, double elapsed, const Opts &o, const State &s) {
  std::string e = tracer_check(g, o, s.q.size());
  if (!e.empty()) return e;
  const bool bc = g.cfg.baroclinic != 0;
  if (!s.u || !s.v || !s.gzs || (bc ? !s.pt || !s.phs : !s.gz)) return "a restart field is missing";
  Header h;
  h.gatts.push_back(num("time_step_size", g.cfg.dt_dyn));
  if (!o.restart_interval.empty()) h.gatts.push_back(text("restart_interval", o.restart_interval));
  const Dims d = add_dims(h, g);
  add_coords(h, d, o);
  if (bc) {   // restart_mod.F90:82-92
    add_var(h, "u", {d.time, d.lev, d.lat, d.ilon}, nc::DOUBLE, "u wind component", "m s-1");
    add_var(h, "v", {d.time, d.lev, d.ilat, d.lon}, nc::DOUBLE, "v wind component", "m s-1");
    add_var(h, "phs", {d.time, d.lat, d.lon}, nc::DOUBLE, "hydrostatic surface pressure", "Pa");
    add_var(h, "pt", {d.time, d.lev, d.lat, d.lon}, nc::DOUBLE, "potential temperature", "K");
  } else {   // :93-97
    add_var(h, "u", {d.time, d.lat, d.ilon}, nc::DOUBLE, "u wind component", "m s-1");
    add_var(h, "v", {d.time, d.ilat, d.lon}, nc::DOUBLE, "v wind component", "m s-1");
    add_var(h, "gz", {d.time, d.lat, d.lon}, nc::DOUBLE, "geopotential height", "m2 s-2");
  }
  add_var(h, "gzs", {d.time, d.lat, d.lon}, nc::DOUBLE, "surface geopotential height", "m2 s-2");
  const std::vector<int> cell = bc ? std::vector<int>{d.time, d.lev, d.lat, d.lon} : std::vector<int>{d.time, d.lat, d.lon};
  for (const std::string &n : o.tracer_names) add_var(h, n, cell, nc::DOUBLE, n, "");
  nc::File f;
  if (!(e = f.create(path, h)).empty()) return e;
  const double tv = elapsed / o.unit_seconds;
  if (!(e = put_coords(f, g)).empty()) return e;
  if (!(e = f.put("time", 0, &tv)).empty()) return e;
  if (!(e = f.put("u", 0, s.u)).empty()) return e;
  if (!(e = f.put("v", 0, s.v)).empty()) return e;
  if (bc) {
    if (!(e = f.put("phs", 0, s.phs)).empty()) return e;
    if (!(e = f.put("pt", 0, s.pt)).empty()) return e;
  } else if (!(e = f.put("gz", 0, s.gz)).empty()) {
    return e;
  }
  if (!(e = f.put("gzs", 0, s.gzs)).empty()) return e;
  for (size_t l = 0; l < s.q.size(); ++l)
    if (!(e = f.put(o.tracer_names[l], 0, s.q[l])).empty()) return e;
  return f.close();
}

std::string read_restart(const Grid &g, const std::string &path, const Opts &o, double &elapsed, State &s,
                         std::vector<bool> &found) {
  std::string e = tracer_check(g, o, s.q.size());
  if (!e.empty()) return e;
  nc::File f;
  if (!(e = f.open(path, false)).empty()) return e;
  const bool bc = g.cfg.baroclinic != 0;
  // every variable the model needs must be there with this grid's shape
  struct Need {
    const char *name;
    double *dst;
    uint64_t count;
  };
  const uint64_t n3 = (uint64_t)g.nlev * g.nlat * g.nlon, h3 = (uint64_t)g.nlev * g.nhalf * g.nlon,
                 n2 = (uint64_t)g.nlat * g.nlon;
  std::vector<Need> need = {{"u", s.u, bc ? n3 : n2},
                            {"v", s.v, bc ? h3 : (uint64_t)g.nhalf * g.nlon},
                            {"gzs", s.gzs, n2}};
  if (bc) {
    need.push_back({"phs", s.phs, n2});
    need.push_back({"pt", s.pt, n3});
  } else {
    need.push_back({"gz", s.gz, n2});
  }
  if (f.h.numrecs < 1) return "'" + path + "' holds no record";
  for (const Need &n : need) {
    const int vi = f.h.var(n.name);
    if (vi < 0) return "'" + path + "' has no variable '" + n.name + "'";
    const Var &v = f.h.vars[(size_t)vi];
    if (!v.record || v.count != n.count)
      return "variable '" + std::string(n.name) + "' of '" + path + "' does not match this grid";
  }
  const int ti = f.h.var("time");
  elapsed = 0;
  if (ti >= 0) {
    double tv = 0;
    if (!(e = f.get("time", 0, &tv)).empty()) return e;
    const nc::Att *u = f.h.att(ti, "units");
    std::string unit;
    double sec = 1;
    if (u && u->type == nc::CHAR && !unit_of(u->text, unit, sec)) return "'" + path + "': unknown time units '" + u->text + "'";
    elapsed = tv * sec;
  }
  for (const Need &n : need)
    if (n.dst && !(e = f.get(n.name, 0, n.dst)).empty()) return e;
  found.assign(s.q.size(), false);
  for (size_t l = 0; l < s.q.size(); ++l) {
    const int vi = f.h.var(o.tracer_names[l]);
    if (vi < 0) continue;
    found[l] = true;
    const Var &v = f.h.vars[(size_t)vi];
    if (!v.record || v.count != (bc ? n3 : n2)) return "tracer '" + o.tracer_names[l] + "' of '" + path + "' does not match this grid";
    if (s.q[l] && !(e = f.get(o.tracer_names[l], 0, s.q[l])).empty()) return e;
  }
  return f.close();
}

std::string write_history(const Grid &g, const std::string &path, double elapsed, bool append, const Opts &o,
                          const History &hv) {
  std::string e = tracer_check(g, o, hv.q.size());
  if (!e.empty()) return e;
  const bool bc = g.cfg.baroclinic != 0;
  if (!hv.u || !hv.v || !hv.gzs || !hv.z || !hv.div || (bc ? !hv.pt || !hv.phs || !hv.ph || !hv.t || !hv.vor : !hv.pv))
    return "a history field is missing";
  Header h;
  h.gatts.push_back(num("time_step_size", g.cfg.dt_dyn));
  const Dims d = add_dims(h, g);
  add_coords(h, d, o);
  if (bc) {   // history_setup_h0_hydrostatic (history_mod.F90:209-238)
    add_var(h, "tm", {d.time}, nc::FLOAT, "total mass", "m");
    add_var(h, "te", {d.time}, nc::DOUBLE, "total energy", "m4 s-4");
    add_var(h, "tpe", {d.time}, nc::DOUBLE, "total potential enstrophy", "m2 s-5");
    add_var(h, "te_ke", {d.time}, nc::DOUBLE, "total kinetic energy", "");
    add_var(h, "te_ie", {d.time}, nc::DOUBLE, "total internal energy", "");
    add_var(h, "te_pe", {d.time}, nc::DOUBLE, "total potential energy", "");
    add_var(h, "zs", {d.lat, d.lon}, nc::DOUBLE, "surface height", "m");
    add_var(h, "phs", {d.time, d.lat, d.lon}, nc::DOUBLE, "surface hydrostatic pressure", "Pa");
    add_var(h, "u", {d.time, d.lev, d.lat, d.ilon}, nc::DOUBLE, "u wind component", "m s-1");
    add_var(h, "v", {d.time, d.lev, d.ilat, d.lon}, nc::DOUBLE, "v wind component", "m s-1");
    add_var(h, "pt", {d.time, d.lev, d.lat, d.lon}, nc::DOUBLE, "potential temperature", "K");
    add_var(h, "t", {d.time, d.lev, d.lat, d.lon}, nc::DOUBLE, "temperature", "K");
    add_var(h, "z", {d.time, d.lev, d.lat, d.lon}, nc::DOUBLE, "height", "m");
    add_var(h, "ph", {d.time, d.lev, d.lat, d.lon}, nc::FLOAT, "hydrostatic pressure", "Pa");
    add_var(h, "vor", {d.time, d.lev, d.ilat, d.ilon}, nc::FLOAT, "relative vorticity", "s-1");
    add_var(h, "div", {d.time, d.lev, d.lat, d.lon}, nc::FLOAT, "divergence", "s-1");
    for (const std::string &n : o.tracer_names) add_var(h, n, {d.time, d.lev, d.lat, d.lon}, nc::DOUBLE, n, "");
  } else {   // history_setup_h0_swm (history_mod.F90:136-147)
    add_var(h, "tm", {d.time}, nc::FLOAT, "total mass", "m");
    add_var(h, "te", {d.time}, nc::DOUBLE, "total energy", "m4 s-4");
    add_var(h, "tpe", {d.time}, nc::DOUBLE, "total potential enstrophy", "m2 s-5");
    add_var(h, "u", {d.time, d.lat, d.ilon}, nc::DOUBLE, "u wind component", "m s-1");
    add_var(h, "v", {d.time, d.ilat, d.lon}, nc::DOUBLE, "v wind component", "m s-1");
    add_var(h, "z", {d.time, d.lat, d.lon}, nc::DOUBLE, "height", "m");
    add_var(h, "pv", {d.time, d.ilat, d.ilon}, nc::DOUBLE, "potential vorticity", "s-1 m-1");
    add_var(h, "div", {d.time, d.lat, d.lon}, nc::DOUBLE, "divergence", "s-1");
    add_var(h, "zs", {d.lat, d.lon}, nc::FLOAT, "surface height", "m");
  }
  nc::File f;
  uint64_t rec = 0;
  bool fresh = true;
  if (append) {
    if (FILE *probe = std::fopen(path.c_str(), "rb")) {
      std::fclose(probe);
      if (!(e = f.open(path, true)).empty()) return e;
      // the file must hold this layout: the same variables on the same dimensions
      bool same = f.h.vars.size() == h.vars.size() && f.h.dims.size() == h.dims.size();
      for (size_t k = 0; same && k < h.dims.size(); ++k)
        same = f.h.dims[k].name == h.dims[k].name && f.h.dims[k].len == h.dims[k].len;
      for (size_t k = 0; same && k < h.vars.size(); ++k)
        same = f.h.vars[k].name == h.vars[k].name && f.h.vars[k].dims == h.vars[k].dims &&
               f.h.vars[k].type == h.vars[k].type;
      if (!same) return "'" + path + "' is not a history file of this model";
      rec = f.h.numrecs;
      fresh = false;
    }
  }
  if (fresh) {
    if (!(e = f.create(path, h)).empty()) return e;
    if (!(e = put_coords(f, g)).empty()) return e;
    std::vector<double> zs((size_t)g.nlat * g.nlon);
    for (size_t c = 0; c < zs.size(); ++c) zs[c] = hv.gzs[c] / g.cfg.g;
    if (!(e = f.put("zs", 0, zs.data())).empty()) return e;
  }
  const double tv = elapsed / o.unit_seconds;
  if (!(e = f.put("time", rec, &tv)).empty()) return e;
  const double tm = hv.diag.tm, te = hv.diag.te, tpe = hv.diag.tpe;
  if (!(e = f.put("tm", rec, &tm)).empty()) return e;
  if (!(e = f.put("te", rec, &te)).empty()) return e;
  if (!(e = f.put("tpe", rec, &tpe)).empty()) return e;
  if (!(e = f.put("u", rec, hv.u)).empty()) return e;
  if (!(e = f.put("v", rec, hv.v)).empty()) return e;
  if (!(e = f.put("z", rec, hv.z)).empty()) return e;
  if (!(e = f.put("div", rec, hv.div)).empty()) return e;
  if (bc) {
    const double ke = hv.diag.te_ke, ie = hv.diag.te_ie, pe = hv.diag.te_pe;
    if (!(e = f.put("te_ke", rec, &ke)).empty()) return e;
    if (!(e = f.put("te_ie", rec, &ie)).empty()) return e;
    if (!(e = f.put("te_pe", rec, &pe)).empty()) return e;
    if (!(e = f.put("phs", rec, hv.phs)).empty()) return e;
    if (!(e = f.put("pt", rec, hv.pt)).empty()) return e;
    if (!(e = f.put("t", rec, hv.t)).empty()) return e;
    if (!(e = f.put("ph", rec, hv.ph)).empty()) return e;
    if (!(e = f.put("vor", rec, hv.vor)).empty()) return e;
    for (size_t l = 0; l < hv.q.size(); ++l)
      if (!(e = f.put(o.tracer_names[l], rec, hv.q[l])).empty()) return e;
  } else if (!(e = f.put("pv", rec, hv.pv)).empty()) {
    return e;
  }
  return f.close();
}

}  // namespace out
}  // namespace gmc
