// History (h0) and restart (r0) files of a model state in the reference's
// layout, on top of the netCDF classic codec.
//   restart: restart_mod.F90:54-151 (write), :153-251 (read)
//   history: history_mod.F90:125-150 (shallow water), :194-240 (hydrostatic),
//            :398-444, :519-580 (the values written)
// Host arrays are dense FP64 interiors in the library's [k][j][i] order,
// which is netCDF's (time, lev, lat, lon) order of the reference's
// Fortran (lon, lat, lev, time) variables.
#pragma once

#include <string>
#include <vector>

#include "gmcore_gpu.h"
#include "grid.hpp"

namespace gmc {
namespace out {

struct Opts {
  std::string time_units = "hours";
  double unit_seconds = 3600;
  std::string start_time = "2000-01-01 00:00:00";
  std::vector<std::string> tracer_names;
  std::string restart_interval;   // empty: no attribute
};
// Options from the C struct (null: defaults) for a model with ntracer tracers.
std::string parse_opts(const gmc_file_opts *o, int ntracer, Opts &out);

struct State {   // restart variables (read: destinations; null pointers skipped)
  double *u = nullptr, *v = nullptr, *pt = nullptr, *phs = nullptr, *gz = nullptr, *gzs = nullptr;
  std::vector<double *> q;   // per tracer
};

struct History {   // one h0 record
  const double *u = nullptr, *v = nullptr, *pt = nullptr, *phs = nullptr, *gz = nullptr, *gzs = nullptr;
  const double *ph = nullptr, *t = nullptr, *z = nullptr, *div = nullptr, *vor = nullptr, *pv = nullptr;
  std::vector<const double *> q;
  gmc_diag diag{};
};

std::string write_restart(const Grid &g, const std::string &path, double elapsed, const Opts &o, const State &s);
// Reads the first record; tracers whose names the file lacks are left alone
// (found[l] = false).
std::string read_restart(const Grid &g, const std::string &path, const Opts &o, double &elapsed, State &s,
                         std::vector<bool> &found);
// Writes a new history file, or with `append` adds a record to the history
// file at `path` (created when absent).
std::string write_history(const Grid &g, const std::string &path, double elapsed, bool append, const Opts &o,
                          const History &h);

}  // namespace out
}  // namespace gmc
