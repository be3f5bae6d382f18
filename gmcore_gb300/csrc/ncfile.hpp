// netCDF classic files (CDF-1 and the 64-bit-offset CDF-2), written and read
// without the netCDF library.
//
// The reference writes its history and restart files through the fiona
// library (src/utils/history_mod.F90, src/utils/restart_mod.F90), a wrapper of
// netCDF.  This is a self-contained codec of the published classic format:
// a big-endian header (magic "CDF" + version, record count, dimension,
// global-attribute and variable lists, each variable with its dimension ids,
// attributes, type, byte size and file offset) followed by the fixed-size
// variables and then the record variables interleaved record by record.
// One dimension may be unlimited (the record dimension, here "time").
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace gmc {
namespace nc {

enum Type : int32_t { BYTE = 1, CHAR = 2, SHORT = 3, INT = 4, FLOAT = 5, DOUBLE = 6 };

struct Dim {
  std::string name;
  uint64_t len = 0;   // 0: the unlimited (record) dimension
};

struct Att {
  std::string name;
  Type type = CHAR;
  std::string text;          // CHAR
  std::vector<double> num;   // numeric types, stored as `type`
};

struct Var {
  std::string name;
  std::vector<int> dims;   // dimension ids, slowest first (the record dimension first if any)
  std::vector<Att> atts;
  Type type = DOUBLE;
  uint64_t vsize = 0;   // bytes of the variable (fixed) or of one record of it, padded to 4
  uint64_t begin = 0;   // file offset of its data (of record 0 for record variables)
  bool record = false;
  uint64_t count = 0;   // values of the variable (fixed) or of one record
};

struct Header {
  int version = 2;        // 1: CDF-1 (32-bit offsets), 2: CDF-2 (64-bit offsets)
  uint64_t numrecs = 0;
  std::vector<Dim> dims;
  std::vector<Att> gatts;
  std::vector<Var> vars;
  uint64_t recsize = 0;   // bytes of one record of all record variables

  int dim(const std::string &name) const;
  int var(const std::string &name) const;
  const Att *att(int var, const std::string &name) const;   // var < 0: global
  // Sizes and offsets of every variable from the definitions, in the order the
  // variables were added: fixed variables first, then the records.
  std::string layout();
  std::vector<uint8_t> encode() const;
  // Parses a header; returns "" or a message.  `need` receives the number of
  // bytes still missing when `n` is too short.
  static std::string decode(const uint8_t *p, size_t n, Header &h, size_t &need);
};

size_t type_size(Type t);

// One open netCDF classic file.
class File {
 public:
  Header h;
  File() = default;
  File(const File &) = delete;
  File &operator=(const File &) = delete;
  ~File();
  // Writes the header of a new file (replacing any file at `path`).
  std::string create(const std::string &path, Header hdr);
  // Opens an existing file and reads its header; `update` opens it for
  // writing more records.
  std::string open(const std::string &path, bool update);
  // Writes a fixed variable whole (rec ignored) or record `rec` of a record
  // variable from FP64 values, converted to the variable's type.  Writing
  // record numrecs or beyond extends the record count.
  std::string put(const std::string &var, uint64_t rec, const double *src);
  // Reads a fixed variable or one record of a record variable as FP64.
  std::string get(const std::string &var, uint64_t rec, double *dst);
  // Writes the record count back into the header and closes the file.
  std::string close();

 private:
  int fd_ = -1;
  bool write_ = false;
  bool dirty_ = false;
  std::string path_;
};

}  // namespace nc
}  // namespace gmc
