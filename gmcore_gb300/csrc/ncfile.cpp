// netCDF classic codec (see ncfile.hpp).  Every multi-byte value in the file
// is big-endian; values are assembled and split with shifts, so the code is
// the same on little- and big-endian hosts.
#include "ncfile.hpp"

#include <fcntl.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cstring>
#include <limits>
#include <thread>

namespace gmc {
namespace nc {

namespace {

constexpr uint32_t kDimTag = 0x0A, kVarTag = 0x0B, kAttTag = 0x0C;
constexpr uint64_t kMaxVsize = 0xFFFFFFFCull;   // larger sizes are written as 2^32 - 1

uint64_t pad4(uint64_t n) { return (n + 3) & ~uint64_t(3); }

struct Out {
  std::vector<uint8_t> b;
  void u32(uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) b.push_back((uint8_t)(v >> s));
  }
  void u64(uint64_t v) {
    for (int s = 56; s >= 0; s -= 8) b.push_back((uint8_t)(v >> s));
  }
  void name(const std::string &s) {
    u32((uint32_t)s.size());
    b.insert(b.end(), s.begin(), s.end());
    b.resize(pad4(b.size()), 0);
  }
};

void put_be(uint8_t *p, uint64_t v, int n) {
  for (int i = 0; i < n; ++i) p[i] = (uint8_t)(v >> (8 * (n - 1 - i)));
}
uint64_t get_be(const uint8_t *p, int n) {
  uint64_t v = 0;
  for (int i = 0; i < n; ++i) v = (v << 8) | p[i];
  return v;
}

// One value of type t at p (big-endian) as a double, and the reverse.
double load_value(Type t, const uint8_t *p) {
  switch (t) {
    case DOUBLE: {
      const uint64_t u = get_be(p, 8);
      double d;
      std::memcpy(&d, &u, 8);
      return d;
    }
    case FLOAT: {
      const uint32_t u = (uint32_t)get_be(p, 4);
      float f;
      std::memcpy(&f, &u, 4);
      return f;
    }
    case INT: return (double)(int32_t)(uint32_t)get_be(p, 4);
    case SHORT: return (double)(int16_t)(uint16_t)get_be(p, 2);
    case BYTE: return (double)(int8_t)p[0];
    default: return (double)p[0];
  }
}
void store_value(Type t, double v, uint8_t *p) {
  switch (t) {
    case DOUBLE: {
      uint64_t u;
      std::memcpy(&u, &v, 8);
      put_be(p, u, 8);
      break;
    }
    case FLOAT: {
      const float f = (float)v;
      uint32_t u;
      std::memcpy(&u, &f, 4);
      put_be(p, u, 4);
      break;
    }
    case INT: put_be(p, (uint32_t)(int32_t)v, 4); break;
    case SHORT: put_be(p, (uint16_t)(int16_t)v, 2); break;
    default: p[0] = (uint8_t)(int8_t)v; break;
  }
}

void encode_atts(Out &o, const std::vector<Att> &atts) {
  if (atts.empty()) {
    o.u32(0);
    o.u32(0);
    return;
  }
  o.u32(kAttTag);
  o.u32((uint32_t)atts.size());
  for (const Att &a : atts) {
    o.name(a.name);
    o.u32((uint32_t)a.type);
    if (a.type == CHAR) {
      o.u32((uint32_t)a.text.size());
      o.b.insert(o.b.end(), a.text.begin(), a.text.end());
    } else {
      o.u32((uint32_t)a.num.size());
      const size_t at = o.b.size(), es = type_size(a.type);
      o.b.resize(at + a.num.size() * es);
      for (size_t n = 0; n < a.num.size(); ++n) store_value(a.type, a.num[n], &o.b[at + n * es]);
    }
    o.b.resize(pad4(o.b.size()), 0);
  }
}

// Bounded big-endian reader over a header buffer.
struct In {
  const uint8_t *p;
  size_t n, at = 0;
  bool short_ = false;
  size_t need = 0;
  bool take(size_t k) {
    if (at + k > n) {
      short_ = true;
      need = std::max(need, at + k - n);
      return false;
    }
    return true;
  }
  uint64_t u(int k) {
    if (!take((size_t)k)) return 0;
    const uint64_t v = get_be(p + at, k);
    at += (size_t)k;
    return v;
  }
  std::string name() {
    const uint64_t len = u(4);
    if (short_ || len > (1u << 20)) return std::string();
    const size_t padded = (size_t)pad4(len);
    if (!take(padded)) return std::string();
    std::string s(reinterpret_cast<const char *>(p + at), (size_t)len);
    at += padded;
    return s;
  }
};

std::string decode_atts(In &in, std::vector<Att> &atts) {
  const uint32_t tag = (uint32_t)in.u(4), cnt = (uint32_t)in.u(4);
  if (in.short_) return "";
  if (tag == 0 && cnt == 0) return "";
  if (tag != kAttTag) return "bad attribute list tag";
  if (cnt > (1u << 20)) return "implausible attribute count";
  for (uint32_t a = 0; a < cnt && !in.short_; ++a) {
    Att t;
    t.name = in.name();
    t.type = (Type)in.u(4);
    const uint64_t ne = in.u(4);
    if (in.short_) break;
    if (t.type < BYTE || t.type > DOUBLE) return "attribute '" + t.name + "' has an unknown type";
    const size_t es = type_size(t.type);
    if (ne > (uint64_t(1) << 28)) return "implausible attribute length";
    const size_t bytes = (size_t)pad4(ne * es);
    if (!in.take(bytes)) break;
    if (t.type == CHAR) {
      t.text.assign(reinterpret_cast<const char *>(in.p + in.at), (size_t)ne);
    } else {
      t.num.resize((size_t)ne);
      for (size_t k = 0; k < ne; ++k) t.num[k] = load_value(t.type, in.p + in.at + k * es);
    }
    in.at += bytes;
    atts.push_back(std::move(t));
  }
  return "";
}

}  // namespace

size_t type_size(Type t) {
  switch (t) {
    case DOUBLE: return 8;
    case FLOAT:
    case INT: return 4;
    case SHORT: return 2;
    default: return 1;
  }
}

int Header::dim(const std::string &name) const {
  for (size_t d = 0; d < dims.size(); ++d)
    if (dims[d].name == name) return (int)d;
  return -1;
}
int Header::var(const std::string &name) const {
  for (size_t v = 0; v < vars.size(); ++v)
    if (vars[v].name == name) return (int)v;
  return -1;
}
const Att *Header::att(int v, const std::string &name) const {
  const std::vector<Att> &l = v < 0 ? gatts : vars[(size_t)v].atts;
  for (const Att &a : l)
    if (a.name == name) return &a;
  return nullptr;
}

std::string Header::layout() {
  if (version != 1 && version != 2) return "netCDF classic version must be 1 or 2";
  int nrec_dims = 0;
  for (const Dim &d : dims) nrec_dims += d.len == 0;
  if (nrec_dims > 1) return "more than one unlimited dimension";
  for (Var &v : vars) {
    v.record = false;
    v.count = 1;
    for (size_t k = 0; k < v.dims.size(); ++k) {
      const int d = v.dims[k];
      if (d < 0 || d >= (int)dims.size()) return "variable '" + v.name + "' names an unknown dimension";
      if (dims[(size_t)d].len == 0) {
        if (k != 0) return "variable '" + v.name + "': the unlimited dimension must come first";
        v.record = true;
      } else {
        v.count *= dims[(size_t)d].len;
      }
    }
    v.vsize = pad4(v.count * type_size(v.type));
  }
  // header size with zero offsets (the offsets have a fixed width)
  for (Var &v : vars) v.begin = 0;
  uint64_t at = encode().size();
  const size_t nvars = vars.size();
  size_t last_fixed = nvars, last_rec = nvars, nrec = 0;
  for (size_t v = 0; v < nvars; ++v) {
    if (vars[v].record) { last_rec = v; ++nrec; }
    else last_fixed = v;
  }
  for (size_t v = 0; v < nvars; ++v) {
    if (vars[v].record) continue;
    if (vars[v].vsize > kMaxVsize && v != last_fixed) return "variable '" + vars[v].name + "' is too large for this format";
    vars[v].begin = at;
    at += vars[v].vsize;
  }
  recsize = 0;
  for (size_t v = 0; v < nvars; ++v) {
    if (!vars[v].record) continue;
    if (vars[v].vsize > kMaxVsize && v != last_rec) return "variable '" + vars[v].name + "' is too large for this format";
    vars[v].begin = at + recsize;
    recsize += vars[v].vsize;
  }
  if (nrec == 1) recsize = vars[last_rec].count * type_size(vars[last_rec].type);   // one record variable: no padding
  if (version == 1)
    for (const Var &v : vars)
      if (v.begin > 0x7FFFFFFFull) return "file too large for CDF-1 offsets";
  return "";
}

std::vector<uint8_t> Header::encode() const {
  Out o;
  o.b = {'C', 'D', 'F', (uint8_t)version};
  o.u32((uint32_t)numrecs);
  if (dims.empty()) {
    o.u32(0);
    o.u32(0);
  } else {
    o.u32(kDimTag);
    o.u32((uint32_t)dims.size());
    for (const Dim &d : dims) {
      o.name(d.name);
      o.u32((uint32_t)d.len);
    }
  }
  encode_atts(o, gatts);
  if (vars.empty()) {
    o.u32(0);
    o.u32(0);
  } else {
    o.u32(kVarTag);
    o.u32((uint32_t)vars.size());
    for (const Var &v : vars) {
      o.name(v.name);
      o.u32((uint32_t)v.dims.size());
      for (int d : v.dims) o.u32((uint32_t)d);
      encode_atts(o, v.atts);
      o.u32((uint32_t)v.type);
      o.u32(v.vsize > kMaxVsize ? 0xFFFFFFFFu : (uint32_t)v.vsize);
      if (version == 1) o.u32((uint32_t)v.begin);
      else o.u64(v.begin);
    }
  }
  return o.b;
}

std::string Header::decode(const uint8_t *p, size_t n, Header &h, size_t &need) {
  need = 0;
  h = Header();
  In in{p, n};
  if (!in.take(4)) { need = in.need; return "short header"; }
  if (p[0] != 'C' || p[1] != 'D' || p[2] != 'F') return "not a netCDF classic file";
  if (p[3] != 1 && p[3] != 2) return "unsupported netCDF format version " + std::to_string(p[3]);
  h.version = p[3];
  in.at = 4;
  h.numrecs = in.u(4);
  const uint32_t dtag = (uint32_t)in.u(4), nd = (uint32_t)in.u(4);
  if (!in.short_ && !(dtag == 0 && nd == 0)) {
    if (dtag != kDimTag) return "bad dimension list tag";
    if (nd > (1u << 16)) return "implausible dimension count";
    for (uint32_t d = 0; d < nd && !in.short_; ++d) {
      Dim dm;
      dm.name = in.name();
      dm.len = in.u(4);
      h.dims.push_back(dm);
    }
  }
  std::string e = decode_atts(in, h.gatts);
  if (!e.empty()) return e;
  const uint32_t vtag = (uint32_t)in.u(4), nv = (uint32_t)in.u(4);
  if (!in.short_ && !(vtag == 0 && nv == 0)) {
    if (vtag != kVarTag) return "bad variable list tag";
    if (nv > (1u << 20)) return "implausible variable count";
    for (uint32_t v = 0; v < nv && !in.short_; ++v) {
      Var vr;
      vr.name = in.name();
      const uint64_t ndim = in.u(4);
      if (ndim > 1024) return "implausible dimension count of a variable";
      for (uint64_t k = 0; k < ndim && !in.short_; ++k) vr.dims.push_back((int)in.u(4));
      e = decode_atts(in, vr.atts);
      if (!e.empty()) return e;
      vr.type = (Type)in.u(4);
      vr.vsize = in.u(4);
      vr.begin = in.u(h.version == 1 ? 4 : 8);
      h.vars.push_back(std::move(vr));
    }
  }
  if (in.short_) {
    need = in.need;
    return "short header";
  }
  // counts, record flags and the record size from the dimensions
  size_t nrec = 0, last_rec = 0;
  for (size_t v = 0; v < h.vars.size(); ++v) {
    Var &vr = h.vars[v];
    if (vr.type < BYTE || vr.type > DOUBLE) return "variable '" + vr.name + "' has an unknown type";
    vr.count = 1;
    for (size_t k = 0; k < vr.dims.size(); ++k) {
      const int d = vr.dims[k];
      if (d < 0 || d >= (int)h.dims.size()) return "variable '" + vr.name + "' names an unknown dimension";
      if (h.dims[(size_t)d].len == 0) {
        if (k != 0) return "variable '" + vr.name + "': the unlimited dimension is not first";
        vr.record = true;
      } else {
        vr.count *= h.dims[(size_t)d].len;
      }
    }
    const uint64_t real = pad4(vr.count * type_size(vr.type));
    if (vr.vsize == 0xFFFFFFFFull) vr.vsize = real;
    if (vr.record) { ++nrec; last_rec = v; h.recsize += vr.vsize; }
  }
  if (nrec == 1) h.recsize = h.vars[last_rec].count * type_size(h.vars[last_rec].type);
  return "";
}

File::~File() {
  if (fd_ >= 0) close();
}

namespace {

// Whole-buffer positioned write and read (retrying short transfers).
bool pwrite_all(int fd, const uint8_t *p, size_t n, uint64_t off) {
  while (n > 0) {
    const ssize_t w = ::pwrite(fd, p, n, (off_t)off);
    if (w < 0 && errno == EINTR) continue;
    if (w <= 0) return false;
    p += w;
    n -= (size_t)w;
    off += (uint64_t)w;
  }
  return true;
}
bool pread_all(int fd, uint8_t *p, size_t n, uint64_t off) {
  while (n > 0) {
    const ssize_t r = ::pread(fd, p, n, (off_t)off);
    if (r < 0 && errno == EINTR) continue;
    if (r <= 0) return false;
    p += r;
    n -= (size_t)r;
    off += (uint64_t)r;
  }
  return true;
}

// Runs body(a, b) over [0, n) split into contiguous parts, one per thread:
// host threads convert and move large variables in parallel.
template <class F>
bool par_ranges(uint64_t n, uint64_t bytes, F body) {
  unsigned nt = std::thread::hardware_concurrency();
  nt = std::max(1u, std::min(nt, 16u));
  if (bytes < (8u << 20)) nt = 1;
  if (nt == 1) return body(uint64_t(0), n);
  std::vector<std::thread> th;
  std::vector<char> ok(nt, 1);
  const uint64_t per = (n + nt - 1) / nt;
  for (unsigned t = 0; t < nt; ++t) {
    const uint64_t a = std::min(n, t * per), b = std::min(n, a + per);
    th.emplace_back([&, t, a, b]() { ok[t] = body(a, b) ? 1 : 0; });
  }
  for (std::thread &x : th) x.join();
  return std::all_of(ok.begin(), ok.end(), [](char c) { return c != 0; });
}

constexpr uint64_t kChunk = 1 << 17;   // values converted per transfer

}  // namespace

std::string File::create(const std::string &path, Header hdr) {
  if (fd_ >= 0) return "file already open";
  std::string e = hdr.layout();
  if (!e.empty()) return e;
  h = std::move(hdr);
  h.numrecs = 0;
  fd_ = ::open(path.c_str(), O_RDWR | O_CREAT | O_TRUNC, 0644);
  if (fd_ < 0) return "cannot create '" + path + "': " + std::strerror(errno);
  path_ = path;
  write_ = true;
  const std::vector<uint8_t> b = h.encode();
  if (!pwrite_all(fd_, b.data(), b.size(), 0)) return "cannot write the header of '" + path + "'";
  dirty_ = true;
  return "";
}

std::string File::open(const std::string &path, bool update) {
  if (fd_ >= 0) return "file already open";
  fd_ = ::open(path.c_str(), update ? O_RDWR : O_RDONLY);
  if (fd_ < 0) return "cannot open '" + path + "': " + std::strerror(errno);
  path_ = path;
  write_ = update;
  struct stat sb;
  if (fstat(fd_, &sb) != 0) return "cannot stat '" + path + "'";
  const uint64_t size = (uint64_t)sb.st_size;
  std::vector<uint8_t> buf((size_t)std::min<uint64_t>(size, 4096));
  for (;;) {
    if (!buf.empty() && !pread_all(fd_, buf.data(), buf.size(), 0)) {
      ::close(fd_);
      fd_ = -1;
      return "cannot read '" + path + "'";
    }
    size_t need = 0;
    std::string e = Header::decode(buf.data(), buf.size(), h, need);
    if (e.empty()) break;
    if (need == 0 || buf.size() >= size) {
      ::close(fd_);
      fd_ = -1;
      return "'" + path + "': " + e;
    }
    buf.resize((size_t)std::min<uint64_t>(size, std::max<uint64_t>(buf.size() * 2, buf.size() + need)));
  }
  if (h.numrecs == 0xFFFFFFFFull) {   // streaming: count the records present
    uint64_t first = size;
    for (const Var &v : h.vars)
      if (v.record) first = std::min(first, v.begin);
    h.numrecs = h.recsize && size > first ? (size - first) / h.recsize : 0;
  }
  return "";
}

std::string File::put(const std::string &name, uint64_t rec, const double *src) {
  if (fd_ < 0 || !write_) return "file not open for writing";
  const int vi = h.var(name);
  if (vi < 0) return "no variable '" + name + "' in '" + path_ + "'";
  const Var &v = h.vars[(size_t)vi];
  if (rec > 0xFFFFFFFEull) return "record index out of range";
  const uint64_t off = v.begin + (v.record ? rec * h.recsize : 0);
  const size_t es = type_size(v.type);
  const bool ok = par_ranges(v.count, v.count * es, [&](uint64_t a, uint64_t b) {
    std::vector<uint8_t> buf((size_t)std::min<uint64_t>(b - a, kChunk) * es);
    for (uint64_t at = a; at < b; at += kChunk) {
      const size_t n = (size_t)std::min<uint64_t>(kChunk, b - at);
      for (size_t k = 0; k < n; ++k) store_value(v.type, src[at + k], &buf[k * es]);
      if (!pwrite_all(fd_, buf.data(), n * es, off + at * es)) return false;
    }
    return true;
  });
  if (!ok) return "write failed in '" + path_ + "'";
  // zero padding to the next 4 bytes (none when a single record variable fills the record)
  const uint64_t pad = pad4(v.count * es) - v.count * es;
  if (pad && !(v.record && h.recsize == v.count * es)) {
    const uint8_t z[4] = {0, 0, 0, 0};
    if (!pwrite_all(fd_, z, (size_t)pad, off + v.count * es)) return "write failed in '" + path_ + "'";
  }
  if (v.record && rec + 1 > h.numrecs) {
    h.numrecs = rec + 1;
    dirty_ = true;
  }
  return "";
}

std::string File::get(const std::string &name, uint64_t rec, double *dst) {
  if (fd_ < 0) return "file not open";
  const int vi = h.var(name);
  if (vi < 0) return "no variable '" + name + "' in '" + path_ + "'";
  const Var &v = h.vars[(size_t)vi];
  if (v.record && rec >= h.numrecs) return "record " + std::to_string(rec) + " of '" + name + "' not in '" + path_ + "'";
  const uint64_t off = v.begin + (v.record ? rec * h.recsize : 0);
  const size_t es = type_size(v.type);
  const bool ok = par_ranges(v.count, v.count * es, [&](uint64_t a, uint64_t b) {
    std::vector<uint8_t> buf((size_t)std::min<uint64_t>(b - a, kChunk) * es);
    for (uint64_t at = a; at < b; at += kChunk) {
      const size_t n = (size_t)std::min<uint64_t>(kChunk, b - at);
      if (!pread_all(fd_, buf.data(), n * es, off + at * es)) return false;
      for (size_t k = 0; k < n; ++k) dst[at + k] = load_value(v.type, &buf[k * es]);
    }
    return true;
  });
  if (!ok) return "'" + path_ + "' ends inside variable '" + name + "'";
  return "";
}

std::string File::close() {
  if (fd_ < 0) return "";
  std::string e;
  if (write_ && dirty_) {
    uint8_t b[4];
    put_be(b, (uint32_t)h.numrecs, 4);
    if (!pwrite_all(fd_, b, 4, 4)) e = "cannot update the record count of '" + path_ + "'";
  }
  if (::close(fd_) != 0 && e.empty()) e = "closing '" + path_ + "' failed";
  fd_ = -1;
  dirty_ = false;
  return e;
}

}  // namespace nc
}  // namespace gmc
