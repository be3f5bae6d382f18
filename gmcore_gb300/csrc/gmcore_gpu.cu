// C ABI of the GB300 GMCORE dynamics step: context set-up, state transfer,
// the time loop (time_integrate, gmcore_mod.F90:577-591) and diagnostics.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <condition_variable>
#include <memory>
#include <tuple>
#include <map>
#include <set>
#include <mutex>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "gmcore_gpu.h"
#include "grid.hpp"
#include "kernels.hpp"
#include "output.hpp"

using namespace gmc;

namespace {

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct CudaError {
  std::string msg;
  explicit CudaError(std::string m) : msg(std::move(m)) {}
};
struct ApiError {
  int code;
  std::string msg;
};

// Bump allocator over one device allocation.
struct Arena {
  char *base = nullptr;
  size_t size = 0, used = 0;
  void reserve(size_t bytes) {
    size = bytes;
    cudaError_t e = cudaMalloc(&base, bytes);
    if (e != cudaSuccess) {
      base = nullptr;
      cudaGetLastError();   // a failed allocation must not surface as a later call's error
      throw ApiError{GMC_ENOMEM, std::string("device allocation of ") + std::to_string(bytes) + " bytes failed: " +
                                     cudaGetErrorString(e)};
    }
    CK(cudaMemset(base, 0, bytes));
  }
  template <class T>
  T *take(size_t n) {
    size_t off = (used + 255) & ~(size_t)255;
    size_t bytes = n * sizeof(T);
    if (off + bytes > size) throw ApiError{GMC_ENOMEM, "arena overflow"};
    used = off + bytes;
    return reinterpret_cast<T *>(base + off);
  }
  void release() {
    if (base) cudaFree(base);
    base = nullptr;
  }
};

// Size of a request: run the same sequence of takes on a counting arena.
struct Counter {
  size_t used = 0;
  template <class T>
  T *take(size_t n) {
    used = ((used + 255) & ~(size_t)255) + n * sizeof(T);
    return nullptr;
  }
};

enum FieldKind { FULL3, HALF3, LEV3, TWO_D };

struct FieldInfo {
  FieldKind kind;
  int nrow, nk;
};

}  // namespace

// ---------------------------------------------------------------------------
// Engine: one precision instantiation of the step.
// ---------------------------------------------------------------------------
// Host-side parallel loop over [0, n) in contiguous chunks (the row gathers,
// scatters and FP64<->FP32 conversions of field transfers), on a persistent
// pool of worker threads shared by all contexts; the calling thread works too.
class HostPool {
 public:
  static HostPool &get() {
    static HostPool pool;
    return pool;
  }
  template <class F>
  void run(size_t n, F &&f) {
    const unsigned nt = (unsigned)std::min<size_t>(workers_.size() + 1, std::max<size_t>(1, n / 16));
    if (nt <= 1) {
      f((size_t)0, n);
      return;
    }
    std::unique_lock<std::mutex> call(call_mu_);   // one parallel loop at a time
    const size_t chunk = (n + nt - 1) / nt;
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = [&f, n, chunk](unsigned t) {
        const size_t a = t * chunk, b = std::min(n, a + chunk);
        if (a < b) f(a, b);
      };
      ntasks_ = nt;
      next_ = 0;
      remaining_ = nt;
      ++gen_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return remaining_ == 0; });
    job_ = nullptr;
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto &w : workers_) w.join();
  }

 private:
  HostPool() {
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    for (unsigned t = 1; t < hw; ++t)
      workers_.emplace_back([this] {
        uint64_t seen = 0;
        for (;;) {
          {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
            if (stop_) return;
            seen = gen_;
          }
          work();
        }
      });
  }
  void work() {
    for (;;) {
      unsigned t;
      std::function<void(unsigned)> job;
      {
        std::lock_guard<std::mutex> lk(mu_);
        if (next_ >= ntasks_ || !job_) return;
        t = next_++;
        job = job_;
      }
      job(t);
      std::lock_guard<std::mutex> lk(mu_);
      if (--remaining_ == 0) done_cv_.notify_all();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex mu_, call_mu_;
  std::condition_variable cv_, done_cv_;
  std::function<void(unsigned)> job_;
  unsigned ntasks_ = 0, next_ = 0, remaining_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

template <class F>
void host_par_for(size_t n, F &&f) {
  HostPool::get().run(n, f);
}

// Row r (k-major over nk levels of nrow rows) of the interior of a view.
// Host ranges the caller registered with gmc_host_register (page-locked and
// mapped): transfers of views inside one of them run as device kernels that
// read or write the rows over the host link and convert on the GPU.
struct HostRange {
  uintptr_t base;
  size_t bytes;
  char *dev;   // device address of base
};
std::mutex g_host_mu;
std::vector<HostRange> g_host_ranges;

// Device address of [p, p + bytes) when one registered range holds all of it.
char *mapped_range(const void *p, size_t bytes) {
  std::lock_guard<std::mutex> lk(g_host_mu);
  const uintptr_t a = (uintptr_t)p;
  for (const HostRange &r : g_host_ranges)
    if (a >= r.base && bytes <= r.bytes && a - r.base <= r.bytes - bytes) return r.dev + (a - r.base);
  return nullptr;
}

// Interior row r (0-based, level-major) of a view relative to its row 0,
// in elements (view_row's arithmetic on the device).
struct ViewDims {
  long n0, n1;   // allocated extents of the view's first two dimensions
  int nrow, nlon;
};
__device__ __forceinline__ long view_rel(const ViewDims &d, size_t r) {
  const long j = (long)(r % d.nrow) + 1, k = (long)(r / d.nrow) + 1;
  return d.n0 * ((j - 1) + d.n1 * (k - 1));
}
template <class T>
__global__ void k_view_gather(const double *__restrict__ row0, ViewDims d, size_t rows, T *__restrict__ dst) {
  for (size_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const double *src = row0 + view_rel(d, r);
    T *o = dst + r * d.nlon;
    for (int i = threadIdx.x; i < d.nlon; i += blockDim.x) o[i] = (T)src[i];
  }
}
template <class T>
__global__ void k_view_scatter(const T *__restrict__ src, ViewDims d, size_t rows, double *__restrict__ row0) {
  for (size_t r = blockIdx.x; r < rows; r += gridDim.x) {
    double *o = row0 + view_rel(d, r);
    const T *s = src + r * d.nlon;
    for (int i = threadIdx.x; i < d.nlon; i += blockDim.x) o[i] = (double)s[i];
  }
}

// FP64 staging <-> a field in the form's type (the overlapped transfers of
// gmc_step_io: the DMA moves FP64 rows, the conversion runs on the device).
template <class T>
__global__ void k_from_f64(const double *__restrict__ src, size_t n, T *__restrict__ dst, T *__restrict__ dst2) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const T v = (T)src[t];
    dst[t] = v;
    if (dst2) dst2[t] = v;
  }
}
template <class T>
__global__ void k_to_f64(const T *__restrict__ src, size_t n, double *__restrict__ dst) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    dst[t] = (double)src[t];
}

inline double *view_row(const gmc_view &v, int nrow, size_t r) {
  const long n0 = v.ub[0] - v.lb[0] + 1, n1 = v.ub[1] - v.lb[1] + 1;
  const int k = (int)(r / nrow) + 1, j = (int)(r % nrow) + 1;
  return v.data + (size_t)(1 - v.lb[0]) + (size_t)n0 * ((size_t)(j - v.lb[1]) + (size_t)n1 * (size_t)(k - v.lb[2]));
}

struct EngineBase {
  virtual ~EngineBase() {}
  // host fields cross as gmc_view (interior rows gathered/scattered in place)
  virtual void set_field(int member, const std::string &name, const gmc_view &src) = 0;
  virtual void get_field(int member, const std::string &name, const gmc_view &dst) = 0;
  virtual void prepare() = 0;
  virtual void step(int nsteps) = 0;
  virtual void diagnose(int member, gmc_diag *out) = 0;
  virtual unsigned read_error() = 0;
  virtual void set_tracer(int member, int l, const gmc_view &src) = 0;
  virtual void get_tracer(int member, int l, const gmc_view &dst) = 0;
  virtual void ffsl_hflx(const gmc_ffsl_fields &f, double dt) = 0;
  virtual size_t ffsl_scratch_bytes() const = 0;
  virtual void ffsl_hflx_in(const gmc_ffsl_fields &f, double dt, void *scratch) = 0;
  // tangent-linear and adjoint of nsteps steps from the prepared state; the
  // three fields are u_lon, v_lat, gz (host, dense interior arrays)
  virtual void tlm(int nsteps, const double *const dx0[3], double *const dxn[3]) = 0;
  virtual void adjoint(int nsteps, int ckpt, const double *const lam_n[3], double *const lam_0[3]) = 0;
  // gmc_step_io: inputs set, nsteps steps, outputs read back, with the
  // transfers overlapped with the step where the dependencies allow; an item
  // with tracer >= 0 is that tracer, otherwise the named field
  struct IoItem {
    std::string name;
    int tracer;
    gmc_view view;
  };
  virtual void step_io(int member, const std::vector<IoItem> &in, int nsteps, const std::vector<IoItem> &out) = 0;
  // FP64 history diagnostics of a member's state into dense host arrays:
  // ph, t, z, div [nlev][nlat][nlon] and vor [nlev][nlat-1][nlon] (shallow
  // water: z and div [nlat][nlon], ph, t and vor unused and may be null)
  virtual void output_diag(int member, double *ph, double *t, double *z, double *div, double *vor) = 0;
  virtual const Grid &host_grid() const = 0;
  // Device copies of a member's output fields, for a file written in the
  // background while the steps go on: the state and tracers (and, for a
  // history record, the FP64 diagnostics and the integrals), taken in stream
  // order after the steps issued so far, in one stream-ordered allocation
  // that the writer frees.  Field pointers are in the form's storage type
  // (float when fp32), phs, gzs and the diagnostics in double.
  struct OutSnap {
    bool fp32 = false;
    char *block = nullptr;
    const void *u = nullptr, *v = nullptr, *pt = nullptr, *gz = nullptr, *pv = nullptr;
    const double *phs = nullptr, *gzs = nullptr;
    std::vector<const void *> q;
    const double *ph = nullptr, *t = nullptr, *z = nullptr, *div = nullptr, *vor = nullptr;
    gmc_diag diag{};
    cudaEvent_t ready = nullptr;   // recorded after the copies
  };
  virtual OutSnap snapshot(int member, bool history) = 0;
  virtual void set_graphs(bool on) = 0;
  virtual int layout_in_use() const = 0;
  virtual bool set_layout(int lay) = 0;
  virtual bool layout_is_tuned() const = 0;
  long time_step = 0;
  int device = 0;   // device current when the context was created
  // timing and profiling
  double last_step_ms = 0;
  long last_steps = 0, last_launches = 0, launches = 0;
  bool prof = false;
  struct Prof { std::string name; double ms = 0; long count = 0; };
  std::vector<Prof> prof_table;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_pending;
  std::vector<cudaEvent_t> event_pool;
};

template <class R>
struct Engine : EngineBase {
  Grid grid;
  DGrid dg{};
  Arena tables, arena;
  cudaStream_t stream = nullptr;
  Launch L{};
  int nm = 1;
  std::vector<Slot<R>> slots;   // [member * 3 + s]
  std::vector<Work<R>> work;    // [member]
  std::vector<double *> gzs;    // [member]
  unsigned *err = nullptr;
  double *diag_partial = nullptr, *diag_out = nullptr;
  int old_i = 0, new_i = 1;
  bool prepared = false;
  double *pinned = nullptr;
  size_t pinned_n = 0;
  R *staging = nullptr;
  // tracer batch (one per member) and its host-side cadence state
  int ntr = 0;
  std::vector<TracerBatch<R>> tb;     // [member]
  // one member with several tracers: each tracer's advection runs on its own
  // stream (forked from and joined to the context stream) with its own FFSL
  // scratch, so that the tracers' kernels overlap
  struct TracerScratch {
    R *qx, *qy, *fx, *fy;
  };
  std::vector<TracerScratch> tsc;     // [tracer]
  std::vector<cudaStream_t> tstreams;
  std::vector<cudaEvent_t> tevents;
  cudaEvent_t tfork_ev = nullptr;
  bool tracer_streams() const { return nm == 1 && ntr > 1; }
  // one baroclinic member: the forward pass runs its batch-CFL / column-mass /
  // potential-temperature FFSL chain on a side stream, overlapping the
  // tangent-wind / KE / PV / momentum chain of the context stream
  cudaStream_t dside = nullptr;
  cudaEvent_t dfork_ev = nullptr, dmf_ev = nullptr, dcm_ev = nullptr, dpt_ev = nullptr;
  bool dyn_split() const { return nm == 1 && grid.cfg.baroclinic && !prof; }
  std::vector<R *> q;                 // [(member * 2 + slot) * ntr + l]
  int q_old = 0;
  int nstep_adv = 1, uv_step = 0, mf_step = 0, we_step = 0;
  double alert_last = 0, curr_time = 0;
  bool alert_ring = false;

  static constexpr bool kFP32 = std::is_same<R, float>::value;

  size_t full3() const { return (size_t)grid.nlev * grid.nlat * grid.nlon; }
  size_t half3() const { return (size_t)grid.nlev * grid.nhalf * grid.nlon; }
  size_t lev3() const { return (size_t)(grid.nlev + 1) * grid.nlat * grid.nlon; }
  size_t two_d() const { return (size_t)grid.nlat * grid.nlon; }

  template <class A>
  void carve(A &a, Slot<R> &s, bool baroclinic) {
    s.u_lon = a.template take<R>(full3());
    s.v_lat = a.template take<R>(half3());
    s.u_f = a.template take<R>(full3());
    s.v_f = a.template take<R>(half3());
    s.mfx_lon = a.template take<R>(full3());
    s.mfy_lat = a.template take<R>(half3());
    s.pv = a.template take<R>(half3());
    s.pv_lon = a.template take<R>(full3());
    s.pv_lat = a.template take<R>(half3());
    if (baroclinic) {
      s.pt = a.template take<R>(full3());
      s.phs = a.template take<double>(two_d());
      s.phs_f = a.template take<double>(two_d());
      s.psr = kFP32 ? a.template take<float>(two_d()) : nullptr;
      s.we_lev = a.template take<R>(lev3());
      s.gz = s.gz_f = nullptr;
    } else {
      s.gz = a.template take<R>(two_d());
      s.gz_f = a.template take<R>(two_d());
      s.pt = nullptr;
      s.phs = s.phs_f = nullptr;
      s.psr = nullptr;
      s.we_lev = nullptr;
    }
  }
  template <class A>
  void carve(A &a, Work<R> &w, bool baroclinic) {
    w.u_lat = a.template take<R>(half3());
    w.v_lon = a.template take<R>(full3());
    w.ke = a.template take<R>(full3());
    w.du = a.template take<R>(full3());
    w.dv = a.template take<R>(half3());
    if (baroclinic) {
      w.cflx = a.template take<R>(full3());
      w.cfly = a.template take<R>(half3());
      w.cflz = a.template take<R>(lev3());
      w.divx = a.template take<R>(full3());
      w.divy = a.template take<R>(full3());
      w.qmfx = a.template take<R>(full3());
      w.qmfy = a.template take<R>(half3());
      w.qx = a.template take<R>(full3());
      w.qy = a.template take<R>(full3());
      w.ptf_lon = a.template take<R>(full3());
      w.ptf_lat = a.template take<R>(half3());
      w.dpt = a.template take<R>(full3());
      w.dphs = a.template take<double>(two_d());
      w.ph_exn_lev = a.template take<double>(lev3());
      w.gz_lev = a.template take<double>(lev3());
      w.pea = kFP32 ? reinterpret_cast<float *>(w.ph_exn_lev) : nullptr;
      w.gzhl = kFP32 ? reinterpret_cast<float2 *>(w.gz_lev) : nullptr;
      w.dgz = nullptr;
    } else {
      w.dgz = a.template take<R>(two_d());
      w.cflx = w.cfly = w.cflz = w.divx = w.divy = nullptr;
      w.qmfx = w.qmfy = w.qx = w.qy = w.ptf_lon = w.ptf_lat = w.dpt = nullptr;
      w.dphs = w.ph_exn_lev = w.gz_lev = nullptr;
      w.pea = nullptr;
      w.gzhl = nullptr;
    }
  }

  template <class A>
  void carve_member(A &a, int m, bool baroclinic) {
    double *z = a.template take<double>(two_d());
    for (int s = 0; s < 3; ++s) {
      Slot<R> &sl = slots[m * 3 + s];
      carve(a, sl, baroclinic);
      sl.gzs = z;
    }
    carve(a, work[m], baroclinic);
    work[m].gzs = z;
    gzs[m] = z;
    if (ntr > 0) {
      TracerBatch<R> &b = tb[m];
      b.u = a.template take<R>(full3());
      b.v = a.template take<R>(half3());
      b.mfx = a.template take<R>(full3());
      b.mfy = a.template take<R>(half3());
      b.we = a.template take<R>(lev3());
      b.m_lev = a.template take<R>(lev3());
      b.cflx = a.template take<R>(full3());
      b.cfly = a.template take<R>(half3());
      b.divx = a.template take<R>(full3());
      b.divy = a.template take<R>(full3());
      b.cflz = a.template take<R>(lev3());
      b.old_phs_f = a.template take<double>(two_d());
      b.old_psr = kFP32 ? a.template take<float>(two_d()) : nullptr;
      for (int t = 0; t < 2 * ntr; ++t) q[(size_t)m * 2 * ntr + t] = a.template take<R>(full3());
      if (tracer_streams()) {
        tsc.resize(ntr);
        for (TracerScratch &t : tsc) {
          t.qx = a.template take<R>(full3());
          t.qy = a.template take<R>(full3());
          t.fx = a.template take<R>(full3());
          t.fy = a.template take<R>(half3());
        }
      }
    }
  }

  // Members sharing this grid step in member-batched launches (grid z =
  // member) when every member-owned pointer of member m is member 0's plus m
  // times one stride; the arena carves the members identically, and the
  // check below confirms it pointer by pointer.
  bool batched_members = false;
  void member_batching_setup() {
    dg.mstride = 0;
    if (nm <= 1) return;
    const uintptr_t stride = (uintptr_t)gzs[1] - (uintptr_t)gzs[0];
    bool ok = stride > 0;
    auto same = [&](const void *p0, const void *pm, int m) {
      if (!p0 && !pm) return;
      ok = ok && p0 && pm && (uintptr_t)pm - (uintptr_t)p0 == stride * (uintptr_t)m;
    };
    for (int m = 1; m < nm && ok; ++m) {
      for (int t = 0; t < 3; ++t) {
        const Slot<R> &a = slots[t], &b = slots[m * 3 + t];
        for (auto pp : {std::make_pair((const void *)a.u_lon, (const void *)b.u_lon), {a.v_lat, b.v_lat}, {a.u_f, b.u_f},
                        {a.v_f, b.v_f}, {a.pt, b.pt}, {a.gz, b.gz}, {a.gz_f, b.gz_f}, {a.phs, b.phs}, {a.phs_f, b.phs_f},
                        {a.psr, b.psr}, {a.mfx_lon, b.mfx_lon}, {a.mfy_lat, b.mfy_lat}, {a.pv, b.pv},
                        {a.pv_lon, b.pv_lon}, {a.pv_lat, b.pv_lat}, {a.we_lev, b.we_lev}, {a.gzs, b.gzs}})
          same(pp.first, pp.second, m);
      }
      const Work<R> &a = work[0], &b = work[m];
      for (auto pp : {std::make_pair((const void *)a.u_lat, (const void *)b.u_lat), {a.v_lon, b.v_lon}, {a.ke, b.ke},
                      {a.cflx, b.cflx}, {a.cfly, b.cfly}, {a.cflz, b.cflz}, {a.divx, b.divx}, {a.divy, b.divy},
                      {a.qmfx, b.qmfx}, {a.qmfy, b.qmfy}, {a.qx, b.qx}, {a.qy, b.qy}, {a.ptf_lon, b.ptf_lon},
                      {a.ptf_lat, b.ptf_lat}, {a.du, b.du}, {a.dv, b.dv}, {a.dpt, b.dpt}, {a.dgz, b.dgz},
                      {a.dphs, b.dphs}, {a.ph_exn_lev, b.ph_exn_lev}, {a.gz_lev, b.gz_lev}, {a.pea, b.pea},
                      {a.gzhl, b.gzhl}, {a.gzs, b.gzs}})
        same(pp.first, pp.second, m);
    }
    if (ok) {
      dg.mstride = stride;
      batched_members = true;
    }
  }

  explicit Engine(const gmc_config &cfg) {
    try {
      construct(cfg);
    } catch (...) {
      release_all();   // a constructor that throws runs no destructor
      throw;
    }
  }
  void construct(const gmc_config &cfg) {
    std::string e = grid.build(cfg);
    if (!e.empty()) throw ApiError{GMC_EINVAL, e};
    nm = cfg.n_members;
    const bool bc = cfg.baroclinic != 0;
    ntr = bc ? cfg.ntracer : 0;
    tb.resize(nm);
    q.assign((size_t)nm * 2 * std::max(ntr, 1), nullptr);
    nstep_adv = std::max(1, (int)(cfg.dt_adv / cfg.dt_dyn));
    CK(cudaGetDevice(&device));
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    L.stream = stream;
    L.threads = grid.nlon >= 512 ? 256 : 128;
    upload_tables();
    slots.resize(3 * nm);
    work.resize(nm);
    gzs.resize(nm);
    Counter cnt;
    {
      std::vector<Slot<R>> s2(3 * nm);
      std::swap(s2, slots);
      for (int m = 0; m < nm; ++m) carve_member(cnt, m, bc);
      std::swap(s2, slots);
    }
    size_t nblk = (size_t)grid.nlat * grid.nlev;
    cnt.take<double>(8 * nblk + 64);
    cnt.take<unsigned>(64);
    cnt.take<R>(std::max(lev3(), full3()));
    arena.reserve(cnt.used + 4096);
    for (int m = 0; m < nm; ++m) carve_member(arena, m, bc);
    member_batching_setup();
    diag_partial = arena.take<double>(8 * nblk);
    member_streams();
    setup_layouts();
    if (nm == 1 && bc) {
      CK(cudaStreamCreateWithFlags(&dside, cudaStreamNonBlocking));
      for (cudaEvent_t *e : {&dfork_ev, &dmf_ev, &dcm_ev, &dpt_ev}) CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    if (tracer_streams()) {
      tstreams.resize(ntr);
      tevents.resize(ntr);
      for (int t = 0; t < ntr; ++t) {
        CK(cudaStreamCreateWithFlags(&tstreams[t], cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&tevents[t], cudaEventDisableTiming));
      }
      CK(cudaEventCreateWithFlags(&tfork_ev, cudaEventDisableTiming));
    }
    diag_out = arena.take<double>(64);
    err = arena.take<unsigned>(64);
    staging = arena.take<R>(std::max(lev3(), full3()));
    dg.err = err;
    pinned_n = std::max(lev3(), full3());
    CK(cudaMallocHost(&pinned, pinned_n * sizeof(double)));
  }

  ~Engine() override { release_all(); }
  void release_all() {
    if (stream) cudaStreamSynchronize(stream);
    for (cudaEvent_t e : event_pool) cudaEventDestroy(e);
    for (auto &p : prof_pending) { cudaEventDestroy(p.second.first); cudaEventDestroy(p.second.second); }
    if (ev_a) cudaEventDestroy(ev_a);
    if (ev_b) cudaEventDestroy(ev_b);
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    for (cudaStream_t st : mstreams) cudaStreamDestroy(st);
    for (cudaEvent_t e : mevents) cudaEventDestroy(e);
    for (cudaEvent_t e : xfer_ev) cudaEventDestroy(e);
    if (fork_ev) cudaEventDestroy(fork_ev);
    for (cudaStream_t st : tstreams) cudaStreamDestroy(st);
    for (cudaEvent_t e : tevents) cudaEventDestroy(e);
    if (tfork_ev) cudaEventDestroy(tfork_ev);
    if (dside) cudaStreamDestroy(dside);
    for (cudaEvent_t e : {dfork_ev, dmf_ev, dcm_ev, dpt_ev})
      if (e) cudaEventDestroy(e);
    arena.release();
    tables.release();
    if (tl) {
      tl->drop_graphs();
      tl->release_streams();
      tl->arena.release();
      tl->zarena.release();
      tl->store.release();
    }
    if (pinned) cudaFreeHost(pinned);
    pinned = nullptr;
    if (xstream) cudaStreamDestroy(xstream);
    if (qstream) cudaStreamDestroy(qstream);
    for (cudaEvent_t e : qev) cudaEventDestroy(e);
    if (xin_ev) cudaEventDestroy(xin_ev);
    if (xdyn_ev) cudaEventDestroy(xdyn_ev);
    if (xpt_ev) cudaEventDestroy(xpt_ev);
    if (xlate_ev) cudaEventDestroy(xlate_ev);
    if (xptf_ev) cudaEventDestroy(xptf_ev);
    if (xphs_ev) cudaEventDestroy(xphs_ev);
    if (xstage) cudaFree(xstage);
    xstream = nullptr;
    xstage = nullptr;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }

  void upload_tables() {
    const Grid &g = grid;
    std::vector<char> host;
    auto push = [&](const void *p, size_t bytes) {
      size_t off = (host.size() + 255) & ~(size_t)255;
      host.resize(off + bytes);
      std::memcpy(host.data() + off, p, bytes);
      return off;
    };
    struct Fix { size_t off; const void **dst; };
    std::vector<Fix> fixes;
    auto row = [&](const RowTable &t, const double **dst, const float **dst_f) {
      fixes.push_back({push(t.v.data(), t.v.size() * 8), (const void **)dst});
      std::vector<float> tf(t.v.begin(), t.v.end());
      fixes.push_back({push(tf.data(), tf.size() * 4), (const void **)dst_f});
    };
    auto vec = [&](const std::vector<double> &t, const double **dst) {
      fixes.push_back({push(t.data(), t.size() * 8), (const void **)dst});
    };
    row(g.area_cell, &dg.area_cell, &dg.f.area_cell); row(g.area_subcell1, &dg.area_subcell1, &dg.f.area_subcell1); row(g.area_subcell2, &dg.area_subcell2, &dg.f.area_subcell2);
    row(g.area_lon, &dg.area_lon, &dg.f.area_lon); row(g.area_lon_west, &dg.area_lon_west, &dg.f.area_lon_west); row(g.area_lon_east, &dg.area_lon_east, &dg.f.area_lon_east);
    row(g.area_lon_north, &dg.area_lon_north, &dg.f.area_lon_north); row(g.area_lon_south, &dg.area_lon_south, &dg.f.area_lon_south);
    row(g.area_lat, &dg.area_lat, &dg.f.area_lat); row(g.area_lat_west, &dg.area_lat_west, &dg.f.area_lat_west); row(g.area_lat_east, &dg.area_lat_east, &dg.f.area_lat_east);
    row(g.area_lat_north, &dg.area_lat_north, &dg.f.area_lat_north); row(g.area_lat_south, &dg.area_lat_south, &dg.f.area_lat_south);
    row(g.area_vtx, &dg.area_vtx, &dg.f.area_vtx); row(g.de_lon, &dg.de_lon, &dg.f.de_lon); row(g.le_lon, &dg.le_lon, &dg.f.le_lon); row(g.de_lat, &dg.de_lat, &dg.f.de_lat);
    row(g.le_lat, &dg.le_lat, &dg.f.le_lat); row(g.full_f, &dg.full_f, &dg.f.full_f); row(g.half_f, &dg.half_f, &dg.f.half_f);
    row(g.full_tangent_wgt1, &dg.ftw1, &dg.f.ftw1); row(g.full_tangent_wgt2, &dg.ftw2, &dg.f.ftw2);
    row(g.half_tangent_wgt1, &dg.htw1, &dg.f.htw1); row(g.half_tangent_wgt2, &dg.htw2, &dg.f.htw2);
    row(g.full_cos_lat, &dg.full_cos_lat, &dg.f.full_cos_lat); row(g.half_cos_lat, &dg.half_cos_lat, &dg.f.half_cos_lat); row(g.half_lat, &dg.half_lat, &dg.f.half_lat);
    row(g.full_sin_lat, &dg.full_sin_lat, &dg.f.full_sin_lat);
    vec(g.hyai, &dg.hyai); vec(g.hybi, &dg.hybi); vec(g.half_lev, &dg.half_lev); vec(g.half_dlev, &dg.half_dlev);
    vec(g.full_dlev, &dg.full_dlev); vec(g.lon_damp_wgt_full, &dg.lon_damp_full);
    vec(g.full_lev, &dg.full_lev);
    {   // FP32 hybrid pressure coefficients of the half levels (Held-Suarez forcing)
      std::vector<float> pa(g.nlev + 2, 0.f);
      for (int k = 0; k <= g.nlev && g.cfg.baroclinic; ++k)
        pa[k] = (float)(g.hyai[k] * (g.cfg.hybrid_coord_p0 - g.local_ptop) + g.local_ptop);
      fixes.push_back({push(pa.data(), pa.size() * 4), (const void **)&dg.ph_lev_a});
    }
    vec(g.div_c_lon, &dg.div_c_lon); vec(g.div_c_lat, &dg.div_c_lat);
    {
      std::vector<float> yo((size_t)g.nhalf * 4, 0.f);
      for (int j = 1; j <= g.nhalf; ++j)
        for (int t = 0; t < 4; ++t) {
          int l = j - 1 + t;
          if (l >= 1 && l <= g.nhalf)
            yo[(size_t)(j - 1) * 4 + t] =
                (float)(g.cfg.radius * (g.half_lat.v[l + 1] - g.half_lat.v[j + 1]) / g.de_lat.v[j + 1]);
        }
      yo.push_back(0.f);
      fixes.push_back({push(yo.data(), yo.size() * 4), (const void **)&dg.cfl_yoff});
    }
    // FP32 layer-mass coefficients
    std::vector<float> dA(g.nlev + 1, 0.f), dB(g.nlev + 1, 0.f);
    for (int k = 0; k < g.nlev && g.cfg.baroclinic; ++k) {
      dA[k] = (float)((g.hyai[k + 1] - g.hyai[k]) * (g.cfg.hybrid_coord_p0 - g.local_ptop));
      dB[k] = (float)(g.hybi[k + 1] - g.hybi[k]);
    }
    size_t offA = push(dA.data(), dA.size() * 4), offB = push(dB.data(), dB.size() * 4);
    std::vector<float> hlf(g.half_lev.begin(), g.half_lev.end()), hdf(g.half_dlev.begin(), g.half_dlev.end()),
        fdf(g.full_dlev.begin(), g.full_dlev.end());
    hlf.push_back(0.f); hdf.push_back(0.f); fdf.push_back(0.f);
    size_t offHL = push(hlf.data(), hlf.size() * 4), offHD = push(hdf.data(), hdf.size() * 4),
           offFD = push(fdf.data(), fdf.size() * 4);
    std::vector<float> hbf(g.hybi.begin(), g.hybi.end());
    hbf.push_back(0.f);
    size_t offHB = push(hbf.data(), hbf.size() * 4);
    std::vector<float> rfd;
    for (double d : g.full_dlev) rfd.push_back(d != 0 ? (float)(1.0 / d) : 0.f);
    rfd.push_back(0.f);
    size_t offRFD = push(rfd.data(), rfd.size() * 4);
    // FP32 column sweep about a reference column at ps_ref = p0
    const int nl = g.nlev;
    const double ps_ref = g.cfg.p0, kap = g.cfg.Rd / g.cfg.cpd;
    std::vector<float> prc(nl + 2, 0.f), per(nl + 2, 0.f), dper(nl + 1, 0.f), cff(nl + 1, 0.f), tfr(nl + 1, 0.f),
        dlr(nl + 1, 0.f);
    if (g.cfg.baroclinic) {
      std::vector<double> pr(nl + 1), pe(nl + 1);
      for (int k = 0; k <= nl; ++k) {
        pr[k] = g.hyai[k] * (g.cfg.hybrid_coord_p0 - g.local_ptop) + g.hybi[k] * (ps_ref - g.local_ptop) + g.local_ptop;
        pe[k] = std::pow(pr[k], kap);
        prc[k] = (float)(g.hybi[k] / pr[k]);
        per[k] = (float)pe[k];
      }
      for (int k = 0; k < nl; ++k) {
        const double ph = 0.5 * (pr[k] + pr[k + 1]);
        dper[k] = (float)(pe[k + 1] - pe[k]);
        cff[k] = (float)(0.5 * (g.hybi[k] + g.hybi[k + 1]) / ph);
        tfr[k] = (float)std::pow(ph / g.cfg.p0, kap);
        dlr[k] = (float)std::log(pr[k + 1] / pr[k]);
      }
    }
    const size_t offPRC = push(prc.data(), prc.size() * 4), offPER = push(per.data(), per.size() * 4),
                 offDPER = push(dper.data(), dper.size() * 4), offCF = push(cff.data(), cff.size() * 4),
                 offTF = push(tfr.data(), tfr.size() * 4), offDL = push(dlr.data(), dlr.size() * 4);
    // filters
    struct FFix { size_t nf, nh, of, oh, w, wf; FilterDev *d; int maxt; };
    std::vector<FFix> ff;
    for (const Filter *f : {&g.big, &g.small1, &g.small2}) {
      std::vector<int> of(g.nlat), oh(g.nhalf);
      std::vector<double> w;
      for (int j = 0; j < g.nlat; ++j) { of[j] = (int)w.size(); w.insert(w.end(), f->wgt_full[j].begin(), f->wgt_full[j].end()); }
      for (int j = 0; j < g.nhalf; ++j) { oh[j] = (int)w.size(); w.insert(w.end(), f->wgt_half[j].begin(), f->wgt_half[j].end()); }
      w.push_back(0.0);
      FFix x;
      x.nf = push(f->ngrid_full.data(), f->ngrid_full.size() * 4);
      x.nh = push(f->ngrid_half.data(), f->ngrid_half.size() * 4);
      x.of = push(of.data(), of.size() * 4);
      x.oh = push(oh.data(), oh.size() * 4);
      x.w = push(w.data(), w.size() * 8);
      std::vector<float> wf(w.begin(), w.end());
      x.wf = push(wf.data(), wf.size() * 4);
      x.d = f == &g.big ? &dg.big : f == &g.small1 ? &dg.small1 : &dg.small2;
      x.maxt = f->max_taps();
      ff.push_back(x);
    }
    tables.reserve(host.size() + 256);
    CK(cudaMemcpy(tables.base, host.data(), host.size(), cudaMemcpyHostToDevice));
    for (const Fix &f : fixes) *f.dst = tables.base + f.off;
    dg.dmA = reinterpret_cast<const float *>(tables.base + offA);
    dg.dmB = reinterpret_cast<const float *>(tables.base + offB);
    dg.half_lev_f = reinterpret_cast<const float *>(tables.base + offHL);
    dg.half_dlev_f = reinterpret_cast<const float *>(tables.base + offHD);
    dg.full_dlev_f = reinterpret_cast<const float *>(tables.base + offFD);
    dg.hybi_f = reinterpret_cast<const float *>(tables.base + offHB);
    dg.full_dlev_rf = reinterpret_cast<const float *>(tables.base + offRFD);
    dg.pr_c = reinterpret_cast<const float *>(tables.base + offPRC);
    dg.pe_ref = reinterpret_cast<const float *>(tables.base + offPER);
    dg.dpe_ref = reinterpret_cast<const float *>(tables.base + offDPER);
    dg.cf = reinterpret_cast<const float *>(tables.base + offCF);
    dg.tf_ref = reinterpret_cast<const float *>(tables.base + offTF);
    dg.dlnp_ref = reinterpret_cast<const float *>(tables.base + offDL);
    dg.ps_ref = ps_ref;
    dg.f_layer_mass = kFP32 ? 1 : 0;
    dg.forcing = grid.cfg.forcing;
    dg.smag_coef = grid.cfg.smag_damp_coef;
    // the FP32 edge PV's default path (upwind order 3, pairs aligned beyond the
    // poles) forms the tangential winds itself: each has one reader there
    dg.tangent_inline = kFP32 && grid.cfg.baroclinic && grid.cfg.pv_scheme == GMC_PV_UPWIND &&
                        grid.cfg.upwind_order_pv == 3 && (grid.cfg.nlon / 2) % 2 == 0;
    for (const FFix &x : ff) {
      x.d->ntaps_full = reinterpret_cast<const int *>(tables.base + x.nf);
      x.d->ntaps_half = reinterpret_cast<const int *>(tables.base + x.nh);
      x.d->off_full = reinterpret_cast<const int *>(tables.base + x.of);
      x.d->off_half = reinterpret_cast<const int *>(tables.base + x.oh);
      x.d->wgt = reinterpret_cast<const double *>(tables.base + x.w);
      x.d->wgt_f = reinterpret_cast<const float *>(tables.base + x.wf);
      x.d->max_taps = x.maxt;
    }
    const gmc_config &c = g.cfg;
    dg.nlon = g.nlon; dg.nlat = g.nlat; dg.nhalf = g.nhalf; dg.nlev = g.nlev; dg.hx = g.lon_halo_width;
    dg.half = g.nlon / 2;
    dg.baroclinic = c.baroclinic;
    dg.radius = c.radius; dg.g = c.g; dg.Rd = c.Rd; dg.cpd = c.cpd; dg.p0 = c.p0; dg.kappa = c.Rd / c.cpd;
    dg.p0h = c.hybrid_coord_p0; dg.ptop = g.local_ptop; dg.dlon = g.dlon;
    dg.ke_scheme = c.ke_scheme; dg.ke_cell_wgt = c.ke_cell_wgt;
    dg.pv_scheme = c.pv_scheme; dg.upwind_order_pv = c.upwind_order_pv; dg.pv_pole_stokes = c.pv_pole_stokes;
    dg.coriolis_scheme = c.coriolis_scheme; dg.limiter = c.limiter_type; dg.upwind_wgt_pv = c.upwind_wgt_pv;
    dg.ke_cell_wgt_f = (float)c.ke_cell_wgt; dg.upwind_wgt_pv_f = (float)c.upwind_wgt_pv;
    dg.kappa_f = (float)(c.Rd / c.cpd); dg.Rd_f = (float)c.Rd; dg.g_f = (float)c.g;
    dg.flux_type = c.ffsl_flux_type; dg.tvd_limiter = c.tvd_limiter_type; dg.div_damp_order = c.div_damp_order;
  }

  FieldInfo info(const std::string &name) const {
    const int nlat = grid.nlat, nhalf = grid.nhalf, nlev = grid.nlev;
    if (name == "u_lon" || name == "u_f" || name == "pt" || name == "mfx_lon" || name == "pv_lon")
      return {FULL3, nlat, nlev};
    if (name == "v_lat" || name == "v_f" || name == "mfy_lat" || name == "pv" || name == "pv_lat")
      return {HALF3, nhalf, nlev};
    if (name == "we_lev") return {LEV3, nlat, nlev + 1};
    return {TWO_D, nlat, 1};
  }

  // Device pointer of a named field of a slot (R or double flavour).
  void locate(const Slot<R> &s, int m, const std::string &name, R **pr, double **pd) {
    *pr = nullptr;
    *pd = nullptr;
    const bool bc = grid.cfg.baroclinic != 0;
    if (name == "u_lon") *pr = s.u_lon;
    else if (name == "v_lat") *pr = s.v_lat;
    else if (name == "u_f") *pr = s.u_f;
    else if (name == "v_f") *pr = s.v_f;
    else if (name == "mfx_lon") *pr = s.mfx_lon;
    else if (name == "mfy_lat") *pr = s.mfy_lat;
    else if (name == "pv") *pr = s.pv;
    else if (name == "pv_lon") *pr = s.pv_lon;
    else if (name == "pv_lat") *pr = s.pv_lat;
    else if (name == "pt" && bc) *pr = s.pt;
    else if (name == "gz" && !bc) *pr = s.gz;
    else if (name == "gz_f" && !bc) *pr = s.gz_f;
    else if (name == "phs" && bc) *pd = s.phs;
    else if (name == "phs_f" && bc) *pd = s.phs_f;
    else if (name == "we_lev" && bc) *pr = s.we_lev;
    else if (name == "gzs") *pd = gzs[m];
    if (!*pr && !*pd) throw ApiError{GMC_EINVAL, "unknown field '" + name + "' for this model"};
  }

  size_t count(const FieldInfo &f) const { return (size_t)f.nk * f.nrow * grid.nlon; }

  // Host <-> device transfers of a field given as a view.  The rows are moved
  // in chunks: while one chunk's DMA runs the host pool converts the next
  // (gather and FP64 -> T on upload, T -> FP64 and scatter on download).
  static constexpr int kXferChunks = 8;
  std::vector<cudaEvent_t> xfer_ev;
  void xfer_events() {
    if (!xfer_ev.empty()) return;
    xfer_ev.resize(kXferChunks);
    for (auto &e : xfer_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  // Device address of the view's first interior row when the caller has
  // registered the whole span of its interior rows (nullptr otherwise).
  double *mapped_view(const gmc_view &v, int nrow, int nk, ViewDims &d) const {
    const size_t rows = (size_t)nrow * nk;
    const double *first = view_row(v, nrow, 0), *last = view_row(v, nrow, rows - 1) + grid.nlon;
    char *dev = mapped_range(first, (size_t)(last - first) * sizeof(double));
    d = {v.ub[0] - v.lb[0] + 1, v.ub[1] - v.lb[1] + 1, nrow, grid.nlon};
    return reinterpret_cast<double *>(dev);
  }
  static int xfer_blocks(size_t rows) { return (int)std::min<size_t>(rows, 152 * 8); }

  template <class T>
  void upload_view(const gmc_view &v, int nrow, int nk, T *dev, T *const *also = nullptr, int nalso = 0) {
    const int nlon = grid.nlon;
    const size_t rows = (size_t)nrow * nk, per = (rows + kXferChunks - 1) / kXferChunks;
    ViewDims vd;
    if (const double *row0 = mapped_view(v, nrow, nk, vd)) {   // registered: gather and convert on the GPU
      k_view_gather<T><<<xfer_blocks(rows), 256, 0, stream>>>(row0, vd, rows, dev);
      CK(cudaGetLastError());
      for (int t = 0; t < nalso; ++t)
        CK(cudaMemcpyAsync(also[t], dev, rows * nlon * sizeof(T), cudaMemcpyDeviceToDevice, stream));
      CK(cudaStreamSynchronize(stream));
      return;
    }
    T *host = reinterpret_cast<T *>(pinned);
    for (size_t a = 0; a < rows; a += per) {
      const size_t b = std::min(rows, a + per);
      host_par_for(b - a, [&](size_t x, size_t y) {
        for (size_t r = a + x; r < a + y; ++r) {
          const double *src = view_row(v, nrow, r);
          T *d = host + r * nlon;
          for (int i = 0; i < nlon; ++i) d[i] = (T)src[i];
        }
      });
      CK(cudaMemcpyAsync(dev + a * nlon, host + a * nlon, (b - a) * nlon * sizeof(T), cudaMemcpyHostToDevice, stream));
    }
    for (int t = 0; t < nalso; ++t)   // further device copies of the same field
      CK(cudaMemcpyAsync(also[t], dev, rows * nlon * sizeof(T), cudaMemcpyDeviceToDevice, stream));
    CK(cudaStreamSynchronize(stream));
  }
  template <class T>
  void download_view(const T *dev, int nrow, int nk, const gmc_view &v) {
    xfer_events();
    const int nlon = grid.nlon;
    const size_t rows = (size_t)nrow * nk, per = (rows + kXferChunks - 1) / kXferChunks;
    ViewDims vd;
    if (double *row0 = mapped_view(v, nrow, nk, vd)) {   // registered: convert and scatter on the GPU
      k_view_scatter<T><<<xfer_blocks(rows), 256, 0, stream>>>(dev, vd, rows, row0);
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(stream));
      return;
    }
    T *host = reinterpret_cast<T *>(pinned);
    int c = 0;
    for (size_t a = 0; a < rows; a += per, ++c) {
      const size_t b = std::min(rows, a + per);
      CK(cudaMemcpyAsync(host + a * nlon, dev + a * nlon, (b - a) * nlon * sizeof(T), cudaMemcpyDeviceToHost, stream));
      CK(cudaEventRecord(xfer_ev[c], stream));
    }
    c = 0;
    for (size_t a = 0; a < rows; a += per, ++c) {
      const size_t b = std::min(rows, a + per);
      CK(cudaEventSynchronize(xfer_ev[c]));
      host_par_for(b - a, [&](size_t x, size_t y) {
        for (size_t r = a + x; r < a + y; ++r) {
          double *dst = view_row(v, nrow, r);
          const T *src = host + r * nlon;
          for (int i = 0; i < nlon; ++i) dst[i] = (double)src[i];
        }
      });
    }
  }

  void set_field(int m, const std::string &name, const gmc_view &src) override {
    FieldInfo f = info(name);
    R *pr;
    double *pd;
    locate(slots[m * 3 + old_i], m, name, &pr, &pd);
    if (pd)
      upload_view<double>(src, f.nrow, f.nk, pd);
    else
      upload_view<R>(src, f.nrow, f.nk, pr);
  }

  void get_field(int m, const std::string &name, const gmc_view &dst) override {
    FieldInfo f = info(name);
    R *pr;
    double *pd;
    locate(slots[m * 3 + old_i], m, name, &pr, &pd);
    if (pd)
      download_view<double>(pd, f.nrow, f.nk, dst);
    else
      download_view<R>(pr, f.nrow, f.nk, dst);
  }

  void set_tracer(int m, int l, const gmc_view &src) override {
    if (l < 0 || l >= ntr) throw ApiError{GMC_EINVAL, "tracer index out of range"};
    // both time levels start from the initial mixing ratio
    R *second = q[((size_t)m * 2 + 1) * ntr + l];
    upload_view<R>(src, grid.nlat, grid.nlev, q[((size_t)m * 2 + 0) * ntr + l], &second, 1);
  }
  void get_tracer(int m, int l, const gmc_view &dst) override {
    if (l < 0 || l >= ntr) throw ApiError{GMC_EINVAL, "tracer index out of range"};
    download_view<R>(q[((size_t)m * 2 + q_old) * ntr + l], grid.nlat, grid.nlev, dst);
  }

  // ---- gmc_step_io: transfers overlapped with the step (one member) --------
  // The dynamics of the first step need only the prognostic fields, so tracer
  // inputs move over the host link while it runs, and its tracer step waits
  // for them (xin_ev); the last step's fields are final when its dynamics end
  // (xdyn_ev), so they move back while its tracer step runs.  The overlapped
  // transfers are copy-engine DMA of FP64 rows between registered host memory
  // and a device staging area, converted on the device; other items take the
  // gmc_set_* / gmc_get_* paths before and after the step.
  // Tracer outputs of registered arrays are pipelined with the last step's
  // tracer advection: the tracers then advect one after the other on the
  // context stream, each recording qev[l] when done, and tracer l moves back
  // on qstream while the next ones advect.
  // The first step's first stage reads pt from its potential-temperature
  // transport on, and u_lon, v_lat, phs only in its update kernels, so those
  // inputs cross the link on xstream while the stage's forward pass starts:
  // pt first (xpt_ev, waited before the first transport kernel), then the
  // others (xlate_ev, waited before the updates), then the tracers.
  cudaStream_t xstream = nullptr, qstream = nullptr;
  cudaEvent_t xin_ev = nullptr, xdyn_ev = nullptr, xpt_ev = nullptr, xlate_ev = nullptr, xphs_ev = nullptr;
  // Without test forcing (which changes pt after the integrator) the last
  // stage's update_pt leaves pt and phs final, so they move back from there
  // (xptf_ev) while the column sweep and the wind update still run.
  cudaEvent_t xptf_ev = nullptr;
  bool stage_last = false;   // the stage being issued is the step's last
  bool ptf_recorded = false;
  bool io_pt = false, io_late = false, cur_io_pt = false, cur_io_late = false, pt_waited = false,
       late_waited = false;
  bool io_phs = false, cur_io_phs = false, phs_waited = false;   // phs ahead of u_lon, v_lat (xphs_ev)
  std::vector<cudaEvent_t> qev;                  // [tracer]
  bool io_wait = false, io_rec = false;          // requested for this call's first / last step
  bool cur_io_wait = false, cur_io_rec = false;  // in effect for the step being issued
  bool io_qout = false, cur_io_qout = false;     // tracer outputs pipelined with the last step
  bool q_piped = false;                          // the last step advected its tracers pipelined
  bool io_waited = false;                        // the current step has issued its wait
  double *xstage = nullptr;
  size_t xstage_n = 0;
  std::function<void()> after_last;              // enqueued after the last step's launches
  void io_streams() {
    if (xstream) return;
    // the transfer streams' conversion kernels are small and gate the step's
    // readers (or the end of the call): they go ahead of the step's blocks
    int lo = 0, hi = 0;
    CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    CK(cudaStreamCreateWithPriority(&xstream, cudaStreamNonBlocking, hi));
    CK(cudaStreamCreateWithPriority(&qstream, cudaStreamNonBlocking, hi));
    CK(cudaEventCreateWithFlags(&xin_ev, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&xdyn_ev, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&xpt_ev, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&xlate_ev, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&xptf_ev, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&xphs_ev, cudaEventDisableTiming));
    qev.resize((size_t)ntr);
    for (cudaEvent_t &e : qev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  double *io_stage(size_t n) {
    if (n > xstage_n) {
      if (xstage) CK(cudaFree(xstage));
      xstage = nullptr;
      xstage_n = 0;
      if (cudaMalloc(&xstage, n * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        throw ApiError{GMC_ENOMEM, "device allocation failed (gmc_step_io staging)"};
      }
      xstage_n = n;
    }
    return xstage;
  }
  // registered host rows of a view (nullptr otherwise): the first interior
  // row, the row pitch and the level stride in bytes
  const double *io_rows(const gmc_view &v, int nrow, int nk, size_t &pitch, size_t &lstride) const {
    ViewDims vd;
    const double *row0 = mapped_view(v, nrow, nk, vd);
    if (!row0) return nullptr;
    pitch = (size_t)vd.n0 * sizeof(double);
    lstride = (size_t)vd.n0 * vd.n1 * sizeof(double);
    return view_row(v, nrow, 0);   // host address: the DMA reads the registered range
  }
  static bool capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cs));
    return cs == cudaStreamCaptureStatusActive;
  }
  void io_dyn_done(cudaStream_t st) {   // after the stages of a step
    if (!cur_io_rec || dry) return;
    CK(cudaEventRecordWithFlags(xdyn_ev, st, capturing(st) ? cudaEventRecordExternal : cudaEventRecordDefault));
  }
  void io_pt_ready(cudaStream_t st) {   // before the first stage reads pt
    if (!cur_io_pt || pt_waited) return;
    pt_waited = true;
    if (dry) return;
    CK(cudaStreamWaitEvent(st, xpt_ev, capturing(st) ? cudaEventWaitExternal : cudaEventWaitDefault));
  }
  void io_phs_ready(cudaStream_t st) {   // before the first stage's update_phs reads phs
    if (!cur_io_phs || phs_waited) return;
    phs_waited = true;
    if (dry) return;
    CK(cudaStreamWaitEvent(st, xphs_ev, capturing(st) ? cudaEventWaitExternal : cudaEventWaitDefault));
  }
  void io_late_ready(cudaStream_t st) {   // before the first stage's update_uv reads u_lon, v_lat
    if (!cur_io_late || late_waited) return;
    late_waited = true;
    if (dry) return;
    CK(cudaStreamWaitEvent(st, xlate_ev, capturing(st) ? cudaEventWaitExternal : cudaEventWaitDefault));
  }
  void io_tracers_ready(cudaStream_t st) {   // before the tracer step reads q
    if (!cur_io_wait || io_waited) return;
    io_waited = true;
    if (dry) return;
    CK(cudaStreamWaitEvent(st, xin_ev, capturing(st) ? cudaEventWaitExternal : cudaEventWaitDefault));
  }

  void step_io(int m, const std::vector<IoItem> &in, int nsteps, const std::vector<IoItem> &out) override {
    // every field name is known before anything moves
    for (const std::vector<IoItem> *v : {&in, &out})
      for (const IoItem &x : *v)
        if (x.tracer < 0) {
          R *pr;
          double *pd;
          locate(slots[m * 3 + old_i], m, x.name, &pr, &pd);
        }
    const bool overlap = nm == 1 && ntr > 0 && nsteps > 0;
    const int nlon = grid.nlon;
    // an overlapped item: registered host rows, the device field (R or FP64)
    // and, for R fields, a slice of the FP64 staging area
    struct Xfer {
      double *host;
      size_t pitch, lstride, rows;
      int nrow, nk;
      R *pr, *pr2;
      double *pd;
      size_t stage;   // offset in xstage (R fields)
      std::string name;
      int tracer;
    };
    std::vector<Xfer> in_main, in_x, out_x, out_main;
    std::vector<const IoItem *> in_sync, out_sync;
    size_t nstage = 0;
    auto plan = [&](const IoItem &x, bool input, std::vector<Xfer> &to) {
      int nrow = grid.nlat, nk = grid.nlev;
      if (x.tracer < 0) {
        FieldInfo f = info(x.name);
        nrow = f.nrow;
        nk = f.nk;
      }
      size_t pitch = 0, lstride = 0;
      const double *h = overlap ? io_rows(x.view, nrow, nk, pitch, lstride) : nullptr;
      if (!h) return false;
      Xfer t{const_cast<double *>(h), pitch, lstride, (size_t)nrow * nk, nrow, nk, nullptr, nullptr, nullptr, 0,
             x.name, x.tracer};
      // the device fields of an input; an output's are found again after the
      // step (download), these give its type
      if (x.tracer >= 0) {
        t.pr = q[((size_t)m * 2 + 0) * ntr + x.tracer];
        if (input) t.pr2 = q[((size_t)m * 2 + 1) * ntr + x.tracer];   // both levels, as gmc_set_tracer
      }
      if (t.pr || t.tracer < 0) {
        if (t.tracer < 0) locate(slots[m * 3 + old_i], m, x.name, &t.pr, &t.pd);
        if (t.pr) {
          t.stage = nstage;
          nstage += t.rows * nlon;
        }
      }
      to.push_back(t);
      return true;
    };
    for (const IoItem &x : in)
      if (!plan(x, true, x.tracer < 0 ? in_main : in_x)) in_sync.push_back(&x);
    for (const IoItem &x : out)
      if (!plan(x, false, x.tracer < 0 ? out_x : out_main)) out_sync.push_back(&x);
    // the inputs that take the calls' own paths first (each synchronous)
    for (const IoItem *x : in_sync) {
      if (x->tracer >= 0) set_tracer(m, x->tracer, x->view);
      else set_field(m, x->name, x->view);
    }
    if (nstage || !in_main.empty() || !in_x.empty() || !out_x.empty() || !out_main.empty()) {
      io_streams();
      io_stage(std::max<size_t>(nstage, 1));
    }
    auto blocks = [](size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); };
    // the rows of a view: one pitched copy when its levels follow each other
    // at the row pitch, else one per level
    auto copy_rows = [&](const Xfer &t, double *dev, bool h2d, cudaStream_t st) {
      const size_t w = nlon * sizeof(double);
      const bool one = t.nk == 1 || t.lstride == t.pitch * t.nrow;
      for (int k = 0; k < (one ? 1 : t.nk); ++k) {
        double *d = dev + (size_t)k * t.nrow * nlon;
        char *h = reinterpret_cast<char *>(t.host) + (size_t)k * t.lstride;
        const size_t rows = one ? t.rows : (size_t)t.nrow;
        if (h2d) CK(cudaMemcpy2DAsync(d, w, h, t.pitch, w, rows, cudaMemcpyHostToDevice, st));
        else CK(cudaMemcpy2DAsync(h, t.pitch, d, w, w, rows, cudaMemcpyDeviceToHost, st));
      }
    };
    auto upload = [&](const Xfer &t, cudaStream_t st) {
      double *dst = t.pr ? xstage + t.stage : t.pd;
      copy_rows(t, dst, true, st);
      if (t.pr) {
        const size_t n = t.rows * nlon;
        k_from_f64<R><<<blocks(n), 256, 0, st>>>(xstage + t.stage, n, t.pr, t.pr2);
        CK(cudaGetLastError());
      }
    };
    auto download = [&](const Xfer &t, cudaStream_t st) {
      // the state after the step: its new slot and tracer time level
      R *pr = nullptr;
      double *pd = nullptr;
      if (t.tracer >= 0) pr = q[((size_t)m * 2 + q_old) * ntr + t.tracer];
      else locate(slots[m * 3 + old_i], m, t.name, &pr, &pd);
      const double *src = pd;
      if (pr) {
        const size_t n = t.rows * nlon;
        k_to_f64<R><<<blocks(n), 256, 0, st>>>(pr, n, xstage + t.stage);
        CK(cudaGetLastError());
        src = xstage + t.stage;
      }
      copy_rows(t, const_cast<double *>(src), false, st);
    };
    // pt, then u_lon, v_lat, phs on xstream while the first stage starts
    // (see xpt_ev); other fields on the context stream ahead of the step;
    // then the tracers on xstream, which the first step's tracer advection
    // waits for
    std::vector<Xfer> in_pt, in_phs, in_late, in_early;
    for (const Xfer &t : in_main) {
      if (t.name == "pt") in_pt.push_back(t);
      else if (t.name == "phs") in_phs.push_back(t);
      else if (t.name == "u_lon" || t.name == "v_lat") in_late.push_back(t);
      else in_early.push_back(t);
    }
    for (const Xfer &t : in_early) upload(t, stream);
    if (!in_pt.empty() || !in_phs.empty() || !in_late.empty() || !in_x.empty()) {
      CK(cudaEventRecord(xin_ev, stream));
      CK(cudaStreamWaitEvent(xstream, xin_ev, 0));
    }
    if (!in_pt.empty()) {
      for (const Xfer &t : in_pt) upload(t, xstream);
      CK(cudaEventRecord(xpt_ev, xstream));
      io_pt = true;
    }
    if (!in_phs.empty()) {
      for (const Xfer &t : in_phs) upload(t, xstream);
      CK(cudaEventRecord(xphs_ev, xstream));
      io_phs = true;
    }
    if (!in_late.empty()) {
      for (const Xfer &t : in_late) upload(t, xstream);
      CK(cudaEventRecord(xlate_ev, xstream));
      io_late = true;
    }
    if (!in_x.empty()) {
      for (const Xfer &t : in_x) upload(t, xstream);
      CK(cudaEventRecord(xin_ev, xstream));
      io_wait = true;
    }
    // after the last step's launches: its fields once its dynamics are done
    // (xstream), the tracers after the step (context stream)
    if (!out_x.empty() || !out_main.empty()) {
      io_rec = !out_x.empty();
      io_qout = !out_main.empty();
      after_last = [&]() {
        if (!out_x.empty()) {
          // pt and phs first, from the last stage's update_pt on when recorded
          auto early = [&](const Xfer &t) { return ptf_recorded && (t.name == "pt" || t.name == "phs"); };
          bool any_early = false;
          for (const Xfer &t : out_x) any_early = any_early || early(t);
          if (any_early) {
            CK(cudaStreamWaitEvent(xstream, xptf_ev, 0));
            for (const Xfer &t : out_x)
              if (early(t)) download(t, xstream);
          }
          CK(cudaStreamWaitEvent(xstream, xdyn_ev, 0));
          for (const Xfer &t : out_x)
            if (!early(t)) download(t, xstream);
        }
        for (const Xfer &t : out_main) {
          if (q_piped) {   // each tracer once its own advection is done
            CK(cudaStreamWaitEvent(qstream, qev[(size_t)t.tracer], 0));
            download(t, qstream);
          } else {
            download(t, stream);
          }
        }
      };
    }
    struct Reset {
      Engine *e;
      ~Reset() {
        e->io_wait = e->io_rec = e->io_qout = e->q_piped = e->io_pt = e->io_late = e->ptf_recorded = false;
        e->io_phs = false;
        e->after_last = nullptr;
        if (e->xstream) cudaStreamSynchronize(e->xstream);
        if (e->qstream) cudaStreamSynchronize(e->qstream);
      }
    } reset{this};
    step(nsteps);
    if (xstream) CK(cudaStreamSynchronize(xstream));
    if (qstream) CK(cudaStreamSynchronize(qstream));
    for (const IoItem *x : out_sync) {
      if (x->tracer >= 0) get_tracer(m, x->tracer, x->view);
      else get_field(m, x->name, x->view);
    }
  }

  // Operator entry point: one horizontal FFSL flux with pool-allocated scratch.
  void ffsl_hflx(const gmc_ffsl_fields &f, double dt) override {
    if (!f.q || !f.u || !f.v || !f.mfx || !f.mfy || !f.cflx || !f.cfly || !f.divx || !f.divy || !f.qmfx || !f.qmfy)
      throw ApiError{GMC_EINVAL, "null field pointer"};
    R *scr = nullptr;
    const size_t n = full3();
    CK(cudaMallocAsync((void **)&scr, ffsl_scratch_bytes(), stream));
    BatchView<R> b{};
    b.u = (const R *)f.u; b.v = (const R *)f.v; b.mfx = (const R *)f.mfx; b.mfy = (const R *)f.mfy;
    b.cflx = (const R *)f.cflx; b.cfly = (const R *)f.cfly; b.divx = (const R *)f.divx; b.divy = (const R *)f.divy;
    launch_ffsl_hflx<R>(dg, L, b, (const R *)f.q, scr, scr + n, (R *)f.qmfx, (R *)f.qmfy, dt);
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(scr, stream);
    if (e != cudaSuccess) throw CudaError(std::string("ffsl_hflx: ") + cudaGetErrorString(e));
    CK(cudaStreamSynchronize(stream));
  }

  // Bytes of the scratch of one horizontal FFSL flux: its intermediates qx, qy
  // (two cell fields), the size the no-allocation entry point documents.
  size_t ffsl_scratch_bytes() const override { return 2 * full3() * sizeof(R); }

  // The same flux with the scratch supplied by the caller (no allocation).
  void ffsl_hflx_in(const gmc_ffsl_fields &f, double dt, void *scratch) override {
    if (!f.q || !f.u || !f.v || !f.mfx || !f.mfy || !f.cflx || !f.cfly || !f.divx || !f.divy || !f.qmfx || !f.qmfy)
      throw ApiError{GMC_EINVAL, "null field pointer"};
    R *scr = static_cast<R *>(scratch);
    const size_t n = full3();
    BatchView<R> b{};
    b.u = (const R *)f.u; b.v = (const R *)f.v; b.mfx = (const R *)f.mfx; b.mfy = (const R *)f.mfy;
    b.cflx = (const R *)f.cflx; b.cfly = (const R *)f.cfly; b.divx = (const R *)f.divx; b.divy = (const R *)f.divy;
    launch_ffsl_hflx<R>(dg, L, b, (const R *)f.q, scr, scr + n, (R *)f.qmfx, (R *)f.qmfy, dt);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
  }

  // adv_accum_wind for the static tracer batch (adv_mod.F90:420-455 with
  // adv_batch_accum_uv_cell / _mf_cell / _we_lev, adv_batch_mod.F90:218-632):
  // the first call of a cycle copies, the next nstep-1 add, the last averages
  // over nstep+1 samples and only then refreshes the Courant numbers.  At the
  // run prologue the mass fluxes and half-level masses are still zero.
  void accum_wind(int m, const Slot<R> &s, bool prologue) {
    TracerBatch<R> &b = tb[m];
    const double dt_adv = grid.cfg.dt_adv;
    auto cycle = [&](int &step, int &mode) {
      if (step == 0) { mode = 0; step = step + 1; }
      else if (step == nstep_adv) { mode = 2; step = 0; }
      else { mode = 1; step = step + 1; }
    };
    const double div = nstep_adv + 1;
    int mode_uv, mode_mf, mode_we;
    cycle(uv_step, mode_uv);
    cycle(mf_step, mode_mf);
    cycle(we_step, mode_we);
    AccumSet<R> set{};
    set.e[0] = {b.u, s.u_f, full3(), mode_uv, div};
    set.e[1] = {b.v, s.v_f, half3(), mode_uv, div};
    set.e[2] = {b.mfx, prologue ? nullptr : s.mfx_lon, full3(), mode_mf, div};
    set.e[3] = {b.mfy, prologue ? nullptr : s.mfy_lat, half3(), mode_mf, div};
    set.e[4] = {b.we, prologue ? nullptr : s.we_lev, lev3(), mode_we, div};
    set.count = 5;
    K("tracer_accum", 2, [&] {
      launch_accum_multi<R>(L, set);
      launch_half_level_mass<R>(dg, L, prologue ? SurfP<R>{nullptr, nullptr} : s.surf(), b.m_lev, mode_we, div);
    });
    if (uv_step == 0) K("tracer_batch_cfl", 1, [&] { launch_batch_cfl<R>(dg, L, b.u, b.v, b.cflx, b.cfly, b.divx, b.divy, dt_adv); });
    if (we_step == 0) K("tracer_batch_cflz", 1, [&] { launch_batch_cflz<R>(dg, L, b.we, b.m_lev, b.cflz, dt_adv); });
  }

  // adv_run (adv_mod.F90:152-312) after the dynamics of a step.
  void adv_run(int m, const Slot<R> &n, bool advect) {
    TracerBatch<R> &b = tb[m];
    Work<R> &w = work[m];
    const double dt_adv = grid.cfg.dt_adv;
    accum_wind(m, n, false);
    if (advect) {
      io_tracers_ready(L.stream);   // tracer inputs of gmc_step_io
      BatchView<R> bv{};
      bv.u = b.u; bv.v = b.v; bv.mfx = b.mfx; bv.mfy = b.mfy;
      bv.cflx = b.cflx; bv.cfly = b.cfly; bv.divx = b.divx; bv.divy = b.divy; bv.cflz = b.cflz;
      // tracers on their own streams unless profiling (whose events time
      // the context stream) or pipelined with their transfers back
      const bool qpipe = cur_io_qout;
      if (qpipe) q_piped = true;
      const bool tfork = tracer_streams() && !prof && !qpipe;
      if (tfork && !dry) {
        CK(cudaEventRecord(tfork_ev, L.stream));
        for (cudaStream_t st : tstreams) CK(cudaStreamWaitEvent(st, tfork_ev, 0));
      }
      for (int l = 0; l < ntr; ++l) {
        R *qo = q[((size_t)m * 2 + q_old) * ntr + l], *qn = q[((size_t)m * 2 + (1 - q_old)) * ntr + l];
        Launch Lt = L;
        R *qx = w.qx, *qy = w.qy, *fx = w.ptf_lon, *fy = w.ptf_lat;
        if (tfork) {
          Lt.stream = tstreams[l];
          qx = tsc[l].qx; qy = tsc[l].qy; fx = tsc[l].fx; fy = tsc[l].fy;
        }
        ffsl3(Lt, bv, qo, qx, qy, fx, fy, dt_adv);
        K("tracer_horizontal", 1, [&] { launch_tracer_horizontal<R>(dg, Lt, qo, qn, fx, fy, b.old_surf(), n.surf(), dt_adv); });
        K("tracer_vertical", 1, [&] { launch_tracer_vertical<R>(dg, Lt, qn, b.cflz, b.we, n.surf(), dt_adv); });
        K("tracer_lon_damp", 1, [&] { launch_tracer_lon_damp<R>(dg, Lt, qn); });
        if (qpipe && !dry)
          CK(cudaEventRecordWithFlags(qev[(size_t)l], Lt.stream,
                                      capturing(Lt.stream) ? cudaEventRecordExternal : cudaEventRecordDefault));
      }
      if (tfork && !dry) {
        for (int t = 0; t < ntr; ++t) {
          CK(cudaEventRecord(tevents[t], tstreams[t]));
          CK(cudaStreamWaitEvent(L.stream, tevents[t], 0));
        }
      }
    }
    io_tracers_ready(L.stream);   // a step without tracer advection still orders them
    // copy_old_m
    if (!dry) {
      CK(cudaMemcpyAsync(b.old_phs_f, n.phs_f, two_d() * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
      if (b.old_psr) CK(cudaMemcpyAsync(b.old_psr, n.psr, two_d() * sizeof(float), cudaMemcpyDeviceToDevice, L.stream));
    }
  }

  cudaEvent_t take_event() {
    if (!event_pool.empty()) {
      cudaEvent_t e = event_pool.back();
      event_pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    return e;
  }
  int prof_index(const char *name) {
    for (size_t t = 0; t < prof_table.size(); ++t)
      if (prof_table[t].name == name) return (int)t;
    prof_table.push_back(Prof{name, 0, 0});
    return (int)prof_table.size() - 1;
  }
  // Launch group `name` of nk kernels; bracketed by events when profiling.
  template <class F>
  void K(const char *name, int nk, F &&f) {
    launches += nk;
    if (dry) return;   // a captured graph replays these launches
    if (!prof) {
      f();
      return;
    }
    cudaEvent_t a = take_event(), b = take_event();
    CK(cudaEventRecord(a, stream));
    f();
    CK(cudaEventRecord(b, stream));
    prof_pending.push_back({prof_index(name), {a, b}});
  }
  void prof_collect() {
    for (auto &p : prof_pending) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, p.second.first, p.second.second));
      prof_table[p.first].ms += ms;
      prof_table[p.first].count += 1;
      event_pool.push_back(p.second.first);
      event_pool.push_back(p.second.second);
    }
    prof_pending.clear();
  }

  // horizontal FFSL fluxes fx, fy of q (the launches of launch_ffsl_hflx,
  // profiled per kernel): y inner pass, both x passes, y outer pass
  void ffsl3(const Launch &La, const BatchView<R> &b, const R *qf, R *qx, R *qy, R *fx, R *fy, double dt) {
    K("ffsl_inner_y", 1, [&] { launch_ffsl_inner_y<R>(dg, La, b, qf, qy, dt); });
    K("ffsl_x2", 1, [&] { launch_ffsl_x2<R>(dg, La, b, qf, qy, qx, fx, dt); });
    K("ffsl_hflx_y", 1, [&] { launch_hflx_y<R>(dg, La, b, qx, fy); });
  }

  // operators_prepare forward list (operators_mod.F90:117-122)
  void forward_prepare(int m, const Slot<R> &s, double dt) { forward_prepare_w(work[m], s, dt); }
  void forward_prepare_w(Work<R> &w, const Slot<R> &s, double dt) {
    K("mass_flux", 1, [&] { launch_mass_flux<R>(dg, L, s); });
    if (!dg.tangent_inline) K("tangent_winds", 1, [&] { launch_tangent_winds<R>(dg, L, s, w); });
    K("kinetic_energy", 1, [&] { launch_kinetic_energy<R>(dg, L, s, w); });
    K("pv", 1, [&] { launch_pv<R>(dg, L, s, w); });
    K("pv_edges", 1, [&] { launch_pv_edges<R>(dg, L, s, w, dt); });
  }

  // space_operators forward pass (gmcore_mod.F90:467-528)
  void forward(int m, const Slot<R> &s, double dt) { forward_w(work[m], s, dt); }
  void forward_w(Work<R> &w, const Slot<R> &s, double dt) {
    if (dyn_split()) {
      forward_split(w, s, dt);
      return;
    }
    forward_prepare_w(w, s, dt);
    if (grid.cfg.baroclinic) {
      K("batch_cfl", 1, [&] { launch_batch_cfl<R>(dg, L, s.u_f, s.v_f, w.cflx, w.cfly, w.divx, w.divy, dt); });
      K("column_mass", 1, [&] { launch_column_mass<R>(dg, L, s, w, dt); });
      BatchView<R> b{};
      b.u = s.u_f; b.v = s.v_f; b.mfx = s.mfx_lon; b.mfy = s.mfy_lat;
      b.cflx = w.cflx; b.cfly = w.cfly; b.divx = w.divx; b.divy = w.divy; b.cflz = w.cflz;
      io_pt_ready(L.stream);   // pt of gmc_step_io
      ffsl3(L, b, s.pt, w.qx, w.qy, w.ptf_lon, w.ptf_lat, dt);
      K("pt_tendency", 1, [&] { launch_pt_tendency<R>(dg, L, s, w); });
    } else {
      K("swm_dgz", 1, [&] { launch_swm_dgz<R>(dg, L, s, w); });
    }
    K("momentum_tend", 1, [&] { launch_momentum_tend<R>(dg, L, s, w); });
  }

  // The same launches as forward_w on two streams.  Side: batch_cfl, the y
  // inner pass, (after mass_flux) the x passes and the y outer pass, (after
  // column_mass) pt_tendency.  Context: mass_flux, column_mass, tangent_winds,
  // kinetic_energy, pv, pv_edges, momentum_tend; the context stream joins the
  // side stream before the backward pass.  The two chains write disjoint work
  // fields.
  void forward_split(Work<R> &w, const Slot<R> &s, double dt) {
    Launch Ls = L;
    Ls.stream = dside;
    auto edge = [&](cudaEvent_t e, cudaStream_t from, cudaStream_t to) {
      if (dry) return;   // a captured graph holds the dependency
      CK(cudaEventRecord(e, from));
      CK(cudaStreamWaitEvent(to, e, 0));
    };
    edge(dfork_ev, L.stream, dside);
    // side stream: the potential-temperature transport, which needs the
    // Courant numbers first, the mass fluxes from the x passes on and the
    // column quantities last
    K("batch_cfl", 1, [&] { launch_batch_cfl<R>(dg, Ls, s.u_f, s.v_f, w.cflx, w.cfly, w.divx, w.divy, dt); });
    BatchView<R> b{};
    b.u = s.u_f; b.v = s.v_f; b.mfx = s.mfx_lon; b.mfy = s.mfy_lat;
    b.cflx = w.cflx; b.cfly = w.cfly; b.divx = w.divx; b.divy = w.divy; b.cflz = w.cflz;
    io_pt_ready(dside);   // pt of gmc_step_io
    K("ffsl_inner_y", 1, [&] { launch_ffsl_inner_y<R>(dg, Ls, b, s.pt, w.qy, dt); });
    // context stream: mass fluxes, then the column sweep (which the pt
    // tendency needs) ahead of the PV chain, so that the two chains are of
    // about equal length
    K("mass_flux", 1, [&] { launch_mass_flux<R>(dg, L, s); });
    if (!dry) CK(cudaEventRecord(dmf_ev, L.stream));
    K("column_mass", 1, [&] { launch_column_mass<R>(dg, L, s, w, dt); });
    if (!dry) CK(cudaEventRecord(dcm_ev, L.stream));
    if (!dry) CK(cudaStreamWaitEvent(dside, dmf_ev, 0));
    K("ffsl_x2", 1, [&] { launch_ffsl_x2<R>(dg, Ls, b, s.pt, w.qy, w.qx, w.ptf_lon, dt); });
    K("ffsl_hflx_y", 1, [&] { launch_hflx_y<R>(dg, Ls, b, w.qx, w.ptf_lat); });
    if (!dry) CK(cudaStreamWaitEvent(dside, dcm_ev, 0));
    K("pt_tendency", 1, [&] { launch_pt_tendency<R>(dg, Ls, s, w); });
    if (!dry) CK(cudaEventRecord(dpt_ev, dside));
    if (!dg.tangent_inline) K("tangent_winds", 1, [&] { launch_tangent_winds<R>(dg, L, s, w); });
    K("kinetic_energy", 1, [&] { launch_kinetic_energy<R>(dg, L, s, w); });
    K("pv", 1, [&] { launch_pv<R>(dg, L, s, w); });
    K("pv_edges", 1, [&] { launch_pv_edges<R>(dg, L, s, w, dt); });
    K("momentum_tend", 1, [&] { launch_momentum_tend<R>(dg, L, s, w); });
    if (!dry) CK(cudaStreamWaitEvent(L.stream, dpt_ev, 0));
  }

  // step_forward_backward (time_schemes_mod.F90:102-118)
  void stage(int m, int o, int s, int n, double dt) {
    stage_io(slots[m * 3 + o], slots[m * 3 + s], slots[m * 3 + n], work[m], dt);
  }
  void stage_io(const Slot<R> &O, const Slot<R> &S, const Slot<R> &N, Work<R> &w, double dt) {
    forward_w(w, S, dt);
    io_phs_ready(L.stream);    // phs of gmc_step_io
    if (grid.cfg.baroclinic) {
      K("update_phs", 1, [&] { launch_update_phs<R>(dg, L, O, N, w, dt); });
      K("update_pt", 1, [&] { launch_update_pt<R>(dg, L, O, N, w, dt); });
      if (stage_last && cur_io_rec && grid.cfg.forcing == GMC_FORCING_NONE) {   // pt, phs final (xptf_ev)
        ptf_recorded = true;
        if (!dry)
          CK(cudaEventRecordWithFlags(xptf_ev, L.stream,
                                      capturing(L.stream) ? cudaEventRecordExternal : cudaEventRecordDefault));
      }
      K("column_backward", 1, [&] { launch_column_backward<R>(dg, L, N, w); });
    } else {
      K("update_gz", 1, [&] { launch_update_gz<R>(dg, L, O, N, w, dt); });
    }
    io_late_ready(L.stream);   // u_lon, v_lat of gmc_step_io
    K("update_uv", 1, [&] { launch_update_uv<R>(dg, L, O, N, w, dt); });
  }

  void prepare() override {
    uv_step = mf_step = we_step = 0;
    alert_last = -grid.cfg.dt_adv;
    curr_time = 0;
    alert_ring = false;
    for (int m = 0; m < nm; ++m) {
      const Slot<R> &s = slots[m * 3 + old_i];
      launch_filter_prologue<R>(dg, L, s);
      launch_surface_rel<R>(dg, L, s);
      launch_check_columns<R>(dg, L, s);   // calc_m of the prologue's operators_prepare
      if (ntr > 0) {
        // the prologue's copy_old_m sees the layer mass before operators_prepare
        CK(cudaMemsetAsync(tb[m].old_phs_f, 0, two_d() * sizeof(double), stream));
        if (tb[m].old_psr) CK(cudaMemsetAsync(tb[m].old_psr, 0, two_d() * sizeof(float), stream));
        int save_uv = uv_step, save_mf = mf_step, save_we = we_step;
        if (m > 0) { uv_step = save_uv; }
        accum_wind(m, s, true);
        if (m + 1 < nm) { uv_step = save_uv; mf_step = save_mf; we_step = save_we; }
      }
      forward_prepare(m, s, grid.cfg.dt_dyn);   // operators_prepare(blocks, old, dt_dyn)
      if (grid.cfg.baroclinic) {
        // calc_mf's accum_uv_cell of the mass batch (operators_mod.F90:556): the
        // prologue checks its Courant numbers as the reference does; every
        // forward pass recomputes them
        Work<R> &w = work[m];
        launch_batch_cfl<R>(dg, L, s.u_f, s.v_f, w.cflx, w.cfly, w.divx, w.divy, grid.cfg.dt_dyn);
      }
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    prepared = true;
    time_step = 0;
  }

  // -------------------------------------------------------------------------
  // Tangent-linear and adjoint of the shallow-water step (FP64).
  //
  // States X[0..nst] hold the step's start state and the stage outputs
  // (stage st: old X[0], star X[S(st)], new X[st+1]); D[] and A[] are their
  // tangents and adjoints.  The adjoint re-runs the step's stages from its
  // start state, then walks the stages backwards: adjoint of the updates
  // (consumes A[new], adds to A[0]), adjoint of the forward pass at the star
  // state (adds to A[star]).  Step start states come from checkpoints every
  // `ckpt` steps and a forward recomputation inside each segment.
  // -------------------------------------------------------------------------
  struct Tlad {
    Arena arena, zarena;                      // zarena: the adjoint work arrays, zeroed per stage
    Slot<double> X[4], D[4], A[4], DS, AS;   // DS/AS: tangent/adjoint work slots (mfx, mfy, pv*)
    Work<double> WF, DW, AW;
    bool ready = false;
    // checkpoint and segment storage of the adjoint, kept for repeated calls
    // with the same (segments, interval); two segment buffers (steps
    // [b k, b k + k) of xs/ws), so that the next segment is recomputed on
    // `rs` while the reverse sweep walks the current one
    Arena store;
    int store_nseg = -1, store_k = -1;
    std::vector<double *> cp;
    std::vector<std::array<Slot<double>, 4>> xs;
    std::vector<std::array<Work<double>, 3>> ws;
    cudaStream_t rs = nullptr;
    cudaEvent_t ev_fwd = nullptr, ev_rev = nullptr, ev_rec[2] = {nullptr, nullptr};
    void release_streams() {
      if (rs) cudaStreamDestroy(rs);
      for (cudaEvent_t e : {ev_fwd, ev_rev, ev_rec[0], ev_rec[1]})
        if (e) cudaEventDestroy(e);
      rs = nullptr;
      ev_fwd = ev_rev = ev_rec[0] = ev_rec[1] = nullptr;
    }
    // captured launch sequences keyed by the buffers they touch
    std::map<std::vector<intptr_t>, cudaGraphExec_t> graphs;
    void drop_graphs() {
      for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
      graphs.clear();
    }
  };
  std::unique_ptr<Tlad> tl;

  int tlad_stages() const { return grid.cfg.time_scheme == GMC_TIME_EULER ? 1 : 3; }
  double tlad_dt(int st) const {
    const double dt = grid.cfg.dt_dyn;
    if (grid.cfg.time_scheme == GMC_TIME_EULER) return dt;
    if (grid.cfg.time_scheme == GMC_TIME_PC2) return st == 2 ? dt : dt / 2.0;
    return st == 0 ? dt / 3.0 : (st == 1 ? dt / 2.0 : dt);
  }
  static int tlad_star(int st) { return st; }   // star of stage st is X[st] (X[0] for the first)

  void tlad_check() {
    if (!std::is_same<R, double>::value || grid.cfg.baroclinic)
      throw ApiError{GMC_EINVAL, "tangent-linear/adjoint: available for the FP64 shallow-water model"};
    if (nm != 1) throw ApiError{GMC_EINVAL, "tangent-linear/adjoint: one member"};
    if (grid.cfg.use_div_damp) throw ApiError{GMC_EINVAL, "tangent-linear/adjoint: divergence damping not differentiated"};
    if (!grid.cfg.pv_pole_stokes) throw ApiError{GMC_EINVAL, "tangent-linear/adjoint: needs pv_pole_stokes"};
    if (grid.cfg.pv_scheme == GMC_PV_TVD) throw ApiError{GMC_EINVAL, "tangent-linear/adjoint: pv_scheme tvd not differentiated"};
    if (!prepared || time_step != 0) throw ApiError{GMC_ESTATE, "tangent-linear/adjoint start from the prepared state (gmc_prepare)"};
  }

  size_t state_bytes() const { return (3 * full3() + 2 * half3() + 0) * sizeof(double) + 8 * 256; }
  // copy the prognostic fields (u, v, gz and their filtered copies)
  void copy_state(const Slot<R> &d, const Slot<R> &s) {
    CK(cudaMemcpyAsync(d.u_lon, s.u_lon, full3() * sizeof(R), cudaMemcpyDeviceToDevice, stream));
    CK(cudaMemcpyAsync(d.u_f, s.u_f, full3() * sizeof(R), cudaMemcpyDeviceToDevice, stream));
    CK(cudaMemcpyAsync(d.v_lat, s.v_lat, half3() * sizeof(R), cudaMemcpyDeviceToDevice, stream));
    CK(cudaMemcpyAsync(d.v_f, s.v_f, half3() * sizeof(R), cudaMemcpyDeviceToDevice, stream));
    CK(cudaMemcpyAsync(d.gz, s.gz, two_d() * sizeof(R), cudaMemcpyDeviceToDevice, stream));
    CK(cudaMemcpyAsync(d.gz_f, s.gz_f, two_d() * sizeof(R), cudaMemcpyDeviceToDevice, stream));
  }
  void zero_state(const Slot<R> &d) {
    CK(cudaMemsetAsync(d.u_lon, 0, full3() * sizeof(R), stream));
    CK(cudaMemsetAsync(d.u_f, 0, full3() * sizeof(R), stream));
    CK(cudaMemsetAsync(d.v_lat, 0, half3() * sizeof(R), stream));
    CK(cudaMemsetAsync(d.v_f, 0, half3() * sizeof(R), stream));
    CK(cudaMemsetAsync(d.gz, 0, two_d() * sizeof(R), stream));
    CK(cudaMemsetAsync(d.gz_f, 0, two_d() * sizeof(R), stream));
  }
  // a flat copy of the six prognostic fields, for checkpoints
  void flat_save(R *dst, const Slot<R> &s) {
    R *q = dst;
    for (auto f : {std::make_pair(s.u_lon, full3()), std::make_pair(s.u_f, full3()), std::make_pair(s.v_lat, half3()),
                   std::make_pair(s.v_f, half3()), std::make_pair(s.gz, two_d()), std::make_pair(s.gz_f, two_d())}) {
      CK(cudaMemcpyAsync(q, f.first, f.second * sizeof(R), cudaMemcpyDeviceToDevice, stream));
      q += f.second;
    }
  }
  void flat_load(const Slot<R> &d, const R *src, cudaStream_t on) {
    const R *q = src;
    for (auto f : {std::make_pair(d.u_lon, full3()), std::make_pair(d.u_f, full3()), std::make_pair(d.v_lat, half3()),
                   std::make_pair(d.v_f, half3()), std::make_pair(d.gz, two_d()), std::make_pair(d.gz_f, two_d())}) {
      CK(cudaMemcpyAsync(f.first, q, f.second * sizeof(R), cudaMemcpyDeviceToDevice, on));
      q += f.second;
    }
  }
  size_t flat_count() const { return 2 * full3() + 2 * half3() + 2 * two_d(); }

  void tlad_alloc() {
    if (tl && tl->ready) return;
    tl.reset(new Tlad());
    auto carve_all = [&](auto &a) {
      for (int t = 0; t < 4; ++t) {
        carve(a, tl->X[t], false);
        carve(a, tl->D[t], false);
        carve(a, tl->A[t], false);
      }
      carve(a, tl->DS, false);
      carve(a, tl->WF, false);
      carve(a, tl->DW, false);
    };
    auto carve_zero = [&](auto &a) {
      carve(a, tl->AS, false);
      carve(a, tl->AW, false);
    };
    Counter cnt, zcnt;
    carve_all(cnt);
    carve_zero(zcnt);
    tl->arena.reserve(cnt.used + 4096);
    tl->zarena.reserve(zcnt.used + 4096);
    carve_all(tl->arena);
    carve_zero(tl->zarena);
    for (int t = 0; t < 4; ++t) tl->X[t].gzs = tl->D[t].gzs = tl->A[t].gzs = gzs[0];
    tl->DS.gzs = tl->AS.gzs = gzs[0];
    tl->WF.gzs = tl->DW.gzs = tl->AW.gzs = gzs[0];
    CK(cudaStreamCreateWithFlags(&tl->rs, cudaStreamNonBlocking));
    for (cudaEvent_t *e : {&tl->ev_fwd, &tl->ev_rev, &tl->ev_rec[0], &tl->ev_rec[1]})
      CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    tl->ready = true;
  }

  // tangent slot of the star state with the tangent work arrays
  Slot<R> with_work(const Slot<R> &st, const Slot<R> &wk) {
    Slot<R> c = st;
    c.mfx_lon = wk.mfx_lon; c.mfy_lat = wk.mfy_lat; c.pv = wk.pv; c.pv_lon = wk.pv_lon; c.pv_lat = wk.pv_lat;
    return c;
  }

  void tlad_step_forward() {
    const int nst = tlad_stages();
    for (int st = 0; st < nst; ++st) stage_io(tl->X[0], tl->X[tlad_star(st)], tl->X[st + 1], tl->WF, tlad_dt(st));
    std::swap(tl->X[0], tl->X[nst]);
  }

  void upload3(const Slot<R> &d, const double *const h[3]) {
    CK(cudaMemcpyAsync(d.u_lon, h[0], full3() * sizeof(double), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d.v_lat, h[1], half3() * sizeof(double), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d.gz, h[2], two_d() * sizeof(double), cudaMemcpyHostToDevice, stream));
  }
  void download3(double *const h[3], const Slot<R> &s) {
    CK(cudaMemcpyAsync(h[0], s.u_lon, full3() * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(h[1], s.v_lat, half3() * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(h[2], s.gz, two_d() * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
  }

  void tlm(int nsteps, const double *const dx0[3], double *const dxn[3]) override {
    if constexpr (std::is_same<R, double>::value) {
      tlad_check();
      tlad_alloc();
      Tlad &T = *tl;
      const int nst = tlad_stages();
      copy_state(T.X[0], slots[old_i]);
      for (int t = 0; t < 4; ++t) zero_state(T.D[t]);
      upload3(T.D[0], dx0);
      launch_filter_prologue<R>(dg, L, T.D[0]);   // the prologue filters are linear
      for (int it = 0; it < nsteps; ++it) {
        for (int st = 0; st < nst; ++st) {
          const double dt = tlad_dt(st);
          const Slot<R> &S = T.X[tlad_star(st)];
          forward_w(T.WF, S, dt);
          const Slot<R> Tc = with_work(T.D[tlad_star(st)], T.DS);
          tl_forward_prepare(dg, L, S, T.WF, Tc, T.DW);
          launch_swm_dgz<R>(dg, L, Tc, T.DW);   // linear in the mass fluxes
          tl_momentum(dg, L, S, Tc, T.DW);
          launch_update_gz<R>(dg, L, T.X[0], T.X[st + 1], T.WF, dt);
          launch_update_uv<R>(dg, L, T.X[0], T.X[st + 1], T.WF, dt);
          launch_update_gz<R>(dg, L, T.D[0], T.D[st + 1], T.DW, dt);   // linear updates
          launch_update_uv<R>(dg, L, T.D[0], T.D[st + 1], T.DW, dt);
        }
        std::swap(T.X[0], T.X[nst]);
        std::swap(T.D[0], T.D[nst]);
      }
      CK(cudaGetLastError());
      copy_state(slots[old_i], T.X[0]);
      time_step += nsteps;
      download3(dxn, T.D[0]);
    } else {
      (void)nsteps; (void)dx0; (void)dxn;
      throw ApiError{GMC_EINVAL, "tangent-linear/adjoint: available for the FP64 shallow-water model"};
    }
  }

  // Launch the work f enqueues on the context stream as a CUDA graph captured
  // on first use under `key` (graphs off or profiling: launch directly).
  template <class F>
  void replay(const std::vector<intptr_t> &key, F &&f) {
    replay_on(stream, key, std::forward<F>(f));
  }
  // the same, the graph launched on stream `on` (captured on the context
  // stream, which the capture does not run anything on); without graphs the
  // work runs on the context stream
  template <class F>
  void replay_on(cudaStream_t on, const std::vector<intptr_t> &key, F &&f) {
    if (!graphs_on || prof) {
      f();
      return;
    }
    auto &gm = tl->graphs;
    auto gi = gm.find(key);
    if (gi == gm.end()) {
      cudaGraph_t gr = nullptr;
      CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      try {
        f();
      } catch (...) {
        cudaStreamEndCapture(stream, &gr);
        if (gr) cudaGraphDestroy(gr);
        throw;
      }
      CK(cudaStreamEndCapture(stream, &gr));
      cudaGraphExec_t ex = nullptr;
      cudaError_t e = cudaGraphInstantiate(&ex, gr, 0);
      cudaGraphDestroy(gr);
      if (e != cudaSuccess) throw CudaError(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
      gi = gm.emplace(key, ex).first;
    }
    CK(cudaGraphLaunch(gi->second, on));
  }
  static intptr_t ip(const void *p) { return reinterpret_cast<intptr_t>(p); }

  void adjoint(int nsteps, int ckpt, const double *const lam_n[3], double *const lam_0[3]) override {
    if constexpr (std::is_same<R, double>::value) {
      tlad_check();
      if (ckpt < 1) throw ApiError{GMC_EINVAL, "ckpt_every must be >= 1"};
      tlad_alloc();
      Tlad &T = *tl;
      const int nst = tlad_stages();
      const int k = std::min(ckpt, std::max(nsteps, 1));
      const int nseg = (nsteps + k - 1) / k;
      const size_t fc = flat_count();
      // checkpoints, and one segment's trajectory: for every step of the
      // segment the stage outputs (with the diagnostics forward_prepare left
      // in them when they served as star state) and the forward work of each
      // stage, so the reverse sweep recomputes nothing
      const int nbuf = nseg > 1 ? 2 : 1;
      if (T.store_nseg != nseg || T.store_k != k) {
        T.drop_graphs();
        T.store.release();
        T.cp.assign(nseg, nullptr);
        T.xs.assign(nbuf * k, {});
        T.ws.assign(nbuf * k, {});
        auto carve_store = [&](auto &a) {
          for (int c = 0; c < nseg; ++c) T.cp[c] = a.template take<R>(fc);
          for (int t = 0; t < nbuf * k; ++t) {
            for (int q = 0; q <= nst; ++q) carve(a, T.xs[t][q], false);
            for (int q = 0; q < nst; ++q) carve(a, T.ws[t][q], false);
          }
        };
        Counter cnt;
        carve_store(cnt);
        T.store.reserve(cnt.used + 4096);
        carve_store(T.store);
        for (int t = 0; t < nbuf * k; ++t) {
          for (int q = 0; q <= nst; ++q) T.xs[t][q].gzs = gzs[0];
          for (int q = 0; q < nst; ++q) T.ws[t][q].gzs = gzs[0];
          if (t % k > 0) T.xs[t][0] = T.xs[t - 1][nst];   // a step starts from the previous step's output
        }
        T.store_nseg = nseg;
        T.store_k = k;
      }
      auto &xs = T.xs;
      auto &ws = T.ws;
      // the segment recomputation runs on its own stream while the reverse
      // sweep walks the other buffer (the graphs replay there; without graphs
      // everything runs in order on the context stream)
      const bool overlap = graphs_on && !prof;
      cudaStream_t rstream = overlap ? T.rs : stream;
      // segment step t of buffer b: stages of step s0+t into the segment
      // storage (the final stage's update only when its output is needed)
      auto seg_step = [&](cudaStream_t on, int b, int t, int last) {
        replay_on(on, {2, b, t, last}, [&] {
          std::array<Slot<R>, 4> &X = xs[b * k + t];
          for (int st = 0; st < last; ++st) stage_io(X[0], X[tlad_star(st)], X[st + 1], ws[b * k + t][st], tlad_dt(st));
          if (last < nst) forward_w(ws[b * k + t][nst - 1], X[tlad_star(nst - 1)], tlad_dt(nst - 1));
        });
      };
      // forward sweep with checkpoints; the last segment runs straight into
      // the segment storage, so the reverse sweep starts without recomputing it
      const int slast = (nseg - 1) * k;
      copy_state(T.X[0], slots[old_i]);
      for (int it = 0; it < slast; ++it) {
        if (it % k == 0) flat_save(T.cp[it / k], T.X[0]);
        replay({1, ip(T.X[0].u_lon), ip(T.X[1].u_lon), ip(T.X[2].u_lon), ip(T.X[3].u_lon)}, [&] {
          for (int st = 0; st < nst; ++st) stage_io(T.X[0], T.X[tlad_star(st)], T.X[st + 1], T.WF, tlad_dt(st));
        });
        std::swap(T.X[0], T.X[nst]);
      }
      const int bl = (nseg - 1) % nbuf;   // buffer of segment seg: seg % nbuf
      copy_state(xs[bl * k][0], T.X[0]);
      for (int it = slast; it < nsteps; ++it) seg_step(stream, bl, it - slast, nst);
      copy_state(slots[old_i], xs[bl * k + nsteps - 1 - slast][nst]);   // the model ends at step nsteps
      CK(cudaEventRecord(T.ev_fwd, stream));   // checkpoints written
      // adjoint of the final state
      for (int t = 0; t <= nst; ++t) zero_state(T.A[t]);
      upload3(T.A[nst], lam_n);
      for (int seg = nseg - 1; seg >= 0; --seg) {
        const int b = seg % nbuf;
        const int s0 = seg * k, s1 = std::min(nsteps, s0 + k);
        if (seg >= 1) {
          // recompute segment seg-1 into the other buffer, once the checkpoints
          // exist and the reverse sweep of segment seg+1 (the buffer's last
          // reader) is done: xs[t][0] is step (seg-1) k + t's start state
          const int bp = (seg - 1) % nbuf;
          CK(cudaStreamWaitEvent(rstream, seg == nseg - 1 ? T.ev_fwd : T.ev_rev, 0));
          flat_load(xs[bp * k][0], T.cp[seg - 1], rstream);
          for (int t = 0; t < k; ++t) seg_step(rstream, bp, t, t + 1 < k ? nst : nst - 1);
          CK(cudaEventRecord(T.ev_rec[bp], rstream));
        }
        if (seg < nseg - 1) CK(cudaStreamWaitEvent(stream, T.ev_rec[b], 0));   // segment seg recomputed
        for (int t = s1 - s0 - 1; t >= 0; --t) {
          replay({3, b, t, ip(T.A[0].u_lon), ip(T.A[nst].u_lon)}, [&] {
            std::array<Slot<R>, 4> &X = xs[b * k + t];
            for (int st = nst - 1; st >= 0; --st) {
              const double dt = tlad_dt(st);
              // clears the adjoint work (AS, AW up to AW.du) for the forward-pass adjoint
              ad_update(dg, L, T.A[0], T.A[st + 1], T.AW, T.AS.u_lon, (size_t)(T.AW.du - T.AS.u_lon), dt);
              ad_forward(dg, L, X[tlad_star(st)], ws[b * k + t][st], with_work(T.A[tlad_star(st)], T.AS), T.AW);
            }
          });
          // A[0] is the adjoint of the step's start state: it seeds the step
          // before; every A[st+1] was consumed (zeroed) by its stage's ad_update
          std::swap(T.A[0], T.A[nst]);
        }
        CK(cudaEventRecord(T.ev_rev, stream));   // buffer b free again
      }
      ad_prologue(dg, L, T.A[nst]);
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(stream));
      time_step += nsteps;
      download3(lam_0, T.A[nst]);
    } else {
      (void)nsteps; (void)ckpt; (void)lam_n; (void)lam_0;
      throw ApiError{GMC_EINVAL, "tangent-linear/adjoint: available for the FP64 shallow-water model"};
    }
  }

  // ---- CUDA graphs of one step and member streams ------------------------
  // A step's launches (kernels, arguments, pointers) are fixed by the slot
  // roles, the tracer cadence counters, whether tracers advect and the tracer
  // time level; each such state is captured once into a graph and replayed.
  // While a graph is replayed the host logic of the step still runs (dry
  // mode: launches skipped, counters advanced).
  struct GraphKey {
    int o, n, su, sm, sw, adv, qo, layout, io;   // io: gmc_step_io's wait (1) and record (2)
    bool operator<(const GraphKey &b) const {
      return std::tie(o, n, su, sm, sw, adv, qo, layout, io) <
             std::tie(b.o, b.n, b.su, b.sm, b.sw, b.adv, b.qo, b.layout, b.io);
    }
  };
  std::map<GraphKey, cudaGraphExec_t> graphs;
  bool dry = false;
  bool graphs_on = true;
  void set_graphs(bool on) override { graphs_on = on; }
  // ensemble members run on their own streams (forked from and joined to the
  // context stream) so that small grids fill the GPU
  std::vector<cudaStream_t> mstreams;
  std::vector<cudaEvent_t> mevents;
  cudaEvent_t fork_ev = nullptr;

  void member_streams() {
    if (nm <= 1 || !mstreams.empty()) return;
    const int ns = std::min(nm, 8);
    mstreams.resize(ns);
    mevents.resize(ns);
    for (int t = 0; t < ns; ++t) {
      CK(cudaStreamCreateWithFlags(&mstreams[t], cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&mevents[t], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
  }

  // Launch layouts of an ensemble step, all with identical results:
  // layout 0 launches each member's kernels separately, the members spread
  // over up to 8 streams; layout G > 0 splits the members into G groups of
  // consecutive members, each group one member-batched launch per operator
  // (grid z = member) on its own stream, so that G kernels of different kinds
  // overlap.  The autotuner below times them on the first steps of a context
  // and keeps the fastest.
  std::vector<int> layouts;     // candidates, in tuning order
  int layout = 0;               // in use
  bool tuned = true;            // false while candidates are being timed
  struct LayoutTiming { double ms = 0; int n = 0, queued = 0; };   // queued: timed, not yet read
  std::vector<LayoutTiming> layout_ms;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> tune_pending;

  int layout_in_use() const override { return layout; }
  bool set_layout(int lay) override {
    if (lay < 0) {
      setup_layouts();
      return true;
    }
    if (std::find(layouts.begin(), layouts.end(), lay) == layouts.end()) return false;
    layout = lay;
    tuned = true;
    return true;
  }
  bool layout_is_tuned() const override { return tuned; }
  void setup_layouts() {
    layouts.clear();
    layouts.push_back(0);
    if (batched_members)
      for (int G : {1, 2, 4, 8})
        if (G <= nm && (G == 1 || nm / G >= 2)) layouts.push_back(G);
    layout = 0;
    tuned = layouts.size() <= 1;
    layout_ms.assign(layouts.size(), LayoutTiming{});
  }
  // the candidate to run next while tuning: each is timed twice on replayed
  // graphs (its first step captures the graph and is not timed)
  int next_tuning_layout(bool &timed) {
    for (size_t c = 0; c < layouts.size(); ++c)
      if (layout_ms[c].n + layout_ms[c].queued < 2) {
        timed = captured_layouts.count(layouts[c]) > 0;
        return (int)c;
      }
    timed = false;
    return -1;
  }
  std::set<int> captured_layouts;
  void collect_tuning() {
    for (auto &p : tune_pending) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, p.second.first, p.second.second));
      layout_ms[p.first].ms += ms;
      layout_ms[p.first].n += 1;
      layout_ms[p.first].queued -= 1;
      event_pool.push_back(p.second.first);
      event_pool.push_back(p.second.second);
    }
    tune_pending.clear();
    bool done = true;
    for (const LayoutTiming &t : layout_ms) done = done && t.n >= 2;
    if (!done) return;
    size_t best = 0;
    for (size_t c = 1; c < layouts.size(); ++c)
      if (layout_ms[c].ms / layout_ms[c].n < layout_ms[best].ms / layout_ms[best].n) best = c;
    layout = layouts[best];
    tuned = true;
  }

  // The dynamics of one step for all members in member-batched launches, in
  // G groups on their own streams, then each member's tracer advection.
  void step_body_batched(int o, int n, bool ring, int G) {
    const double dt = grid.cfg.dt_dyn;
    const int t3 = 3 - o - n;
    const int su = uv_step, sm = mf_step, sw = we_step;
    const bool fork = G > 1 && !prof;
    if (fork && !dry) {
      CK(cudaEventRecord(fork_ev, stream));
      for (int t = 0; t < G; ++t) CK(cudaStreamWaitEvent(mstreams[t], fork_ev, 0));
    }
    const int per = (nm + G - 1) / G;
    try {
      for (int gi = 0; gi < G; ++gi) {
        const int m0 = gi * per, cnt = std::min(per, nm - m0);
        if (cnt <= 0) continue;
        L.members = cnt;
        if (fork) L.stream = mstreams[gi];
        switch (grid.cfg.time_scheme) {
          case GMC_TIME_EULER:
            stage(m0, o, o, n, dt);
            break;
          case GMC_TIME_PC2:
            stage(m0, o, o, n, dt / 2.0);
            stage(m0, o, n, t3, dt / 2.0);
            stage(m0, o, t3, n, dt);
            break;
          default:
            stage(m0, o, o, n, dt / 3.0);
            stage(m0, o, n, t3, dt / 2.0);
            stage(m0, o, t3, n, dt);
            break;
        }
        if (grid.cfg.forcing == GMC_FORCING_HELD_SUAREZ)   // test_forcing_run (gmcore_mod.F90:586)
          K("held_suarez", 1, [&] { launch_held_suarez<R>(dg, L, slots[m0 * 3 + n], dt); });
        if (grid.cfg.use_div_damp)
          K("div_damp", grid.cfg.div_damp_order == 4 ? 3 : 2,
            [&] { launch_div_damp<R>(dg, L, slots[m0 * 3 + n], work[m0].ke, work[m0].du); });
        if (grid.cfg.use_smag_damp)   // damp_run (damp_mod.F90:59-61)
          K("smag_damp", 3, [&] {
            launch_smag_damp<R>(dg, L, slots[m0 * 3 + n], work[m0].ke, work[m0].u_lat, work[m0].du, work[m0].dv, dt);
          });
      }
    } catch (...) {
      L.members = 1;
      L.stream = stream;
      throw;
    }
    L.members = 1;
    L.stream = stream;
    if (fork && !dry) {
      for (int t = 0; t < G; ++t) {
        CK(cudaEventRecord(mevents[t], mstreams[t]));
        CK(cudaStreamWaitEvent(stream, mevents[t], 0));
      }
    }
    if (ntr > 0) {
      for (int m = 0; m < nm; ++m) {
        uv_step = su; mf_step = sm; we_step = sw;   // every member runs the same cadence
        adv_run(m, slots[m * 3 + n], ring && time_step > 0);
      }
    }
  }

  // the launches of one step (all members) in launch layout `lay`
  void step_body(int o, int n, bool ring, int lay) {
    if (lay > 0) {
      step_body_batched(o, n, ring, lay);
      return;
    }
    const double dt = grid.cfg.dt_dyn;
    const int t3 = 3 - o - n;
    const int su = uv_step, sm = mf_step, sw = we_step;
    const bool fork = nm > 1 && !prof;
    if (fork && !dry) {
      CK(cudaEventRecord(fork_ev, stream));
      for (cudaStream_t st : mstreams) CK(cudaStreamWaitEvent(st, fork_ev, 0));
    }
    for (int m = 0; m < nm; ++m) {
      if (fork) L.stream = mstreams[m % mstreams.size()];
      switch (grid.cfg.time_scheme) {
        case GMC_TIME_EULER:
          stage_last = true;
          stage(m, o, o, n, dt);
          break;
        case GMC_TIME_PC2:
          stage(m, o, o, n, dt / 2.0);
          stage(m, o, n, t3, dt / 2.0);
          stage_last = true;
          stage(m, o, t3, n, dt);
          break;
        default:
          stage(m, o, o, n, dt / 3.0);
          stage(m, o, n, t3, dt / 2.0);
          stage_last = true;
          stage(m, o, t3, n, dt);
          break;
      }
      stage_last = false;
      const Slot<R> &N = slots[m * 3 + n];
      if (grid.cfg.forcing == GMC_FORCING_HELD_SUAREZ)   // test_forcing_run (gmcore_mod.F90:586)
        K("held_suarez", 1, [&] { launch_held_suarez<R>(dg, L, N, dt); });
      if (grid.cfg.use_div_damp)
        K("div_damp", grid.cfg.div_damp_order == 4 ? 3 : 2, [&] { launch_div_damp<R>(dg, L, N, work[m].ke, work[m].du); });
      if (grid.cfg.use_smag_damp)   // damp_run (damp_mod.F90:59-61)
        K("smag_damp", 3, [&] { launch_smag_damp<R>(dg, L, N, work[m].ke, work[m].u_lat, work[m].du, work[m].dv, dt); });
      io_dyn_done(L.stream);   // the new state's fields are final (gmc_step_io)
      if (ntr > 0) {
        uv_step = su; mf_step = sm; we_step = sw;   // every member runs the same cadence
        adv_run(m, N, ring && time_step > 0);
      }
    }
    L.stream = stream;
    if (fork && !dry) {
      for (size_t t = 0; t < mstreams.size(); ++t) {
        CK(cudaEventRecord(mevents[t], mstreams[t]));
        CK(cudaStreamWaitEvent(stream, mevents[t], 0));
      }
    }
  }

  cudaEvent_t ev_a = nullptr, ev_b = nullptr;
  void step(int nsteps) override {
    if (!prepared) throw ApiError{GMC_ESTATE, "gmc_prepare must be called after setting the state"};
    const double dt = grid.cfg.dt_dyn;
    if (!ev_a) {
      CK(cudaEventCreate(&ev_a));
      CK(cudaEventCreate(&ev_b));
    }
    const long launches0 = launches;
    CK(cudaEventRecord(ev_a, stream));
    // the FP32 surface pressure follows phs_f as set through the API
    if (kFP32 && grid.cfg.baroclinic)
      for (int m = 0; m < nm; ++m) K("surface_rel", 1, [&] { launch_surface_rel<R>(dg, L, slots[m * 3 + old_i]); });
    const bool use_graphs = graphs_on && !prof;
    for (int it = 0; it < nsteps; ++it) {
      const int o = old_i, n = new_i;
      cur_io_wait = io_wait && it == 0;
      cur_io_rec = io_rec && it == nsteps - 1;
      cur_io_qout = io_qout && it == nsteps - 1;
      cur_io_pt = io_pt && it == 0;
      cur_io_late = io_late && it == 0;
      cur_io_phs = io_phs && it == 0;
      io_waited = pt_waited = late_waited = phs_waited = false;
      // tracer alert: time_is_alerted(name) .and. time_step > 0 (adv_mod.F90:166, time_mod.F90:270-291)
      const bool ring = ntr > 0 && alert_last + grid.cfg.dt_adv <= curr_time + 1e-9 * grid.cfg.dt_adv;
      if (ring) alert_ring = true;
      // the launch layout of this step: the tuned one, or while tuning the next
      // candidate (all layouts give identical results)
      int lay = layout, cand = -1;
      bool timed = false;
      if (!tuned && use_graphs) {
        cand = next_tuning_layout(timed);
        if (cand >= 0) lay = layouts[cand];
      }
      if (use_graphs) {
        const GraphKey key{o, n, uv_step, mf_step, we_step, (ring && time_step > 0) ? 1 : 0, q_old, lay,
                           (cur_io_wait ? 1 : 0) | (cur_io_rec ? 2 : 0) | (cur_io_qout ? 4 : 0) |
                               (cur_io_pt ? 8 : 0) | (cur_io_late ? 16 : 0) | (cur_io_phs ? 32 : 0)};
        auto gi = graphs.find(key);
        if (gi == graphs.end()) {
          cudaGraph_t gr = nullptr;
          CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
          try {
            step_body(o, n, ring, lay);
          } catch (...) {
            cudaStreamEndCapture(stream, &gr);
            if (gr) cudaGraphDestroy(gr);
            throw;
          }
          CK(cudaStreamEndCapture(stream, &gr));
          cudaGraphExec_t ex = nullptr;
          cudaError_t e = cudaGraphInstantiate(&ex, gr, 0);
          cudaGraphDestroy(gr);
          if (e != cudaSuccess) throw CudaError(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
          gi = graphs.emplace(key, ex).first;
          timed = false;   // a capture step is not timed
        } else {
          dry = true;
          try {
            step_body(o, n, ring, lay);
          } catch (...) {
            dry = false;
            throw;
          }
          dry = false;
        }
        cudaEvent_t ta = nullptr, tb_ = nullptr;
        if (cand >= 0 && timed) {
          ta = take_event();
          tb_ = take_event();
          CK(cudaEventRecord(ta, stream));
        }
        CK(cudaGraphLaunch(gi->second, stream));
        if (ta) {
          CK(cudaEventRecord(tb_, stream));
          tune_pending.push_back({cand, {ta, tb_}});
          layout_ms[cand].queued += 1;
        }
        if (cand >= 0) captured_layouts.insert(lay);
      } else {
        step_body(o, n, ring, lay);
      }
      if (ntr > 0 && ring && time_step > 0) q_old = 1 - q_old;
      if (alert_ring) { alert_last = curr_time; alert_ring = false; }
      curr_time += dt;
      std::swap(old_i, new_i);
      ++time_step;
    }
    cur_io_wait = cur_io_rec = cur_io_qout = cur_io_pt = cur_io_late = cur_io_phs = false;
    if (after_last) after_last();
    CK(cudaEventRecord(ev_b, stream));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ev_a, ev_b));
    last_step_ms = ms;
    last_steps = nsteps;
    last_launches = launches - launches0;
    if (prof) prof_collect();
    if (!tune_pending.empty()) collect_tuning();
  }

  void diagnose(int m, gmc_diag *out) override {
    const Slot<R> &s = slots[m * 3 + old_i];
    launch_surface_rel<R>(dg, L, s);
    launch_diagnose<R>(dg, L, s, diag_partial, diag_out);
    double h[8];
    CK(cudaMemcpyAsync(h, diag_out, 7 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    out->tm = h[0];
    out->te_ke = h[1];
    out->te_ie = h[2];
    out->te_pe = h[3];
    out->tav = h[4];
    out->tpe = h[5];
    out->tpt = h[6];
    out->te = out->te_ke + out->te_ie + out->te_pe;
  }

  void output_diag(int m, double *ph, double *t, double *z, double *div, double *vor) override {
    const Slot<R> &s = slots[m * 3 + old_i];
    const bool bc = grid.cfg.baroclinic != 0;
    const size_t nf = full3(), nh = half3(), n2 = two_d();
    const size_t ncell = bc ? nf : n2;   // cell fields of the layout
    double *buf = nullptr;
    CK(cudaMallocAsync((void **)&buf, (4 * ncell + nh) * sizeof(double), stream));
    double *dph = buf, *dt = buf + ncell, *dz = buf + 2 * ncell, *ddiv = buf + 3 * ncell, *dvor = buf + 4 * ncell;
    launch_output_diag<R>(dg, stream, s, dph, dt, dz, ddiv, dvor);
    CK(cudaGetLastError());
    auto back = [&](double *host, const double *dev, size_t n) {
      if (host) CK(cudaMemcpyAsync(host, dev, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    };
    if (bc) {
      back(ph, dph, nf);
      back(t, dt, nf);
      back(vor, dvor, nh);
    }
    back(z, dz, ncell);
    back(div, ddiv, ncell);
    CK(cudaFreeAsync(buf, stream));
    CK(cudaStreamSynchronize(stream));
  }
  const Grid &host_grid() const override { return grid; }

  OutSnap snapshot(int m, bool history) override {
    const Slot<R> &s = slots[m * 3 + old_i];
    const bool bc = grid.cfg.baroclinic != 0;
    const size_t nf = full3(), nh = half3(), n2 = two_d(), ncell = bc ? nf : n2;
    size_t bytes = 0;
    auto add = [&](size_t n, size_t es) {
      const size_t off = bytes;
      bytes += (n * es + 255) & ~(size_t)255;
      return off;
    };
    const size_t o_u = add(nf, sizeof(R)), o_v = add(nh, sizeof(R)), o_gzs = add(n2, sizeof(double));
    const size_t o_pt = bc ? add(nf, sizeof(R)) : 0, o_phs = bc ? add(n2, sizeof(double)) : 0;
    const size_t o_gz = bc ? 0 : add(n2, sizeof(R)), o_pv = !bc && history ? add(nh, sizeof(R)) : 0;
    std::vector<size_t> o_q;
    for (int l = 0; l < ntr; ++l) o_q.push_back(add(nf, sizeof(R)));
    size_t o_d[5] = {0, 0, 0, 0, 0};   // ph, t, z, div, vor
    if (history) {
      for (int d = 0; d < 4; ++d) o_d[d] = add(ncell, sizeof(double));
      o_d[4] = add(nh, sizeof(double));
    }
    OutSnap o;
    o.fp32 = kFP32;
    CK(cudaMallocAsync((void **)&o.block, bytes, stream));
    try {
      fill_snapshot(o, s, m, history, bc, nf, nh, n2, o_u, o_v, o_gzs, o_pt, o_phs, o_gz, o_pv, o_q, o_d);
    } catch (...) {
      cudaFreeAsync(o.block, stream);
      if (o.ready) cudaEventDestroy(o.ready);
      throw;
    }
    return o;
  }
  void fill_snapshot(OutSnap &o, const Slot<R> &s, int m, bool history, bool bc, size_t nf, size_t nh, size_t n2,
                     size_t o_u, size_t o_v, size_t o_gzs, size_t o_pt, size_t o_phs, size_t o_gz, size_t o_pv,
                     const std::vector<size_t> &o_q, const size_t (&o_d)[5]) {
    char *b = o.block;
    auto copy = [&](size_t off, const void *src, size_t n) {
      CK(cudaMemcpyAsync(b + off, src, n, cudaMemcpyDeviceToDevice, stream));
      return (const void *)(b + off);
    };
    o.u = copy(o_u, s.u_lon, nf * sizeof(R));
    o.v = copy(o_v, s.v_lat, nh * sizeof(R));
    o.gzs = (const double *)copy(o_gzs, s.gzs, n2 * sizeof(double));
    if (bc) {
      o.pt = copy(o_pt, s.pt, nf * sizeof(R));
      o.phs = (const double *)copy(o_phs, s.phs, n2 * sizeof(double));
    } else {
      o.gz = copy(o_gz, s.gz, n2 * sizeof(R));
      if (history) o.pv = copy(o_pv, s.pv, nh * sizeof(R));
    }
    for (int l = 0; l < ntr; ++l) o.q.push_back(copy(o_q[(size_t)l], q[((size_t)m * 2 + q_old) * ntr + l], nf * sizeof(R)));
    if (history) {
      double *d[5];
      for (int k = 0; k < 5; ++k) d[k] = reinterpret_cast<double *>(b + o_d[k]);
      launch_output_diag<R>(dg, stream, s, d[0], d[1], d[2], d[3], d[4]);
      CK(cudaGetLastError());
      if (bc) {
        o.ph = d[0];
        o.t = d[1];
        o.vor = d[4];
      }
      o.z = d[2];
      o.div = d[3];
      diagnose(m, &o.diag);
    }
    CK(cudaEventCreateWithFlags(&o.ready, cudaEventDisableTiming));
    CK(cudaEventRecord(o.ready, stream));
  }

  // The first error raised on the device since the last read (the error
  // words are cleared): err[1] holds the first bit, err[0] all of them.
  unsigned read_error() override {
    unsigned h[2] = {0, 0};
    CK(cudaMemcpyAsync(h, err, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (h[0] | h[1]) {
      CK(cudaMemsetAsync(err, 0, 2 * sizeof(unsigned), stream));
      CK(cudaStreamSynchronize(stream));
    }
    return h[1] ? h[1] : h[0];
  }
};

// ---------------------------------------------------------------------------
// The C ABI
// ---------------------------------------------------------------------------
struct gmc_ctx {
  gmc_config cfg;
  std::unique_ptr<EngineBase> eng;
  std::string last_error;
  int lon_halo_width = 0;
  // the history or restart file being written in the background, and the
  // status it ended with (read after the join)
  std::thread bg;
  int bg_rc = GMC_OK;
  std::string bg_msg;
  ~gmc_ctx() {
    if (bg.joinable()) bg.join();
  }
};

namespace {

int fail(gmc_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

template <class F>
int guarded(gmc_ctx *ctx, F f) {
  try {
    return f();
  } catch (const ApiError &e) {
    return fail(ctx, e.code, e.msg);
  } catch (const CudaError &e) {
    return fail(ctx, GMC_ECUDA, e.msg);
  } catch (const std::bad_alloc &) {
    return fail(ctx, GMC_ENOMEM, "host allocation failed");
  } catch (const std::exception &e) {   // nothing crosses the C ABI as an exception
    return fail(ctx, GMC_EINVAL, std::string("unexpected error: ") + e.what());
  }
}

int error_word_status(gmc_ctx *ctx, unsigned w) {
  if (!w) return GMC_OK;
  if (w & ERR_NAN) return fail(ctx, GMC_ENAN, "non-finite value in the state");
  if (w & ERR_NONMONO) return fail(ctx, GMC_ENONMONO, "The pressure levels are not monotonic!");
  if (w & ERR_CFLX) return fail(ctx, GMC_ECFL, "cflx exceeds mesh%lon_halo_width");
  if (w & ERR_CFLY) return fail(ctx, GMC_ECFL, "cfly exceeds 1");
  if (w & ERR_CFLZ) return fail(ctx, GMC_ECFL, "cflz exceeds range");
  if (w & ERR_NEGTRACER) return fail(ctx, GMC_ENEGTRACER, "Negative tracer!");
  return fail(ctx, GMC_ECUDA, "unknown device error word");
}

gmc_config normalised(const gmc_config &c) {
  gmc_config n = c;
  // parse_namelist (namelist_mod.F90:227-249)
  if (!n.baroclinic) n.ke_scheme = 1;
  if (!(n.dt_adv > 0)) n.dt_adv = n.dt_dyn;
  return n;
}

// Copy the interior of a Fortran-bounded view into a packed [k][j][i] array.
// The view must have non-empty bounds covering the interior 1..nlon x 1..nrow x 1..nk.
bool check_view(const gmc_view *v, int nlon, int nrow, int nk, std::string &err) {
  if (!v || !v->data) { err = "null view"; return false; }
  for (int d = 0; d < 3; ++d)
    if (v->ub[d] < v->lb[d]) { err = "view bounds are empty"; return false; }
  if (v->lb[0] > 1 || v->ub[0] < nlon || v->lb[1] > 1 || v->ub[1] < nrow || v->lb[2] > 1 || v->ub[2] < nk) {
    err = "view does not cover the interior (" + std::to_string(nlon) + "x" + std::to_string(nrow) + "x" +
          std::to_string(nk) + ")";
    return false;
  }
  return true;
}

bool unpack_view(const gmc_view *v, int nlon, int nrow, int nk, std::vector<double> &out, std::string &err) {
  if (!v || !v->data) { err = "null view"; return false; }
  for (int d = 0; d < 3; ++d)
    if (v->ub[d] < v->lb[d]) { err = "view bounds are empty"; return false; }
  if (v->lb[0] > 1 || v->ub[0] < nlon || v->lb[1] > 1 || v->ub[1] < nrow || v->lb[2] > 1 || v->ub[2] < nk) {
    err = "view does not cover the interior (" + std::to_string(nlon) + "x" + std::to_string(nrow) + "x" +
          std::to_string(nk) + ")";
    return false;
  }
  const long n0 = v->ub[0] - v->lb[0] + 1, n1 = v->ub[1] - v->lb[1] + 1;
  out.resize((size_t)nlon * nrow * nk);
  size_t o = 0;
  for (int k = 1; k <= nk; ++k)
    for (int j = 1; j <= nrow; ++j) {
      const double *src = v->data + (size_t)(1 - v->lb[0]) + (size_t)n0 * ((size_t)(j - v->lb[1]) + (size_t)n1 * (k - v->lb[2]));
      std::memcpy(&out[o], src, nlon * sizeof(double));
      o += nlon;
    }
  return true;
}

bool pack_view(const gmc_view *v, int nlon, int nrow, int nk, const std::vector<double> &in, std::string &err) {
  std::vector<double> dummy;
  if (!v || !v->data) { err = "null view"; return false; }
  if (v->lb[0] > 1 || v->ub[0] < nlon || v->lb[1] > 1 || v->ub[1] < nrow || v->lb[2] > 1 || v->ub[2] < nk) {
    err = "view does not cover the interior";
    return false;
  }
  const long n0 = v->ub[0] - v->lb[0] + 1, n1 = v->ub[1] - v->lb[1] + 1;
  size_t o = 0;
  for (int k = 1; k <= nk; ++k)
    for (int j = 1; j <= nrow; ++j) {
      double *dst = v->data + (size_t)(1 - v->lb[0]) + (size_t)n0 * ((size_t)(j - v->lb[1]) + (size_t)n1 * (k - v->lb[2]));
      std::memcpy(dst, &in[o], nlon * sizeof(double));
      o += nlon;
    }
  return true;
}

void field_dims(const gmc_config &c, const std::string &name, int &nrow, int &nk) {
  nrow = c.nlat;
  nk = c.nlev;
  if (name == "v_lat" || name == "v_f" || name == "mfy_lat" || name == "pv" || name == "pv_lat") nrow = c.nlat - 1;
  if (name == "phs" || name == "phs_f" || name == "gzs" || name == "gz" || name == "gz_f") nk = 1;
  if (name == "we_lev") nk = c.nlev + 1;
}

// ---------------------------------------------------------------------------
// Scratch for gmc_ffsl_hflx_noalloc: a fixed device array that every GPU
// loading this library carries until the process exits.  Host code may not
// use the symbol itself as a device address; the address is looked up once
// per device with cudaGetSymbolAddress while that device is current.
// ---------------------------------------------------------------------------
constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;   // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_addr[kMaxDevices] = {};

// Device address of the scratch array on device `dev`.  The first call for a
// device makes that device current for the lookup and restores the caller's
// device afterwards.
int noalloc_scratch_address(int dev, void **out, std::string &err) {
  if (dev < 0 || dev >= kMaxDevices) { err = "device ordinal out of range"; return GMC_ECUDA; }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    if (e != cudaSuccess) { err = std::string("cudaGetDevice: ") + cudaGetErrorString(e); return GMC_ECUDA; }
    if (cur != dev && (e = cudaSetDevice(dev)) != cudaSuccess) {
      err = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
      return GMC_ECUDA;
    }
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (cur != dev) {
      const cudaError_t r = cudaSetDevice(cur);   // the caller's device, restored before anything is cached
      if (r != cudaSuccess) {
        err = std::string("cudaSetDevice (restoring the caller's device): ") + cudaGetErrorString(r);
        return GMC_ECUDA;
      }
    }
    if (e != cudaSuccess || !p) {
      err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return GMC_ECUDA;
    }
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return GMC_OK;
}

// A dense host array [nk][nrow][nlon] as a view.
gmc_view dense_view(double *p, int nlon, int nrow, int nk) {
  gmc_view v;
  v.data = p;
  v.lb[0] = v.lb[1] = v.lb[2] = 1;
  v.ub[0] = nlon;
  v.ub[1] = nrow;
  v.ub[2] = nk;
  return v;
}

// Host copies of a member's restart variables (FP64, dense interior).
struct HostState {
  std::vector<double> u, v, pt, phs, gz, gzs, q;
  HostState(const gmc_config &c) {
    const size_t n3 = (size_t)c.nlev * c.nlat * c.nlon, h3 = (size_t)c.nlev * (c.nlat - 1) * c.nlon,
                 n2 = (size_t)c.nlat * c.nlon;
    u.resize(n3);
    v.resize(h3);
    gzs.resize(n2);
    if (c.baroclinic) {
      pt.resize(n3);
      phs.resize(n2);
    } else {
      gz.resize(n2);
    }
    q.resize((size_t)c.ntracer * n3);
  }
  out::State view(const gmc_config &c) {
    out::State s;
    s.u = u.data();
    s.v = v.data();
    s.gzs = gzs.data();
    if (c.baroclinic) {
      s.pt = pt.data();
      s.phs = phs.data();
    } else {
      s.gz = gz.data();
    }
    const size_t n3 = (size_t)c.nlev * c.nlat * c.nlon;
    for (int l = 0; l < c.ntracer; ++l) s.q.push_back(q.data() + l * n3);
    return s;
  }
};

// The prognostic fields of a member into h.
void gather_state(EngineBase &e, const gmc_config &c, int m, HostState &h) {
  const int nlon = c.nlon, nlat = c.nlat, nlev = c.nlev;
  e.get_field(m, "u_lon", dense_view(h.u.data(), nlon, nlat, nlev));
  e.get_field(m, "v_lat", dense_view(h.v.data(), nlon, nlat - 1, nlev));
  e.get_field(m, "gzs", dense_view(h.gzs.data(), nlon, nlat, 1));
  if (c.baroclinic) {
    e.get_field(m, "pt", dense_view(h.pt.data(), nlon, nlat, nlev));
    e.get_field(m, "phs", dense_view(h.phs.data(), nlon, nlat, 1));
  } else {
    e.get_field(m, "gz", dense_view(h.gz.data(), nlon, nlat, 1));
  }
  const size_t n3 = (size_t)nlev * nlat * nlon;
  for (int l = 0; l < c.ntracer; ++l) e.get_tracer(m, l, dense_view(h.q.data() + l * n3, nlon, nlat, nlev));
}

void copy_err(char *buf, int32_t len, const std::string &msg) {
  if (!buf || len <= 0) return;
  const size_t n = std::min(msg.size(), (size_t)len - 1);
  std::memcpy(buf, msg.data(), n);
  buf[n] = 0;
}

// Waits for the context's background file write; its status (GMC_OK when
// there was none), with its message as the context's last error.
int join_background(gmc_ctx *ctx) {
  if (ctx->bg.joinable()) ctx->bg.join();
  const int rc = ctx->bg_rc;
  if (rc != GMC_OK) ctx->last_error = ctx->bg_msg;
  ctx->bg_rc = GMC_OK;
  ctx->bg_msg.clear();
  return rc;
}

// Body of a background write (a host thread): waits for the snapshot's
// copies, moves it to host FP64 arrays on a stream of its own, frees it, and
// writes the history record or restart file.
void write_snapshot(gmc_ctx *ctx, EngineBase::OutSnap o, int device, bool history, std::string path, double elapsed,
                    bool append, out::Opts opts) {
  int rc = GMC_OK;
  std::string msg;
  cudaStream_t st = nullptr;
  try {
    const gmc_config &c = ctx->cfg;
    const Grid &grid = ctx->eng->host_grid();
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CK(cudaEventSynchronize(o.ready));
    const size_t n3 = (size_t)c.nlev * c.nlat * c.nlon, h3 = (size_t)c.nlev * (c.nlat - 1) * c.nlon,
                 n2 = (size_t)c.nlat * c.nlon, ncell = c.baroclinic ? n3 : n2;
    std::vector<float> f32;
    // a field of the form's storage type, or a double array (dbl)
    auto get = [&](const void *src, size_t n, std::vector<double> &dst, bool dbl) {
      dst.resize(n);
      if (!src) return;
      if (o.fp32 && !dbl) {
        f32.resize(n);
        CK(cudaMemcpyAsync(f32.data(), src, n * sizeof(float), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (size_t k = 0; k < n; ++k) dst[k] = (double)f32[k];
      } else {
        CK(cudaMemcpyAsync(dst.data(), src, n * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
      }
    };
    HostState h(c);
    get(o.u, n3, h.u, false);
    get(o.v, h3, h.v, false);
    get(o.gzs, n2, h.gzs, true);
    if (c.baroclinic) {
      get(o.pt, n3, h.pt, false);
      get(o.phs, n2, h.phs, true);
    } else {
      get(o.gz, n2, h.gz, false);
    }
    std::vector<double> tmp;
    for (size_t l = 0; l < o.q.size(); ++l) {
      get(o.q[l], n3, tmp, false);
      std::copy(tmp.begin(), tmp.end(), h.q.begin() + (long)(l * n3));
    }
    std::vector<double> ph, t, z, div, vor, pv;
    if (history) {
      if (c.baroclinic) {
        get(o.ph, n3, ph, true);
        get(o.t, n3, t, true);
        get(o.vor, h3, vor, true);
      } else {
        get(o.pv, h3, pv, false);
      }
      get(o.z, ncell, z, true);
      get(o.div, ncell, div, true);
    }
    CK(cudaFreeAsync(o.block, st));
    o.block = nullptr;
    CK(cudaStreamSynchronize(st));
    const out::State sv = h.view(c);
    std::string e;
    if (history) {
      out::History hv;
      hv.u = sv.u;
      hv.v = sv.v;
      hv.pt = sv.pt;
      hv.phs = sv.phs;
      hv.gz = sv.gz;
      hv.gzs = sv.gzs;
      if (c.baroclinic) {
        hv.ph = ph.data();
        hv.t = t.data();
        hv.vor = vor.data();
      } else {
        hv.pv = pv.data();
      }
      hv.z = z.data();
      hv.div = div.data();
      for (double *q : sv.q) hv.q.push_back(q);
      hv.diag = o.diag;
      e = out::write_history(grid, path, elapsed, append, opts, hv);
    } else {
      e = out::write_restart(grid, path, elapsed, opts, sv);
    }
    if (!e.empty()) {
      rc = GMC_EIO;
      msg = e;
    }
  } catch (const CudaError &e) {
    rc = GMC_ECUDA;
    msg = e.msg;
  } catch (const std::bad_alloc &) {
    rc = GMC_ENOMEM;
    msg = "host allocation failed";
  }
  if (o.block) cudaFree(o.block);
  if (o.ready) cudaEventDestroy(o.ready);
  if (st) cudaStreamDestroy(st);
  ctx->bg_rc = rc;
  ctx->bg_msg = msg;
}

// Starts the background write of a member's history record or restart file.
void start_background(gmc_ctx *ctx, int member, bool history, const char *path, double elapsed, bool append,
                      const out::Opts &o) {
  EngineBase::OutSnap snap = ctx->eng->snapshot(member, history);
  try {
    ctx->bg = std::thread(write_snapshot, ctx, snap, ctx->eng->device, history, std::string(path), elapsed, append, o);
  } catch (const std::exception &e) {   // no thread: the snapshot is released here
    cudaEventSynchronize(snap.ready);
    cudaFree(snap.block);
    cudaEventDestroy(snap.ready);
    throw ApiError{GMC_EIO, std::string("cannot start the background writer: ") + e.what()};
  }
}

}  // namespace

extern "C" {

void gmc_config_default(gmc_config *c) {
  std::memset(c, 0, sizeof(*c));
  c->nlon = 360; c->nlat = 180; c->nlev = 1;
  c->baroclinic = 0;
  c->time_scheme = GMC_TIME_WRFRK3;
  c->dt_dyn = 60.0; c->dt_adv = 0.0;
  c->ke_scheme = 2; c->ke_cell_wgt = 0.5;
  c->pv_scheme = GMC_PV_UPWIND; c->upwind_order_pv = 3; c->upwind_wgt_pv = 1.0; c->pv_pole_stokes = 1;
  c->coriolis_scheme = 1;
  c->ffsl_flux_type = GMC_FLUX_PPM; c->limiter_type = GMC_LIMITER_MONO;
  c->use_div_damp = 0; c->div_damp_order = 2; c->div_damp_coef2 = 1.0 / 128.0;
  c->vert_coord_template = GMC_VCOORD_NONE;
  c->ptop = 2.194e2; c->hybrid_coord_p0 = 1.0e5;
  c->max_wave_speed = 300; c->max_cfl = 0.5;
  c->filter_coef_a = 1.0; c->filter_coef_b = 0.4; c->filter_coef_c = 0.2; c->filter_coef_d = 0.375; c->filter_coef_e = 0.16;
  c->lon_halo_width = 2;
  c->ntracer = 0;
  c->precision = GMC_PREC_FP64;
  c->n_members = 1;
  const double pi = std::atan(1.0) * 4.0;
  c->radius = 6.37122e6; c->omega = 2 * pi / 86400.0; c->g = 9.80616; c->Rd = 287.04; c->cpd = 1004.0; c->p0 = 1.0e5;
  c->tvd_limiter_type = GMC_TVD_VAN_LEER;
  c->div_damp_coef4 = 0.01;
  c->forcing = GMC_FORCING_NONE;
  c->use_smag_damp = 0;
  c->smag_damp_coef = 0.1;
}

int gmc_create(const gmc_config *cfg, gmc_ctx **out) {
  if (!cfg || !out) return GMC_EINVAL;
  *out = nullptr;
  gmc_ctx *ctx = new gmc_ctx();
  ctx->cfg = normalised(*cfg);
  int rc = guarded(ctx, [&]() {
    std::string e = validate_config(ctx->cfg);
    if (!e.empty()) throw ApiError{GMC_EINVAL, e};
    if (ctx->cfg.precision == GMC_PREC_FP64)
      ctx->eng.reset(new Engine<double>(ctx->cfg));
    else
      ctx->eng.reset(new Engine<float>(ctx->cfg));
    ctx->lon_halo_width = ctx->cfg.precision == GMC_PREC_FP64 ? static_cast<Engine<double> *>(ctx->eng.get())->grid.lon_halo_width
                                                              : static_cast<Engine<float> *>(ctx->eng.get())->grid.lon_halo_width;
    return GMC_OK;
  });
  if (rc != GMC_OK) {
    // keep the context so the caller can read the message
    *out = ctx;
    ctx->eng.reset();
    return rc;
  }
  *out = ctx;
  return GMC_OK;
}

int gmc_lon_halo_width(const gmc_ctx *ctx, int32_t *out) {
  if (!ctx || !out || !ctx->eng) return GMC_EINVAL;
  *out = ctx->lon_halo_width;
  return GMC_OK;
}

int gmc_set_field(gmc_ctx *ctx, int32_t member, const char *name, const gmc_view *v) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (!name) return fail(ctx, GMC_EINVAL, "null field name");
  if (member < 0 || member >= ctx->cfg.n_members) return fail(ctx, GMC_EINVAL, "member out of range");
  return guarded(ctx, [&]() {
    int nrow, nk;
    std::string n(name), err;
    field_dims(ctx->cfg, n, nrow, nk);
    if (!check_view(v, ctx->cfg.nlon, nrow, nk, err)) throw ApiError{GMC_EINVAL, err};
    ctx->eng->set_field(member, n, *v);
    return GMC_OK;
  });
}

int gmc_set_tracer(gmc_ctx *ctx, int32_t member, int32_t tracer, const gmc_view *v) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (member < 0 || member >= ctx->cfg.n_members) return fail(ctx, GMC_EINVAL, "member out of range");
  if (tracer < 0 || tracer >= ctx->cfg.ntracer) return fail(ctx, GMC_EINVAL, "tracer index out of range");
  return guarded(ctx, [&]() {
    std::string err;
    if (!check_view(v, ctx->cfg.nlon, ctx->cfg.nlat, ctx->cfg.nlev, err)) throw ApiError{GMC_EINVAL, err};
    ctx->eng->set_tracer(member, tracer, *v);
    return GMC_OK;
  });
}

int gmc_get_tracer(gmc_ctx *ctx, int32_t member, int32_t tracer, const gmc_view *v) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (member < 0 || member >= ctx->cfg.n_members) return fail(ctx, GMC_EINVAL, "member out of range");
  if (tracer < 0 || tracer >= ctx->cfg.ntracer) return fail(ctx, GMC_EINVAL, "tracer index out of range");
  return guarded(ctx, [&]() {
    std::string err;
    if (!check_view(v, ctx->cfg.nlon, ctx->cfg.nlat, ctx->cfg.nlev, err)) throw ApiError{GMC_EINVAL, err};
    ctx->eng->get_tracer(member, tracer, *v);
    return GMC_OK;
  });
}

int gmc_prepare(gmc_ctx *ctx) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  return guarded(ctx, [&]() {
    ctx->eng->prepare();
    return error_word_status(ctx, ctx->eng->read_error());
  });
}

int gmc_step(gmc_ctx *ctx, int32_t nsteps) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (nsteps < 0) return fail(ctx, GMC_EINVAL, "nsteps < 0");
  return guarded(ctx, [&]() {
    ctx->eng->step(nsteps);
    return error_word_status(ctx, ctx->eng->read_error());
  });
}

int gmc_step_io(gmc_ctx *ctx, int32_t member, const gmc_io *in, int32_t n_in, int32_t nsteps, const gmc_io *out,
                int32_t n_out) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (member < 0 || member >= ctx->cfg.n_members) return fail(ctx, GMC_EINVAL, "member out of range");
  if (nsteps < 0 || n_in < 0 || n_out < 0 || (n_in > 0 && !in) || (n_out > 0 && !out))
    return fail(ctx, GMC_EINVAL, "negative count or null item array");
  return guarded(ctx, [&]() {
    // every item is checked before anything moves
    auto items = [&](const gmc_io *a, int n) {
      std::vector<EngineBase::IoItem> v;
      for (int t = 0; t < n; ++t) {
        std::string err;
        int nrow = ctx->cfg.nlat, nk = ctx->cfg.nlev;
        if (a[t].name) {
          field_dims(ctx->cfg, a[t].name, nrow, nk);
        } else if (a[t].tracer < 0 || a[t].tracer >= ctx->cfg.ntracer) {
          throw ApiError{GMC_EINVAL, "tracer index out of range"};
        }
        if (!check_view(&a[t].view, ctx->cfg.nlon, nrow, nk, err)) throw ApiError{GMC_EINVAL, err};
        v.push_back({a[t].name ? std::string(a[t].name) : std::string(), a[t].name ? -1 : a[t].tracer, a[t].view});
      }
      return v;
    };
    const std::vector<EngineBase::IoItem> vin = items(in, n_in), vout = items(out, n_out);
    ctx->eng->step_io(member, vin, nsteps, vout);
    return error_word_status(ctx, ctx->eng->read_error());
  });
}

int gmc_get_field(gmc_ctx *ctx, int32_t member, const char *name, const gmc_view *v) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (!name) return fail(ctx, GMC_EINVAL, "null field name");
  if (member < 0 || member >= ctx->cfg.n_members) return fail(ctx, GMC_EINVAL, "member out of range");
  return guarded(ctx, [&]() {
    int nrow, nk;
    std::string n(name), err;
    field_dims(ctx->cfg, n, nrow, nk);
    if (!check_view(v, ctx->cfg.nlon, nrow, nk, err)) throw ApiError{GMC_EINVAL, err};
    ctx->eng->get_field(member, n, *v);
    return GMC_OK;
  });
}

int gmc_diagnose(gmc_ctx *ctx, int32_t member, gmc_diag *out) {
  if (!ctx || !out) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (member < 0 || member >= ctx->cfg.n_members) return fail(ctx, GMC_EINVAL, "member out of range");
  return guarded(ctx, [&]() {
    ctx->eng->diagnose(member, out);
    return GMC_OK;
  });
}

int gmc_time_step(const gmc_ctx *ctx, int64_t *out) {
  if (!ctx || !out || !ctx->eng) return GMC_EINVAL;
  *out = ctx->eng->time_step;
  return GMC_OK;
}

int gmc_ffsl_hflx(gmc_ctx *ctx, const gmc_ffsl_fields *f, double dt) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (!f) return fail(ctx, GMC_EINVAL, "null field set");
  return guarded(ctx, [&]() {
    ctx->eng->ffsl_hflx(*f, dt);
    return error_word_status(ctx, ctx->eng->read_error());
  });
}

int gmc_ffsl_hflx_noalloc(gmc_ctx *ctx, const gmc_ffsl_fields *f, double dt) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (!f) return fail(ctx, GMC_EINVAL, "null field set");
  const size_t need = ctx->eng->ffsl_scratch_bytes();
  if (need > kNoAllocScratchBytes)
    return fail(ctx, GMC_EINVAL, "gmc_ffsl_hflx_noalloc: grid needs " + std::to_string(need) +
                                     " scratch bytes, the fixed scratch holds " + std::to_string(kNoAllocScratchBytes) +
                                     " (2 x nlon x nlat x nlev values); use gmc_ffsl_hflx");
  return guarded(ctx, [&]() {
    void *scr = nullptr;
    std::string err;
    int rc = noalloc_scratch_address(ctx->eng->device, &scr, err);
    if (rc != GMC_OK) throw ApiError{rc, err};
    ctx->eng->ffsl_hflx_in(*f, dt, scr);
    return error_word_status(ctx, ctx->eng->read_error());
  });
}

namespace {
const char *const kTladFields[3] = {"u_lon", "v_lat", "gz"};
}

int gmc_tlm_step(gmc_ctx *ctx, int32_t nsteps, const gmc_view dx0[3], const gmc_view dxn[3]) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (!dx0 || !dxn) return fail(ctx, GMC_EINVAL, "null view array");
  if (nsteps < 0) return fail(ctx, GMC_EINVAL, "nsteps < 0");
  return guarded(ctx, [&]() {
    std::vector<double> in[3], out[3];
    const double *pin[3];
    double *pout[3];
    for (int f = 0; f < 3; ++f) {
      int nrow, nk;
      std::string err;
      field_dims(ctx->cfg, kTladFields[f], nrow, nk);
      if (!unpack_view(&dx0[f], ctx->cfg.nlon, nrow, nk, in[f], err)) throw ApiError{GMC_EINVAL, err};
      out[f].assign((size_t)ctx->cfg.nlon * nrow * nk, 0.0);
      pin[f] = in[f].data();
      pout[f] = out[f].data();
    }
    ctx->eng->tlm(nsteps, pin, pout);
    for (int f = 0; f < 3; ++f) {
      int nrow, nk;
      std::string err;
      field_dims(ctx->cfg, kTladFields[f], nrow, nk);
      if (!pack_view(&dxn[f], ctx->cfg.nlon, nrow, nk, out[f], err)) throw ApiError{GMC_EINVAL, err};
    }
    return error_word_status(ctx, ctx->eng->read_error());
  });
}

int gmc_adjoint(gmc_ctx *ctx, int32_t nsteps, int32_t ckpt_every, const gmc_view lambda_n[3], const gmc_view lambda_0[3]) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (!lambda_n || !lambda_0) return fail(ctx, GMC_EINVAL, "null view array");
  if (nsteps < 0) return fail(ctx, GMC_EINVAL, "nsteps < 0");
  if (ckpt_every < 1) return fail(ctx, GMC_EINVAL, "ckpt_every must be >= 1");
  return guarded(ctx, [&]() {
    std::vector<double> in[3], out[3];
    const double *pin[3];
    double *pout[3];
    for (int f = 0; f < 3; ++f) {
      int nrow, nk;
      std::string err;
      field_dims(ctx->cfg, kTladFields[f], nrow, nk);
      if (!unpack_view(&lambda_n[f], ctx->cfg.nlon, nrow, nk, in[f], err)) throw ApiError{GMC_EINVAL, err};
      out[f].assign((size_t)ctx->cfg.nlon * nrow * nk, 0.0);
      pin[f] = in[f].data();
      pout[f] = out[f].data();
    }
    ctx->eng->adjoint(nsteps, ckpt_every, pin, pout);
    for (int f = 0; f < 3; ++f) {
      int nrow, nk;
      std::string err;
      field_dims(ctx->cfg, kTladFields[f], nrow, nk);
      if (!pack_view(&lambda_0[f], ctx->cfg.nlon, nrow, nk, out[f], err)) throw ApiError{GMC_EINVAL, err};
    }
    return error_word_status(ctx, ctx->eng->read_error());
  });
}

int gmc_set_graphs(gmc_ctx *ctx, int32_t on) {
  if (!ctx || !ctx->eng) return GMC_EINVAL;
  ctx->eng->set_graphs(on != 0);
  return GMC_OK;
}

int gmc_host_register(void *ptr, size_t bytes) {
  if (!ptr || bytes == 0) return GMC_EINVAL;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    const uintptr_t a = (uintptr_t)ptr;
    for (const HostRange &r : g_host_ranges)
      if (a < r.base + r.bytes && r.base < a + bytes) return GMC_EINVAL;   // overlaps a registered range
  }
  if (cudaHostRegister(ptr, bytes, cudaHostRegisterMapped | cudaHostRegisterPortable) != cudaSuccess) {
    cudaGetLastError();
    return GMC_ECUDA;
  }
  void *dev = nullptr;
  if (cudaHostGetDevicePointer(&dev, ptr, 0) != cudaSuccess || !dev) {
    cudaGetLastError();
    cudaHostUnregister(ptr);
    cudaGetLastError();
    return GMC_ECUDA;
  }
  std::lock_guard<std::mutex> lk(g_host_mu);
  g_host_ranges.push_back({(uintptr_t)ptr, bytes, static_cast<char *>(dev)});
  return GMC_OK;
}

int gmc_host_unregister(void *ptr) {
  if (!ptr) return GMC_EINVAL;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    auto it = std::find_if(g_host_ranges.begin(), g_host_ranges.end(),
                           [&](const HostRange &r) { return r.base == (uintptr_t)ptr; });
    if (it == g_host_ranges.end()) return GMC_EINVAL;
    g_host_ranges.erase(it);
  }
  if (cudaHostUnregister(ptr) != cudaSuccess) {
    cudaGetLastError();
    return GMC_ECUDA;
  }
  return GMC_OK;
}

int gmc_get_stats(const gmc_ctx *ctx, gmc_stats *out) {
  if (!ctx || !out || !ctx->eng) return GMC_EINVAL;
  out->step_ms = ctx->eng->last_step_ms;
  out->steps = ctx->eng->last_steps;
  out->kernel_launches = ctx->eng->last_launches;
  out->member_layout = ctx->eng->layout_in_use();
  out->layout_tuned = ctx->eng->layout_is_tuned() ? 1 : 0;
  return GMC_OK;
}

int gmc_set_member_layout(gmc_ctx *ctx, int32_t layout) {
  if (!ctx || !ctx->eng) return GMC_EINVAL;
  if (!ctx->eng->set_layout(layout)) return fail(ctx, GMC_EINVAL, "launch layout not available for this context");
  return GMC_OK;
}

int gmc_set_profiling(gmc_ctx *ctx, int32_t on) {
  if (!ctx || !ctx->eng) return GMC_EINVAL;
  ctx->eng->prof = on != 0;
  if (on) ctx->eng->prof_table.clear();
  return GMC_OK;
}

int gmc_kernel_profile(const gmc_ctx *ctx, int32_t index, char *name, size_t name_len, double *total_ms,
                       int64_t *launches) {
  if (!ctx || !ctx->eng || index < 0 || (size_t)index >= ctx->eng->prof_table.size()) return GMC_EINVAL;
  const EngineBase::Prof &p = ctx->eng->prof_table[index];
  if (name && name_len) snprintf(name, name_len, "%s", p.name.c_str());
  if (total_ms) *total_ms = p.ms;
  if (launches) *launches = p.count;
  return GMC_OK;
}

const char *gmc_last_error(const gmc_ctx *ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

void gmc_destroy(gmc_ctx *ctx) { delete ctx; }

int gmc_output_wait(gmc_ctx *ctx) {
  if (!ctx) return GMC_EINVAL;
  return join_background(ctx);
}

int gmc_mesh_metric(const gmc_config *cfg, const char *name, double *out, size_t n) {
  if (!cfg || !name || !out) return GMC_EINVAL;
  try {
    Grid g;
    if (!g.build(normalised(*cfg)).empty()) return GMC_EINVAL;
    const RowTable *t = g.metric(name);
    if (!t) return GMC_EINVAL;
    size_t len = t->v.size() - 4;
    if (n != len) return GMC_EINVAL;
    for (size_t j = 1; j <= len; ++j) out[j - 1] = (*t)[(int)j];
    return GMC_OK;
  } catch (...) {
    return GMC_EINVAL;
  }
}

int gmc_filter_taps(const gmc_config *cfg, int32_t which, int32_t lat, int32_t *out, size_t n) {
  if (!cfg || !out || which < 0 || which > 2) return GMC_EINVAL;
  try {
    Grid g;
    if (!g.build(normalised(*cfg)).empty()) return GMC_EINVAL;
    const Filter &f = which == 0 ? g.big : which == 1 ? g.small1 : g.small2;
    const std::vector<int> &v = lat ? f.ngrid_half : f.ngrid_full;
    if (n != v.size()) return GMC_EINVAL;
    for (size_t j = 0; j < n; ++j) out[j] = v[j];
    return GMC_OK;
  } catch (...) {
    return GMC_EINVAL;
  }
}

int gmc_make_ic(const gmc_config *cfg, int32_t kind, uint64_t seed, double noise_k, double *u_lon, double *v_lat,
                double *pt_or_gz, double *phs, double *gzs, double *q) {
  if (!cfg) return GMC_EINVAL;
  try {
    Grid g;
    if (!g.build(normalised(*cfg)).empty()) return GMC_EINVAL;
    std::string e = make_ic(g, kind, seed, noise_k, u_lon, v_lat, pt_or_gz, phs, gzs, q);
    return e.empty() ? GMC_OK : GMC_EINVAL;
  } catch (...) {
    return GMC_EINVAL;
  }
}

int gmc_restart_write(gmc_ctx *ctx, int32_t member, const char *path, double elapsed_seconds,
                      const gmc_file_opts *opts) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (!path) return fail(ctx, GMC_EINVAL, "null path");
  if (member < 0 || member >= ctx->cfg.n_members) return fail(ctx, GMC_EINVAL, "member out of range");
  if (const int prev = join_background(ctx)) return prev;   // the previous background write first
  return guarded(ctx, [&]() {
    const gmc_config &c = ctx->cfg;
    out::Opts o;
    std::string e = out::parse_opts(opts, c.ntracer, o);
    if (!e.empty()) throw ApiError{GMC_EINVAL, e};
    if (opts && opts->background) {
      start_background(ctx, member, false, path, elapsed_seconds, false, o);
      return GMC_OK;
    }
    HostState h(c);
    gather_state(*ctx->eng, c, member, h);
    e = out::write_restart(ctx->eng->host_grid(), path, elapsed_seconds, o, h.view(c));
    if (!e.empty()) throw ApiError{GMC_EIO, e};
    return GMC_OK;
  });
}

int gmc_restart_read(gmc_ctx *ctx, int32_t member, const char *path, const gmc_file_opts *opts,
                     double *elapsed_seconds) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (!path) return fail(ctx, GMC_EINVAL, "null path");
  if (member < 0 || member >= ctx->cfg.n_members) return fail(ctx, GMC_EINVAL, "member out of range");
  if (const int prev = join_background(ctx)) return prev;   // the previous background write first
  return guarded(ctx, [&]() {
    const gmc_config &c = ctx->cfg;
    out::Opts o;
    std::string e = out::parse_opts(opts, c.ntracer, o);
    if (!e.empty()) throw ApiError{GMC_EINVAL, e};
    HostState h(c);
    out::State st = h.view(c);
    std::vector<bool> found;
    double t = 0;
    e = out::read_restart(ctx->eng->host_grid(), path, o, t, st, found);
    if (!e.empty()) throw ApiError{GMC_EIO, e};
    // the whole file is read before the state changes
    const int nlon = c.nlon, nlat = c.nlat, nlev = c.nlev;
    EngineBase &eng = *ctx->eng;
    eng.set_field(member, "u_lon", dense_view(h.u.data(), nlon, nlat, nlev));
    eng.set_field(member, "v_lat", dense_view(h.v.data(), nlon, nlat - 1, nlev));
    eng.set_field(member, "gzs", dense_view(h.gzs.data(), nlon, nlat, 1));
    if (c.baroclinic) {
      eng.set_field(member, "pt", dense_view(h.pt.data(), nlon, nlat, nlev));
      eng.set_field(member, "phs", dense_view(h.phs.data(), nlon, nlat, 1));
    } else {
      eng.set_field(member, "gz", dense_view(h.gz.data(), nlon, nlat, 1));
    }
    const size_t n3 = (size_t)nlev * nlat * nlon;
    for (int l = 0; l < c.ntracer; ++l)
      if (found[(size_t)l]) eng.set_tracer(member, l, dense_view(h.q.data() + l * n3, nlon, nlat, nlev));
    if (elapsed_seconds) *elapsed_seconds = t;
    return GMC_OK;
  });
}

int gmc_history_write(gmc_ctx *ctx, int32_t member, const char *path, double elapsed_seconds, int32_t append,
                      const gmc_file_opts *opts) {
  if (!ctx) return GMC_EINVAL;
  if (!ctx->eng) return fail(ctx, GMC_ESTATE, "context has no engine");
  if (!path) return fail(ctx, GMC_EINVAL, "null path");
  if (member < 0 || member >= ctx->cfg.n_members) return fail(ctx, GMC_EINVAL, "member out of range");
  if (const int prev = join_background(ctx)) return prev;   // the previous background write first
  return guarded(ctx, [&]() {
    const gmc_config &c = ctx->cfg;
    out::Opts o;
    std::string e = out::parse_opts(opts, c.ntracer, o);
    if (!e.empty()) throw ApiError{GMC_EINVAL, e};
    if (opts && opts->background) {
      start_background(ctx, member, true, path, elapsed_seconds, append != 0, o);
      return GMC_OK;
    }
    EngineBase &eng = *ctx->eng;
    HostState h(c);
    gather_state(eng, c, member, h);
    const size_t n3 = (size_t)c.nlev * c.nlat * c.nlon, h3 = (size_t)c.nlev * (c.nlat - 1) * c.nlon;
    std::vector<double> ph, t, z(n3), div(n3), vor, pv;
    if (c.baroclinic) {
      ph.resize(n3);
      t.resize(n3);
      vor.resize(h3);
    } else {
      pv.resize(h3);
      eng.get_field(member, "pv", dense_view(pv.data(), c.nlon, c.nlat - 1, 1));
    }
    eng.output_diag(member, ph.empty() ? nullptr : ph.data(), t.empty() ? nullptr : t.data(), z.data(), div.data(),
                    vor.empty() ? nullptr : vor.data());
    out::History hv;
    const out::State st = h.view(c);
    hv.u = st.u;
    hv.v = st.v;
    hv.pt = st.pt;
    hv.phs = st.phs;
    hv.gz = st.gz;
    hv.gzs = st.gzs;
    hv.ph = ph.empty() ? nullptr : ph.data();
    hv.t = t.empty() ? nullptr : t.data();
    hv.z = z.data();
    hv.div = div.data();
    hv.vor = vor.empty() ? nullptr : vor.data();
    hv.pv = pv.empty() ? nullptr : pv.data();
    for (double *q : st.q) hv.q.push_back(q);
    eng.diagnose(member, &hv.diag);
    e = out::write_history(eng.host_grid(), path, elapsed_seconds, append != 0, o, hv);
    if (!e.empty()) throw ApiError{GMC_EIO, e};
    return GMC_OK;
  });
}

namespace {
// Grid of a configuration for the host-array file calls.
int host_grid_of(const gmc_config *cfg, Grid &g, char *errbuf, int32_t errlen) {
  if (!cfg) { copy_err(errbuf, errlen, "null configuration"); return GMC_EINVAL; }
  const gmc_config c = normalised(*cfg);
  std::string e = validate_config(c);
  if (e.empty()) e = g.build(c);
  if (!e.empty()) { copy_err(errbuf, errlen, e); return GMC_EINVAL; }
  return GMC_OK;
}
out::State host_state(const gmc_config &c, const gmc_restart_arrays *a) {
  out::State s;
  s.u = a->u_lon;
  s.v = a->v_lat;
  s.pt = a->pt;
  s.phs = a->phs;
  s.gz = a->gz;
  s.gzs = a->gzs;
  const size_t n3 = (size_t)c.nlev * c.nlat * c.nlon;
  for (int l = 0; l < c.ntracer; ++l) s.q.push_back(a->q ? a->q + l * n3 : nullptr);
  return s;
}
}  // namespace

int gmc_restart_write_host(const gmc_config *cfg, const char *path, double elapsed_seconds, const gmc_file_opts *opts,
                           const gmc_restart_arrays *a, char *errbuf, int32_t errlen) {
  try {
    Grid g;
    int rc = host_grid_of(cfg, g, errbuf, errlen);
    if (rc != GMC_OK) return rc;
    if (!path || !a) { copy_err(errbuf, errlen, "null path or arrays"); return GMC_EINVAL; }
    out::Opts o;
    std::string e = out::parse_opts(opts, g.cfg.ntracer, o);
    if (!e.empty()) { copy_err(errbuf, errlen, e); return GMC_EINVAL; }
    out::State s = host_state(g.cfg, a);
    if (g.cfg.ntracer > 0 && !a->q) { copy_err(errbuf, errlen, "null tracer array"); return GMC_EINVAL; }
    e = out::write_restart(g, path, elapsed_seconds, o, s);
    if (!e.empty()) { copy_err(errbuf, errlen, e); return GMC_EIO; }
    return GMC_OK;
  } catch (const std::bad_alloc &) {
    copy_err(errbuf, errlen, "host allocation failed");
    return GMC_ENOMEM;
  }
}

int gmc_restart_read_host(const gmc_config *cfg, const char *path, const gmc_file_opts *opts,
                          double *elapsed_seconds, const gmc_restart_arrays *a, char *errbuf, int32_t errlen) {
  try {
    Grid g;
    int rc = host_grid_of(cfg, g, errbuf, errlen);
    if (rc != GMC_OK) return rc;
    if (!path || !a) { copy_err(errbuf, errlen, "null path or arrays"); return GMC_EINVAL; }
    out::Opts o;
    std::string e = out::parse_opts(opts, g.cfg.ntracer, o);
    if (!e.empty()) { copy_err(errbuf, errlen, e); return GMC_EINVAL; }
    out::State s = host_state(g.cfg, a);
    std::vector<bool> found;
    double t = 0;
    e = out::read_restart(g, path, o, t, s, found);
    if (!e.empty()) { copy_err(errbuf, errlen, e); return GMC_EIO; }
    if (elapsed_seconds) *elapsed_seconds = t;
    return GMC_OK;
  } catch (const std::bad_alloc &) {
    copy_err(errbuf, errlen, "host allocation failed");
    return GMC_ENOMEM;
  }
}

}  // extern "C"
