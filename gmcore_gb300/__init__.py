"""GB300 GMCORE dynamics step: Python host side over the C ABI.

The library (``lib/libgmcore_gpu.so``, built from ``csrc/`` for sm_103a)
replaces the reference's ``time_integrate`` (src/dynamics/gmcore_mod.F90:577)
behind the functions of ``include/gmcore_gpu.h``.  This module loads it with
ctypes and mirrors the Fortran driver's sequence: set the initial state,
``prepare`` (the run prologue, gmcore_mod.F90:97-135), ``step`` (the time
loop body) and ``diagnose`` (gmcore_mod.F90:213-341).

There is no CPU fallback: every compute call goes through the CUDA library
and fails with an exception when it is missing or has no GPU.
"""
import ctypes as C
import os
import weakref

import numpy as np

from .abi import (Config, Diag, View, Io, Stats, FfslFields, FileOpts, RestartArrays,  # noqa: F401
                  default_config, STATUS_NAMES, GMC_OK,
                  TIME_EULER, TIME_PC2, TIME_WRFRK3, PV_MIDPOINT, PV_UPWIND, PV_TVD, TVD_NONE, TVD_VAN_LEER,
                  TVD_MC, FLUX_PPM, FLUX_VAN_LEER, LIMITER_NONE,
                  LIMITER_MONO, LIMITER_PD, VCOORD_NONE, VCOORD_TEST_L26, VCOORD_WRF_L32,
                  VCOORD_WRF_L64, PREC_FP64, PREC_MIXED, FORCING_NONE, FORCING_HELD_SUAREZ)

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libgmcore_gpu.so")

EXPORTED = (
    "gmc_config_default", "gmc_create", "gmc_lon_halo_width", "gmc_set_field", "gmc_set_tracer",
    "gmc_prepare", "gmc_step", "gmc_get_field", "gmc_get_tracer", "gmc_diagnose", "gmc_time_step",
    "gmc_last_error", "gmc_destroy", "gmc_mesh_metric", "gmc_filter_taps", "gmc_make_ic",
    "gmc_get_stats", "gmc_set_profiling", "gmc_kernel_profile", "gmc_ffsl_hflx", "gmc_ffsl_hflx_noalloc",
    "gmc_tlm_step", "gmc_adjoint", "gmc_set_graphs", "gmc_host_register", "gmc_host_unregister",
    "gmc_fp64_fma_peak", "gmc_fp32_fma_peak", "gmc_set_member_layout", "gmc_step_io",
    "gmc_restart_write", "gmc_restart_read", "gmc_history_write", "gmc_restart_write_host", "gmc_restart_read_host",
    "gmc_output_wait",
)
# state fields of the tangent-linear and adjoint entry points, in ABI order
TLAD_FIELDS = ("u_lon", "v_lat", "gz")

_lib = None


class GmcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(build_if_missing=True):
    """Load the CUDA library (building it in-tree on first use)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise OSError(f"{LIB_PATH} is missing; run python -m gmcore_gb300.build")
        from .build import build
        build()
    lib = C.CDLL(LIB_PATH)
    P = C.POINTER
    lib.gmc_config_default.argtypes = [P(Config)]
    lib.gmc_config_default.restype = None
    lib.gmc_create.argtypes = [P(Config), P(C.c_void_p)]
    lib.gmc_lon_halo_width.argtypes = [C.c_void_p, P(C.c_int32)]
    lib.gmc_set_field.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, P(View)]
    lib.gmc_get_field.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, P(View)]
    lib.gmc_set_tracer.argtypes = [C.c_void_p, C.c_int32, C.c_int32, P(View)]
    lib.gmc_get_tracer.argtypes = [C.c_void_p, C.c_int32, C.c_int32, P(View)]
    lib.gmc_step_io.argtypes = [C.c_void_p, C.c_int32, P(Io), C.c_int32, C.c_int32, P(Io), C.c_int32]
    lib.gmc_prepare.argtypes = [C.c_void_p]
    lib.gmc_step.argtypes = [C.c_void_p, C.c_int32]
    lib.gmc_diagnose.argtypes = [C.c_void_p, C.c_int32, P(Diag)]
    lib.gmc_time_step.argtypes = [C.c_void_p, P(C.c_int64)]
    lib.gmc_last_error.argtypes = [C.c_void_p]
    lib.gmc_last_error.restype = C.c_char_p
    lib.gmc_destroy.argtypes = [C.c_void_p]
    lib.gmc_destroy.restype = None
    lib.gmc_mesh_metric.argtypes = [P(Config), C.c_char_p, P(C.c_double), C.c_size_t]
    lib.gmc_filter_taps.argtypes = [P(Config), C.c_int32, C.c_int32, P(C.c_int32), C.c_size_t]
    lib.gmc_make_ic.argtypes = [P(Config), C.c_int32, C.c_uint64, C.c_double] + [P(C.c_double)] * 6
    lib.gmc_get_stats.argtypes = [C.c_void_p, P(Stats)]
    lib.gmc_ffsl_hflx.argtypes = [C.c_void_p, P(FfslFields), C.c_double]
    lib.gmc_ffsl_hflx_noalloc.argtypes = [C.c_void_p, P(FfslFields), C.c_double]
    lib.gmc_set_profiling.argtypes = [C.c_void_p, C.c_int32]
    lib.gmc_tlm_step.argtypes = [C.c_void_p, C.c_int32, P(View), P(View)]
    lib.gmc_set_graphs.argtypes = [C.c_void_p, C.c_int32]
    lib.gmc_adjoint.argtypes = [C.c_void_p, C.c_int32, C.c_int32, P(View), P(View)]
    lib.gmc_kernel_profile.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_size_t, P(C.c_double), P(C.c_int64)]
    lib.gmc_host_register.argtypes = [C.c_void_p, C.c_size_t]
    lib.gmc_host_unregister.argtypes = [C.c_void_p]
    lib.gmc_fp64_fma_peak.argtypes = [P(C.c_double)]
    lib.gmc_fp32_fma_peak.argtypes = [P(C.c_double)]
    lib.gmc_set_member_layout.argtypes = [C.c_void_p, C.c_int32]
    lib.gmc_output_wait.argtypes = [C.c_void_p]
    lib.gmc_restart_write.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_double, P(FileOpts)]
    lib.gmc_restart_read.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, P(FileOpts), P(C.c_double)]
    lib.gmc_history_write.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_double, C.c_int32, P(FileOpts)]
    lib.gmc_restart_write_host.argtypes = [P(Config), C.c_char_p, C.c_double, P(FileOpts), P(RestartArrays),
                                           C.c_char_p, C.c_int32]
    lib.gmc_restart_read_host.argtypes = [P(Config), C.c_char_p, P(FileOpts), P(C.c_double), P(RestartArrays),
                                          C.c_char_p, C.c_int32]
    _lib = lib
    return lib


def fp64_fma_peak():
    """Measured FP64 FMA throughput of the current GPU in TFLOP/s."""
    out = C.c_double()
    rc = load().gmc_fp64_fma_peak(C.byref(out))
    if rc != 0:
        raise GmcError(rc, "gmc_fp64_fma_peak")
    return out.value


def fp32_fma_peak():
    """Measured FP32 FMA throughput of the current GPU in TFLOP/s."""
    out = C.c_double()
    rc = load().gmc_fp32_fma_peak(C.byref(out))
    if rc != 0:
        raise GmcError(rc, "gmc_fp32_fma_peak")
    return out.value


def page_aligned(shape):
    """Zeroed float64 array whose memory starts on a host page and shares no
    page with other arrays (so that it can be registered on its own)."""
    import mmap
    page = mmap.PAGESIZE
    n = int(np.prod(shape))
    per = page // 8
    buf = np.zeros(n + 2 * per)
    off = (-buf.ctypes.data % page) // 8
    return buf[off:off + n].reshape(shape)


def host_register(a):
    """Page-lock and map the memory of a C-contiguous array (gmc_host_register):
    transfers of fields and tracers to and from it then gather, scatter and
    convert on the GPU.  Call host_unregister(a) before the array is freed."""
    if not a.flags.c_contiguous:
        raise ValueError("host_register needs a C-contiguous array")
    rc = load().gmc_host_register(C.c_void_p(a.ctypes.data), C.c_size_t(a.nbytes))
    if rc != 0:
        raise GmcError(rc, "gmc_host_register refused the range")


def host_unregister(a):
    rc = load().gmc_host_unregister(C.c_void_p(a.ctypes.data))
    if rc != 0:
        raise GmcError(rc, "gmc_host_unregister: range not registered")


def _dptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_double))


def view_of(a, nk=None):
    """gmc_view over a C-ordered [k][j][i] (or [j][i]) float64 array whose
    Fortran index space is i = 1..ni, j = 1..nj, k = 1..nk."""
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("view needs a C-contiguous float64 array")
    v = View()
    v.data = _dptr(a)
    shape = a.shape if a.ndim == 3 else (1,) + a.shape
    v.lb[0], v.lb[1], v.lb[2] = 1, 1, 1
    v.ub[0], v.ub[1], v.ub[2] = shape[2], shape[1], shape[0]
    return v


def field_shape(cfg, name):
    nlon, nlat, nlev = cfg.nlon, cfg.nlat, cfg.nlev
    if name in ("v_lat", "v_f", "mfy_lat", "pv", "pv_lat"):
        return (nlev, nlat - 1, nlon)
    if name in ("phs", "phs_f", "gzs", "gz", "gz_f"):
        return (nlat, nlon)
    if name == "we_lev":
        return (nlev + 1, nlat, nlon)
    return (nlev, nlat, nlon)


def mesh_metric(cfg, name):
    lib = load()
    n = cfg.nlat - 1 if name.startswith("half") or name.startswith("area_lat") or name in (
        "area_vtx", "de_lat", "le_lat") else cfg.nlat
    out = np.zeros(n)
    rc = lib.gmc_mesh_metric(C.byref(cfg), name.encode(), _dptr(out), n)
    if rc:
        raise GmcError(rc, f"metric {name}")
    return out


def filter_taps(cfg, which, lat):
    lib = load()
    n = cfg.nlat - 1 if lat else cfg.nlat
    out = np.zeros(n, dtype=np.int32)
    rc = lib.gmc_filter_taps(C.byref(cfg), which, lat, out.ctypes.data_as(C.POINTER(C.c_int32)), n)
    if rc:
        raise GmcError(rc, "filter taps")
    return out


def make_ic(cfg, kind, seed, noise_k=1.0):
    """Seeded synthetic initial state (host side, no GPU).  Returns a dict of
    C-ordered float64 arrays."""
    lib = load()
    nlon, nlat, nlev = cfg.nlon, cfg.nlat, cfg.nlev
    u = np.zeros((nlev, nlat, nlon))
    v = np.zeros((nlev, nlat - 1, nlon))
    gzs = np.zeros((nlat, nlon))
    if kind == 1:
        h = np.zeros((nlat, nlon))
        rc = lib.gmc_make_ic(C.byref(cfg), 1, seed, noise_k, _dptr(u), _dptr(v), _dptr(h), None, _dptr(gzs), None)
        out = {"u_lon": u, "v_lat": v, "gz": h, "gzs": gzs}
    else:
        pt = np.zeros((nlev, nlat, nlon))
        phs = np.zeros((nlat, nlon))
        q = np.zeros((max(cfg.ntracer, 0), nlev, nlat, nlon))
        rc = lib.gmc_make_ic(C.byref(cfg), 2, seed, noise_k, _dptr(u), _dptr(v), _dptr(pt), _dptr(phs), _dptr(gzs),
                             _dptr(q) if cfg.ntracer > 0 else None)
        out = {"u_lon": u, "v_lat": v, "pt": pt, "phs": phs, "gzs": gzs}
        if cfg.ntracer > 0:
            out["q"] = q
    if rc:
        raise GmcError(rc, "make_ic")
    return out


def file_opts(time_units=None, start_time=None, tracer_names=None, restart_interval=None, background=False):
    """gmc_file_opts from keywords (None: the library's default)."""
    enc = lambda x: x.encode() if isinstance(x, str) else x
    if isinstance(tracer_names, (list, tuple)):
        tracer_names = ",".join(tracer_names)
    return FileOpts(enc(time_units), enc(start_time), enc(tracer_names), enc(restart_interval), int(background))


def _restart_arrays(cfg, state):
    """RestartArrays over the C-ordered float64 arrays of a state dict."""
    a = RestartArrays()
    for key, name in (("u_lon", "u_lon"), ("v_lat", "v_lat"), ("pt", "pt"), ("phs", "phs"), ("gz", "gz"),
                      ("gzs", "gzs"), ("q", "q")):
        x = state.get(key)
        if x is not None:
            if x.dtype != np.float64 or not x.flags.c_contiguous:
                raise ValueError(f"{key} must be a C-contiguous float64 array")
            setattr(a, name, x.ctypes.data_as(C.POINTER(C.c_double)))
    return a


def restart_write_host(cfg, path, elapsed_seconds, state, **opts):
    """Restart file of a host state (dict of dense float64 arrays as make_ic
    returns them), without a GPU."""
    lib = load()
    err = C.create_string_buffer(512)
    o = file_opts(**opts)
    rc = lib.gmc_restart_write_host(C.byref(cfg), os.fsencode(path), elapsed_seconds, C.byref(o),
                                    C.byref(_restart_arrays(cfg, state)), err, len(err))
    if rc:
        raise GmcError(rc, err.value.decode())


def restart_read_host(cfg, path, **opts):
    """(elapsed seconds, state dict) of a restart file, without a GPU."""
    lib = load()
    nlon, nlat, nlev = cfg.nlon, cfg.nlat, cfg.nlev
    st = {"u_lon": np.zeros((nlev, nlat, nlon)), "v_lat": np.zeros((nlev, nlat - 1, nlon)),
          "gzs": np.zeros((nlat, nlon))}
    if cfg.baroclinic:
        st["pt"] = np.zeros((nlev, nlat, nlon))
        st["phs"] = np.zeros((nlat, nlon))
    else:
        st["gz"] = np.zeros((nlat, nlon))
    if cfg.ntracer > 0:
        st["q"] = np.full((cfg.ntracer, nlev, nlat, nlon), np.nan)
    err = C.create_string_buffer(512)
    t = C.c_double()
    o = file_opts(**opts)
    rc = lib.gmc_restart_read_host(C.byref(cfg), os.fsencode(path), C.byref(o), C.byref(t),
                                   C.byref(_restart_arrays(cfg, st)), err, len(err))
    if rc:
        raise GmcError(rc, err.value.decode())
    return t.value, st


class Model:
    """One GPU context of the dynamics step (all ensemble members)."""

    def __init__(self, cfg):
        self.lib = load()
        self.cfg = cfg
        self._io_cache = {}
        h = C.c_void_p()
        rc = self.lib.gmc_create(C.byref(cfg), C.byref(h))
        self.h = h.value
        if rc:
            msg = self.lib.gmc_last_error(self.h).decode() if self.h else "no context"
            if self.h:
                self.lib.gmc_destroy(self.h)
                self.h = None
            raise GmcError(rc, msg)

    def _check(self, rc):
        if rc:
            raise GmcError(rc, self.lib.gmc_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.gmc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def lon_halo_width(self):
        out = C.c_int32()
        self._check(self.lib.gmc_lon_halo_width(self.h, C.byref(out)))
        return out.value

    def set_field(self, name, a, member=0):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(field_shape(self.cfg, name))
        self._check(self.lib.gmc_set_field(self.h, member, name.encode(), C.byref(view_of(a))))

    def get_field(self, name, member=0, out=None):
        """Field of the current state; written into `out` (a C-contiguous
        float64 array of the field's shape) when given."""
        if out is None:
            out = np.empty(field_shape(self.cfg, name))
        elif out.shape != field_shape(self.cfg, name):
            raise ValueError(f"out has shape {out.shape}, field {name} {field_shape(self.cfg, name)}")
        self._check(self.lib.gmc_get_field(self.h, member, name.encode(), C.byref(view_of(out))))
        return out

    def _views3(self, fields, fill=None):
        arrs = []
        for name in TLAD_FIELDS:
            if fill is None:
                a = np.ascontiguousarray(fields[name], dtype=np.float64).reshape(field_shape(self.cfg, name))
            else:
                a = np.zeros(field_shape(self.cfg, name))
            arrs.append(a)
        views = (View * 3)(*[view_of(a) for a in arrs])
        return arrs, views

    def set_graphs(self, on):
        """Replay captured CUDA graphs in step() (default) or launch directly."""
        self._check(self.lib.gmc_set_graphs(self.h, 1 if on else 0))

    def tlm_step(self, nsteps, dx0):
        """Tangent-linear model over nsteps from the prepared state:
        {u_lon, v_lat, gz} perturbation at step 0 -> perturbation at nsteps.
        The model itself advances nsteps."""
        keep_in, vin = self._views3(dx0)
        out, vout = self._views3(None, fill=True)
        self._check(self.lib.gmc_tlm_step(self.h, nsteps, vin, vout))
        return dict(zip(TLAD_FIELDS, out))

    def adjoint(self, nsteps, lam_n, ckpt_every=8):
        """Adjoint over nsteps from the prepared state: gradient of J with
        respect to {u_lon, v_lat, gz} at step nsteps -> at step 0."""
        keep_in, vin = self._views3(lam_n)
        out, vout = self._views3(None, fill=True)
        self._check(self.lib.gmc_adjoint(self.h, nsteps, ckpt_every, vin, vout))
        return dict(zip(TLAD_FIELDS, out))

    def set_tracer(self, l, q, member=0):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(self.cfg.nlev, self.cfg.nlat, self.cfg.nlon)
        self._check(self.lib.gmc_set_tracer(self.h, member, l, C.byref(view_of(q))))

    def get_tracer(self, l, member=0, out=None):
        shape = (self.cfg.nlev, self.cfg.nlat, self.cfg.nlon)
        if out is None:
            out = np.empty(shape)
        elif out.shape != shape:
            raise ValueError(f"out has shape {out.shape}, tracer {shape}")
        self._check(self.lib.gmc_get_tracer(self.h, member, l, C.byref(view_of(out))))
        return out

    def step_io(self, inputs, nsteps, outputs, member=0):
        """gmc_step_io: set `inputs`, advance nsteps, read `outputs` back into
        the given arrays.  Each item is (name, array) for a field or (l, array)
        for tracer l; arrays are C-ordered float64 of the field's shape
        (registered with host_register for the overlapped transfers)."""
        def items(seq):
            arr = (Io * max(len(seq), 1))()
            for t, (key, a) in enumerate(seq):
                if isinstance(key, str):
                    nk = 1 if a.ndim == 2 else None
                    arr[t].name = key.encode()
                    arr[t].tracer = -1
                    arr[t].view = view_of(a, nk)
                else:
                    arr[t].name = None
                    arr[t].tracer = int(key)
                    arr[t].view = view_of(a)
            return arr
        # a driver exchanges the same arrays call after call: their item
        # arrays are kept (with weak references to the arrays, so that a
        # dead array's id is never taken for a live one)
        key = (tuple((k, id(a)) for k, a in inputs), tuple((k, id(a)) for k, a in outputs))
        hit = self._io_cache.get(key)
        if hit is not None and all(r() is a for r, (_, a) in zip(hit[2], list(inputs) + list(outputs))):
            ain, aout = hit[0], hit[1]
        else:
            ain, aout = items(inputs), items(outputs)
            refs = [weakref.ref(a) for _, a in list(inputs) + list(outputs)]
            if len(self._io_cache) >= 8:
                self._io_cache.pop(next(iter(self._io_cache)))
            self._io_cache[key] = (ain, aout, refs)
        self._check(self.lib.gmc_step_io(self.h, member, ain, len(inputs), nsteps, aout, len(outputs)))
        return outputs

    def set_state(self, state, member=0):
        for name, a in state.items():
            if name == "q":
                for l in range(a.shape[0]):
                    self.set_tracer(l, a[l], member)
            else:
                self.set_field(name, a, member)

    def prepare(self):
        self._check(self.lib.gmc_prepare(self.h))

    def step(self, n=1):
        self._check(self.lib.gmc_step(self.h, n))

    def restart_write(self, path, elapsed_seconds, member=0, **opts):
        """Restart file of the state (gmc_restart_write)."""
        o = file_opts(**opts)
        self._check(self.lib.gmc_restart_write(self.h, member, os.fsencode(path), elapsed_seconds, C.byref(o)))

    def restart_read(self, path, member=0, **opts):
        """Sets the state from a restart file; returns its elapsed seconds
        (gmc_restart_read; prepare() follows)."""
        o = file_opts(**opts)
        t = C.c_double()
        self._check(self.lib.gmc_restart_read(self.h, member, os.fsencode(path), C.byref(o), C.byref(t)))
        return t.value

    def output_wait(self):
        """Waits for a background history or restart write (gmc_output_wait)."""
        self._check(self.lib.gmc_output_wait(self.h))

    def history_write(self, path, elapsed_seconds, append=False, member=0, **opts):
        """One history record of the state (gmc_history_write); background=True
        returns after a device snapshot and writes while the steps go on."""
        o = file_opts(**opts)
        self._check(self.lib.gmc_history_write(self.h, member, os.fsencode(path), elapsed_seconds, int(append),
                                               C.byref(o)))

    def diagnose(self, member=0):
        d = Diag()
        self._check(self.lib.gmc_diagnose(self.h, member, C.byref(d)))
        return d.as_dict()

    def ffsl_hflx(self, fields, dt):
        """Horizontal FFSL flux operator on device buffers.  `fields` maps the
        gmc_ffsl_fields member names to device pointers (ints)."""
        f = FfslFields(**fields)
        self._check(self.lib.gmc_ffsl_hflx(self.h, C.byref(f), dt))

    def ffsl_hflx_noalloc(self, fields, dt):
        """gmc_ffsl_hflx with the library's fixed device scratch (no allocation)."""
        f = FfslFields(**fields)
        self._check(self.lib.gmc_ffsl_hflx_noalloc(self.h, C.byref(f), dt))

    def stats(self):
        """Device time (CUDA events on the context stream) and kernel count of
        the last step() call."""
        st = Stats()
        self._check(self.lib.gmc_get_stats(self.h, C.byref(st)))
        return {"step_ms": st.step_ms, "steps": st.steps, "kernel_launches": st.kernel_launches,
                "member_layout": st.member_layout, "layout_tuned": bool(st.layout_tuned)}

    def set_member_layout(self, layout):
        """Ensemble launch layout: -1 autotune (default), 0 per-member streams,
        G > 0 member-batched launches in G groups."""
        self._check(self.lib.gmc_set_member_layout(self.h, layout))

    def set_profiling(self, on):
        self._check(self.lib.gmc_set_profiling(self.h, 1 if on else 0))

    def kernel_profile(self):
        out, i = {}, 0
        name = C.create_string_buffer(64)
        ms, n = C.c_double(), C.c_int64()
        while self.lib.gmc_kernel_profile(self.h, i, name, 64, C.byref(ms), C.byref(n)) == 0:
            out[name.value.decode()] = (ms.value, n.value)
            i += 1
        return out

    @property
    def time_step(self):
        out = C.c_int64()
        self._check(self.lib.gmc_time_step(self.h, C.byref(out)))
        return out.value
