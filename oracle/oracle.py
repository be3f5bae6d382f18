"""ORACLE -- test infrastructure only.

ctypes wrapper of the FP64 CPU restatement in gmcore_oracle.cpp.  Only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
load it; the product library never does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from gmcore_gb300.abi import Config

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}


def build(variant="parity", quiet=True):
    """Compile the oracle with its Makefile (seconds)."""
    target = "_build/liboracle.so" if variant == "parity" else "_build/liboracle_omp.so"
    out = subprocess.run(["make", "-s", target], cwd=HERE, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(HERE, target)


def load(variant="parity"):
    if variant in _LIBS:
        return _LIBS[variant]
    path = build(variant)
    lib = C.CDLL(path)
    lib.orc_create.restype = C.c_void_p
    lib.orc_create.argtypes = [C.POINTER(Config), C.c_char_p, C.c_int]
    lib.orc_destroy.argtypes = [C.c_void_p]
    lib.orc_lon_halo_width.argtypes = [C.c_void_p]
    for name in ("orc_set_field", "orc_get_field"):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double)]
    for name in ("orc_set_tracer", "orc_get_tracer"):
        getattr(lib, name).argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    lib.orc_prepare.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
    lib.orc_step.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_int]
    lib.orc_diagnose.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    lib.orc_output_diag.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 5
    lib.orc_space_identities.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    lib.orc_metric.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double), C.c_int]
    lib.orc_filter_taps.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int)]
    lib.orc_filter_weights.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_int]
    lib.orc_run_pass.argtypes = [C.c_void_p, C.c_int]
    lib.orc_get_tend.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.POINTER(C.c_double)]
    lib.orc_get_batch.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double)]
    lib.orc_get_tracer_batch.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double)]
    lib.orc_get_tracer_level.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double)]
    lib.orc_tracer_piece.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.orc_ffsl_hflx.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 9 + [C.c_double] + [C.POINTER(C.c_double)] * 2
    lib.orc_make_ic.argtypes = [C.POINTER(Config), C.c_int, C.c_uint64, C.c_double] + [C.POINTER(C.c_double)] * 6
    _LIBS[variant] = lib
    return lib


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_ic(cfg, kind, seed, noise_k=1.0, variant="parity"):
    """The seeded synthetic initial state from the oracle's own build (the
    same generator as the library's gmc_make_ic): a dict of C-ordered float64
    arrays u_lon, v_lat, gz | (pt, phs), gzs and, with tracers, q."""
    lib = load(variant)
    nlon, nlat, nlev = cfg.nlon, cfg.nlat, cfg.nlev
    u = np.zeros((nlev, nlat, nlon))
    v = np.zeros((nlev, nlat - 1, nlon))
    gzs = np.zeros((nlat, nlon))
    if kind == 1:
        h = np.zeros((nlat, nlon))
        rc = lib.orc_make_ic(C.byref(cfg), 1, seed, noise_k, _ptr(u), _ptr(v), _ptr(h), None, _ptr(gzs), None)
        out = {"u_lon": u, "v_lat": v, "gz": h, "gzs": gzs}
    else:
        pt = np.zeros((nlev, nlat, nlon))
        phs = np.zeros((nlat, nlon))
        q = np.zeros((max(cfg.ntracer, 0), nlev, nlat, nlon))
        rc = lib.orc_make_ic(C.byref(cfg), 2, seed, noise_k, _ptr(u), _ptr(v), _ptr(pt), _ptr(phs), _ptr(gzs),
                             _ptr(q) if cfg.ntracer > 0 else None)
        out = {"u_lon": u, "v_lat": v, "pt": pt, "phs": phs, "gzs": gzs}
        if cfg.ntracer > 0:
            out["q"] = q
    if rc:
        raise ValueError(f"orc_make_ic failed ({rc})")
    return out


FIELD_SHAPES = {
    # name: (lat kind, lev kind)  lat: 0 full, 1 half; lev: 0 full, 1 half-levels, 2 two-d
    "u_lon": (0, 0), "v_lat": (1, 0), "u_f": (0, 0), "v_f": (1, 0), "pt": (0, 0), "gz": (0, 0),
    "gz_f": (0, 0), "phs": (0, 2), "phs_f": (0, 2), "gzs": (0, 2), "m": (0, 0), "t": (0, 0),
    "pv": (1, 0), "ke": (0, 0), "pv_lon": (0, 0), "pv_lat": (1, 0), "mfx_lon": (0, 0),
    "mfy_lat": (1, 0), "u_lat": (1, 0), "v_lon": (0, 0), "we_lev": (0, 1), "m_lev": (0, 1),
    "gz_lev": (0, 1), "ph_lev": (0, 1), "ph_exn_lev": (0, 1), "vor": (1, 0),
}


def field_shape(cfg, name):
    lat, lev = FIELD_SHAPES[name]
    nrow = cfg.nlat - 1 if lat else cfg.nlat
    if lev == 2:
        return (nrow, cfg.nlon)
    nk = cfg.nlev + 1 if lev == 1 else cfg.nlev
    return (nk, nrow, cfg.nlon)


class Oracle:
    """One model instance of the restatement (one ensemble member)."""

    def __init__(self, cfg, variant="parity"):
        self.lib = load(variant)
        self.cfg = cfg
        err = C.create_string_buffer(512)
        self.h = self.lib.orc_create(C.byref(cfg), err, 512)
        if not self.h:
            raise ValueError(err.value.decode())

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @property
    def lon_halo_width(self):
        return self.lib.orc_lon_halo_width(self.h)

    def set_field(self, name, a):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(field_shape(self.cfg, name))
        rc = self.lib.orc_set_field(self.h, name.encode(), _ptr(a))
        if rc:
            raise KeyError(name)

    def get_field(self, name):
        out = np.empty(field_shape(self.cfg, name))
        rc = self.lib.orc_get_field(self.h, name.encode(), _ptr(out))
        if rc:
            raise KeyError(name)
        return out

    def set_tracer(self, l, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(self.cfg.nlev, self.cfg.nlat, self.cfg.nlon)
        if self.lib.orc_set_tracer(self.h, l, _ptr(q)):
            raise IndexError(l)

    def get_tracer(self, l):
        out = np.empty((self.cfg.nlev, self.cfg.nlat, self.cfg.nlon))
        if self.lib.orc_get_tracer(self.h, l, _ptr(out)):
            raise IndexError(l)
        return out

    def prepare(self):
        err = C.create_string_buffer(512)
        rc = self.lib.orc_prepare(self.h, err, 512)
        if rc:
            raise RuntimeError(f"oracle prepare failed ({rc}): {err.value.decode()}")

    def step(self, n=1):
        err = C.create_string_buffer(512)
        rc = self.lib.orc_step(self.h, n, err, 512)
        if rc:
            raise RuntimeError(f"oracle step failed ({rc}): {err.value.decode()}")

    def diagnose(self):
        out = np.zeros(8)
        self.lib.orc_diagnose(self.h, _ptr(out))
        return dict(zip(("tm", "te", "te_ke", "te_ie", "te_pe", "tav", "tpe", "tpt"), out))

    def output_diag(self):
        """History diagnostics of the current state: {ph, t, z, div, vor}
        (shallow water: {z, div, vor})."""
        c = self.cfg
        cell = np.zeros((c.nlev, c.nlat, c.nlon))
        out = {"z": cell.copy(), "div": cell.copy(), "vor": np.zeros((c.nlev, c.nlat - 1, c.nlon))}
        if c.baroclinic:
            out["ph"], out["t"] = cell.copy(), cell.copy()
        p = lambda k: _ptr(out[k]) if k in out else None
        self.lib.orc_output_diag(self.h, p("ph"), p("t"), p("z"), p("div"), p("vor"))
        return out

    def space_identities(self):
        """Inner products of debug_check_space_operators at state(old)
        (call after prepare): {name: (sum, sum of |terms|)} per 4 pi r^2."""
        out = np.zeros(8)
        self.lib.orc_space_identities(self.h, _ptr(out))
        return {"coriolis": (out[0], out[1]), "ke": (out[2], out[3]), "mass": (out[4], out[5]), "ptf": (out[6], out[7])}

    def metric(self, name, n):
        out = np.zeros(n)
        if self.lib.orc_metric(self.h, name.encode(), _ptr(out), n):
            raise KeyError(name)
        return out

    def filter_taps(self, which, lat):
        n = self.cfg.nlat - 1 if lat else self.cfg.nlat
        out = np.zeros(n, dtype=np.int32)
        self.lib.orc_filter_taps(self.h, which, lat, out.ctypes.data_as(C.POINTER(C.c_int)))
        return out

    def run_pass(self, which):
        """One space-operator pass on state(old): 0 forward, 1 backward
        (prepare and pressure-gradient force)."""
        rc = self.lib.orc_run_pass(self.h, which)
        if rc:
            raise RuntimeError(f"oracle pass {which} failed ({rc})")

    TEND_HALF = {"dv", "qhu", "dkedlat", "pgf_lat", "wedvdlev"}

    def get_tend(self, which, name):
        """A tendency of the last run_pass(which), [k][j][i] ([j][i] for dphs)."""
        c = self.cfg
        nrow = c.nlat - 1 if name in self.TEND_HALF else c.nlat
        shape = (nrow, c.nlon) if name == "dphs" else (c.nlev, nrow, c.nlon)
        out = np.zeros(shape)
        if self.lib.orc_get_tend(self.h, which, name.encode(), _ptr(out)):
            raise KeyError(name)
        return out

    def _batch(self, fn, name):
        c = self.cfg
        nrow = c.nlat - 1 if name in ("v", "cfly", "mfy") else c.nlat
        nk = c.nlev + 1 if name in ("we", "m_lev", "cflz") else c.nlev
        out = np.zeros((nk, nrow, c.nlon))
        if fn(self.h, name.encode(), _ptr(out)):
            raise KeyError(name)
        return out

    def get_batch(self, name):
        """A field of the dynamic mass batch (u, v, mfx, mfy, cflx, cfly, divx,
        divy, qx, qy, old_m; on half levels we, m_lev, cflz)."""
        return self._batch(self.lib.orc_get_batch, name)

    def get_tracer_batch(self, name):
        """The same fields of the static tracer batch."""
        return self._batch(self.lib.orc_get_tracer_batch, name)

    def get_tracer_level(self, l, lev):
        """Tracer l of the batch's old (lev 0) or new (lev 1) time level with
        two longitude-halo columns each side, [k][j][nlon + 4] from i = -1."""
        c = self.cfg
        out = np.zeros((c.nlev, c.nlat, c.nlon + 4))
        if self.lib.orc_get_tracer_level(self.h, l, lev, _ptr(out)):
            raise KeyError((l, lev))
        return out

    def tracer_piece(self, which, q, m):
        """One tracer-step piece on cell field q with layer masses m: 0 the
        zonal negative fixer, 1 the vertical one, 2 three passes of the
        zonal smoother.  Returns (q after, status)."""
        qa = np.ascontiguousarray(q, dtype=np.float64).copy()
        ma = np.ascontiguousarray(m, dtype=np.float64)
        rc = self.lib.orc_tracer_piece(self.h, which, _ptr(qa), _ptr(ma))
        return qa, rc

    def filter_weights(self, which, lat, j):
        """Weights of polar-filter row j (1-based) of filter `which`
        (0 big, 1 small1, 2 small2) on full (lat=0) or half (lat=1) rows."""
        n = int(self.filter_taps(which, lat)[j - 1])
        out = np.zeros(n)
        if self.lib.orc_filter_weights(self.h, which, lat, j, _ptr(out), n):
            raise IndexError((which, lat, j))
        return out

    def ffsl_hflx(self, q, u, v, mfx, mfy, cflx, cfly, divx, divy, dt):
        """ffsl_calc_tracer_hflx_cell on interior arrays; returns (qmfx, qmfy)."""
        c = self.cfg
        full = (c.nlev, c.nlat, c.nlon)
        half = (c.nlev, c.nlat - 1, c.nlon)
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (q, u, v, mfx, mfy, cflx, cfly, divx, divy)]
        fx, fy = np.zeros(full), np.zeros(half)
        rc = self.lib.orc_ffsl_hflx(self.h, *[_ptr(a) for a in arrs], dt, _ptr(fx), _ptr(fy))
        if rc:
            raise RuntimeError(f"oracle ffsl_hflx failed ({rc})")
        return fx, fy
