"""ctypes mirror of include/gmcore_gpu.h.

The structures here are the exact C layouts of ``gmc_config``, ``gmc_diag``
and ``gmc_view``; the option constants mirror the namelist strings of the
reference (src/utils/namelist_mod.F90:10-113).
"""
import ctypes as C

GMC_OK = 0
GMC_EINVAL = -1
GMC_ECFL = -2
GMC_ENONMONO = -3
GMC_ENEGTRACER = -4
GMC_ENAN = -5
GMC_ECUDA = -7
GMC_ENOMEM = -8
GMC_ESTATE = -9
GMC_EIO = -10

STATUS_NAMES = {
    GMC_OK: "GMC_OK", GMC_EINVAL: "GMC_EINVAL", GMC_ECFL: "GMC_ECFL",
    GMC_ENONMONO: "GMC_ENONMONO", GMC_ENEGTRACER: "GMC_ENEGTRACER", GMC_ENAN: "GMC_ENAN",
    GMC_ECUDA: "GMC_ECUDA", GMC_ENOMEM: "GMC_ENOMEM",
    GMC_ESTATE: "GMC_ESTATE", GMC_EIO: "GMC_EIO",
}

TIME_EULER, TIME_PC2, TIME_WRFRK3 = 0, 1, 2
PV_MIDPOINT, PV_UPWIND, PV_TVD = 0, 1, 2
TVD_NONE, TVD_VAN_LEER, TVD_MC = 0, 1, 2
FLUX_PPM, FLUX_VAN_LEER = 0, 1
LIMITER_NONE, LIMITER_MONO, LIMITER_PD = 0, 1, 2
VCOORD_NONE, VCOORD_TEST_L26, VCOORD_WRF_L32, VCOORD_WRF_L64 = 0, 26, 32, 64
PREC_FP64, PREC_MIXED = 0, 1
FORCING_NONE, FORCING_HELD_SUAREZ = 0, 1


class Config(C.Structure):
    _fields_ = [
        ("nlon", C.c_int32), ("nlat", C.c_int32), ("nlev", C.c_int32),
        ("baroclinic", C.c_int32),
        ("time_scheme", C.c_int32),
        ("dt_dyn", C.c_double), ("dt_adv", C.c_double),
        ("ke_scheme", C.c_int32), ("ke_cell_wgt", C.c_double),
        ("pv_scheme", C.c_int32), ("upwind_order_pv", C.c_int32), ("upwind_wgt_pv", C.c_double),
        ("pv_pole_stokes", C.c_int32),
        ("coriolis_scheme", C.c_int32),
        ("ffsl_flux_type", C.c_int32), ("limiter_type", C.c_int32),
        ("use_div_damp", C.c_int32), ("div_damp_order", C.c_int32), ("div_damp_coef2", C.c_double),
        ("vert_coord_template", C.c_int32),
        ("ptop", C.c_double), ("hybrid_coord_p0", C.c_double),
        ("max_wave_speed", C.c_double), ("max_cfl", C.c_double),
        ("filter_coef_a", C.c_double), ("filter_coef_b", C.c_double), ("filter_coef_c", C.c_double),
        ("filter_coef_d", C.c_double), ("filter_coef_e", C.c_double),
        ("lon_halo_width", C.c_int32),
        ("ntracer", C.c_int32),
        ("precision", C.c_int32),
        ("n_members", C.c_int32),
        ("radius", C.c_double), ("omega", C.c_double), ("g", C.c_double), ("Rd", C.c_double),
        ("cpd", C.c_double), ("p0", C.c_double),
        ("tvd_limiter_type", C.c_int32), ("div_damp_coef4", C.c_double), ("forcing", C.c_int32),
        ("use_smag_damp", C.c_int32), ("smag_damp_coef", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Diag(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("tm", "te", "te_ke", "te_ie", "te_pe", "tav", "tpe", "tpt")]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [("step_ms", C.c_double), ("steps", C.c_int64), ("kernel_launches", C.c_int64),
                ("member_layout", C.c_int32), ("layout_tuned", C.c_int32)]


class FfslFields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("q", "u", "v", "mfx", "mfy", "cflx", "cfly", "divx", "divy", "qmfx", "qmfy")]


class View(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_double)), ("lb", C.c_int32 * 3), ("ub", C.c_int32 * 3)]


class Io(C.Structure):
    """gmc_io: a field (name) or, with name NULL, a tracer, and its view."""
    _fields_ = [("name", C.c_char_p), ("tracer", C.c_int32), ("view", View)]


class FileOpts(C.Structure):
    """gmc_file_opts: time axis, tracer names and restart attribute of the
    history and restart files (NULL members take the defaults)."""
    _fields_ = [("time_units", C.c_char_p), ("start_time", C.c_char_p), ("tracer_names", C.c_char_p),
                ("restart_interval", C.c_char_p), ("background", C.c_int32)]


class RestartArrays(C.Structure):
    """gmc_restart_arrays: dense FP64 host arrays of a restart."""
    _fields_ = [(n, C.POINTER(C.c_double)) for n in ("u_lon", "v_lat", "pt", "phs", "gz", "gzs", "q")]


def default_config(**overrides):
    """Reference namelist defaults (namelist_mod.F90:10-113) with the
    earth constants of const_mod.F90:56-66; keyword overrides win."""
    import math
    c = Config()
    c.nlon, c.nlat, c.nlev = 360, 180, 1
    c.baroclinic = 0
    c.time_scheme = TIME_WRFRK3
    c.dt_dyn, c.dt_adv = 60.0, 0.0
    c.ke_scheme, c.ke_cell_wgt = 2, 0.5
    c.pv_scheme, c.upwind_order_pv, c.upwind_wgt_pv, c.pv_pole_stokes = PV_UPWIND, 3, 1.0, 1
    c.coriolis_scheme = 1
    c.ffsl_flux_type, c.limiter_type = FLUX_PPM, LIMITER_MONO
    c.use_div_damp, c.div_damp_order, c.div_damp_coef2 = 0, 2, 1.0 / 128.0
    c.vert_coord_template = VCOORD_NONE
    c.ptop, c.hybrid_coord_p0 = 2.194e2, 1.0e5
    c.max_wave_speed, c.max_cfl = 300.0, 0.5
    c.filter_coef_a, c.filter_coef_b, c.filter_coef_c = 1.0, 0.4, 0.2
    c.filter_coef_d, c.filter_coef_e = 0.375, 0.16
    c.lon_halo_width = 2
    c.ntracer = 0
    c.precision = PREC_FP64
    c.n_members = 1
    pi = math.atan(1.0) * 4.0
    c.radius, c.omega, c.g, c.Rd, c.cpd, c.p0 = 6.37122e6, 2 * pi / 86400.0, 9.80616, 287.04, 1004.0, 1.0e5
    c.tvd_limiter_type, c.div_damp_coef4 = TVD_VAN_LEER, 0.01
    c.forcing = FORCING_NONE
    c.use_smag_damp, c.smag_damp_coef = 0, 0.1
    for k, v in overrides.items():
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    return c
