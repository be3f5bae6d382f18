"""States that make the step fail, injected on the host (no device fault):
each is a seeded baroclinic state with one defect set through the same
set_field call a host model would make.  The reference stops at these with
log_error / process_stop; the oracle and the library return a status code.

  nonmono: one equatorial column's surface pressure below the model top, so
           the bottom layer masses of calc_m are negative
           (operators_mod.F90:489-500)                         -> GMC_ENONMONO
  cflx:    a zonal wind band whose Courant number exceeds the longitude
           halo width (adv_batch_mod.F90:284-287)               -> GMC_ECFL
  nan:     one non-finite wind value                           -> GMC_ENAN
  negtracer: a tracer row that is negative everywhere, which the zonal
           fixer cannot fill (adv_mod.F90:236-258)              -> GMC_ENEGTRACER
"""
import numpy as np

from helpers import baroclinic_config, initial_state


def config(**kw):
    kw.setdefault("ntracer", 0)
    return baroclinic_config(nlon=72, nlat=37, nlev=26, dt=120.0, **kw)


def low_column(state, cfg):
    """Surface pressure of one equatorial column set to 10 Pa."""
    s = {k: v.copy() for k, v in state.items()}
    s["phs"][cfg.nlat // 2, cfg.nlon // 3] = 10.0
    return s


def fast_band(state, cfg, hx):
    """Zonal wind of the equatorial row at a Courant number of hx + 3."""
    s = {k: v.copy() for k, v in state.items()}
    radius, dlon = cfg.radius, 2 * np.pi / cfg.nlon
    j = cfg.nlat // 2
    lat = -0.5 * np.pi + j * np.pi / (cfg.nlat - 1)
    dx = radius * np.cos(lat) * dlon
    s["u_lon"][:, j, :] = (hx + 3) * dx / cfg.dt_dyn
    return s


def negative_row(state, cfg, tracer=0):
    """Tracer `tracer` negative along a whole mid-latitude row at every level."""
    s = {k: v.copy() for k, v in state.items()}
    s["q"][tracer, :, cfg.nlat // 3, :] = -1.0
    return s


def base_state(cfg, seed=5):
    return initial_state(cfg, seed=seed, noise_k=1.0)
