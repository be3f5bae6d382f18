"""The reference's analytic initial states, built on the oracle's grid
(test infrastructure: the known-answer oracle runs and the GPU parity runs
start from them)."""
import math

import numpy as np

from oracle import Oracle

from helpers import initial_state, load_state


def lon_axes(nlon):
    dl = 2 * math.pi / nlon
    full = np.arange(nlon) * dl
    return full, full + 0.5 * dl


# Rossby-Haurwitz wave, R = 4, w = 7.848e-6 1/s, gz0 = 8000 m g
# (rossby_haurwitz_wave_test_mod.F90:14-15, 38, 46-84).
RH_R, RH_W = 4.0, 7.848e-6


def rossby_haurwitz(o, cfg):
    nlon, nlat = cfg.nlon, cfg.nlat
    a, Om, R, w = cfg.radius, cfg.omega, RH_R, RH_W
    flon, hlon = lon_axes(nlon)
    fc, fs = o.metric("full_cos_lat", nlat)[:, None], o.metric("full_sin_lat", nlat)[:, None]
    hc, hs = o.metric("half_cos_lat", nlat - 1)[:, None], o.metric("half_sin_lat", nlat - 1)[:, None]
    u = a * w * (fc + R * fc ** (R - 1) * fs ** 2 * np.cos(R * hlon) - fc ** (R + 1) * np.cos(R * hlon))
    v = -a * w * R * hc ** (R - 1) * hs * np.sin(R * flon)
    A = 0.5 * w * (2 * Om + w) * fc ** 2 + 0.25 * w ** 2 * (
        (R + 1) * fc ** (2 * R + 2) + (2 * R ** 2 - R - 2) * fc ** (2 * R) - 2 * R ** 2 * fc ** (2 * R - 2))
    B = 2 * (Om + w) * w * fc ** R * (R ** 2 + 2 * R + 2 - (R + 1) ** 2 * fc ** 2) / (R + 1) / (R + 2)
    Cc = 0.25 * w ** 2 * fc ** (2 * R) * ((R + 1) * fc ** 2 - R - 2)
    gz = 8.0e3 * cfg.g + a ** 2 * (A + B * np.cos(R * flon) + Cc * np.cos(2 * R * flon))
    return u, v, gz, np.zeros((nlat, nlon))


# Zonal flow over a conical mountain: u0 = 20 m/s, gz0 = 5960 m g, mountain
# 2000 m high, radius pi/9, centred at (3 pi/2, pi/6)
# (mountain_zonal_flow_test_mod.F90:14-20, 32-77).
def mountain_zonal_flow(o, cfg):
    nlon, nlat = cfg.nlon, cfg.nlat
    a, Om, g = cfg.radius, cfg.omega, cfg.g
    u0, lon0, lat0, R = 20.0, 1.5 * math.pi, math.pi / 6, math.pi / 9
    flon, _ = lon_axes(nlon)
    flat = o.metric("full_lat", nlat)[:, None]
    fc, fs = o.metric("full_cos_lat", nlat)[:, None], o.metric("full_sin_lat", nlat)[:, None]
    dlon = np.abs(flon - lon0)
    dlon = np.minimum(dlon, 2 * math.pi - dlon)
    d = np.minimum(R, np.sqrt(dlon ** 2 + (flat - lat0) ** 2))
    gzs = 2000.0 * g * (1 - d / R)
    u = u0 * fc * np.ones(nlon)
    gz = 5960.0 * g - (a * Om * u0 + 0.5 * u0 ** 2) * fs ** 2 * np.ones(nlon)
    return u, np.zeros((nlat - 1, nlon)), gz, gzs


# Baroclinic wave: u0 = 35 m/s, T0 = 288 K, lapse rate 0.005 K/m,
# dT = 4.8e5 K, eta0 = 0.252, eta_t = 0.2, perturbation of 1 m/s centred at
# (pi/9, 2 pi/9) (baroclinic_wave_test_mod.F90:15-24, 46-167).
JW_U0, JW_T0, JW_GAMMA, JW_DT, JW_ETA0, JW_ETAT = 35.0, 288.0, 0.005, 4.8e5, 0.252, 0.2


def baroclinic_wave_state(cfg, perturb):
    nlon, nlat, nlev = cfg.nlon, cfg.nlat, cfg.nlev
    a, Om, g, Rd = cfg.radius, cfg.omega, cfg.g, cfg.Rd
    st = initial_state(cfg, noise_k=0.0)
    st["phs"][:] = 1.0e5
    o = Oracle(cfg)
    load_state(o, st)
    o.prepare()           # full-level pressure of phs = 1000 hPa
    pl = o.get_field("ph_lev")
    ph = 0.5 * (pl[:-1] + pl[1:])
    eta = o.metric("full_lev", nlev)[:, None, None]
    flat = o.metric("full_lat", nlat)[:, None]
    fc, fs = o.metric("full_cos_lat", nlat)[:, None], o.metric("full_sin_lat", nlat)[:, None]
    o.close()
    _, hlon = lon_axes(nlon)
    etav = (eta - JW_ETA0) * math.pi / 2
    u = JW_U0 * np.cos(etav) ** 1.5 * np.sin(2 * flat) ** 2 * np.ones(nlon)
    if perturb:
        lonc, latc = math.pi / 9, 2 * math.pi / 9
        r = 10.0 * np.arccos(np.clip(math.sin(latc) * fs + math.cos(latc) * fc * np.cos(hlon - lonc), -1, 1))
        u = u + np.where(r ** 2 <= 50, np.exp(-r ** 2), 0.0)
    tbar = JW_T0 * eta ** (Rd * JW_GAMMA / g) + np.where(eta < JW_ETAT, JW_DT * (JW_ETAT - eta) ** 5, 0.0)
    merid = lambda ev: ((-2 * fs ** 6 * (fc ** 2 + 1 / 3) + 10 / 63) * 2 * JW_U0 * np.cos(ev) ** 1.5
                        + (1.6 * fc ** 3 * (fs ** 2 + 2 / 3) - math.pi / 4) * a * Om)
    t = tbar + 0.75 * eta * math.pi * JW_U0 / Rd * np.sin(etav) * np.sqrt(np.cos(etav)) * merid(etav)
    ev1 = (1 - JW_ETA0) * math.pi / 2
    gzs = JW_U0 * math.cos(ev1) ** 1.5 * (
        (-2 * fs ** 6 * (fc ** 2 + 1 / 3) + 10 / 63) * JW_U0 * math.cos(ev1) ** 1.5
        + (1.6 * fc ** 3 * (fs ** 2 + 2 / 3) - math.pi / 4) * a * Om)
    st.update(u_lon=u, v_lat=np.zeros_like(st["v_lat"]), pt=t * (1.0e5 / ph) ** (Rd / cfg.cpd),
              gzs=gzs * np.ones(nlon))
    return st


def swm_state(cfg, ic):
    """A shallow-water case as a state dict for load_state (3-D fields with
    their one level)."""
    o = Oracle(cfg)
    u, v, gz, gzs = ic(o, cfg)
    o.close()
    return {"u_lon": u[None], "v_lat": v[None], "gz": gz[None], "gzs": gzs}
