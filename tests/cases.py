"""The reference's analytic initial states, built on the oracle's grid
(test infrastructure: the known-answer oracle runs and the GPU parity runs
start from them)."""
import math

import numpy as np

from oracle import Oracle

from gmcore_gb300 import abi
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


# Tracer transport with prescribed winds (the reference's advection tests,
# src/tests/adv/): one period T = 12 days, m = 1, mfx = u, mfy = v, u set on
# non-pole rows only; the update is the flux divergence of the FFSL face
# fluxes with the pole cells closed by ring sums of the meridional fluxes.
PERIOD = 12 * 86400.0
H0 = 1000.0


def transport_config(nlon, nlat, dt):
    return abi.default_config(nlon=nlon, nlat=nlat, nlev=1, baroclinic=0, dt_dyn=dt, dt_adv=dt,
                              limiter_type=abi.LIMITER_MONO)


class Transport:
    """One tracer-transport harness on a lat-lon grid of the oracle."""

    def __init__(self, nlon, nlat, dt):
        cfg = transport_config(nlon, nlat, dt)
        self.o = Oracle(cfg)
        self.cfg, self.dt, self.nlon, self.nlat = cfg, dt, nlon, nlat
        m = self.o.metric
        self.full_lat, self.half_lat = m("full_lat", nlat), m("half_lat", nlat - 1)
        self.de_lon, self.le_lon = m("de_lon", nlat), m("le_lon", nlat)
        self.de_lat, self.le_lat = m("de_lat", nlat - 1), m("le_lat", nlat - 1)
        self.area = m("area_cell", nlat)
        dl = 2 * math.pi / nlon
        self.full_lon = np.arange(nlon) * dl
        self.half_lon = self.full_lon + 0.5 * dl
        self.weight = np.broadcast_to(self.area[:, None], (nlat, nlon))

    def batch(self, u, v):
        """Courant numbers and axis divergences of the winds (u on lon edges,
        v on lat edges), the pole rows of u zero."""
        nlat, nlon, dt = self.nlat, self.nlon, self.dt
        u = u.copy()
        u[0], u[-1] = 0.0, 0.0
        cflx = np.zeros_like(u)
        cflx[1:-1] = u[1:-1] * dt / self.de_lon[1:-1, None]
        cfly = v * dt / self.de_lat[:, None]
        area, le_lon, le_lat = self.area, self.le_lon, self.le_lat
        divx = np.zeros((nlat, nlon))
        divy = np.zeros((nlat, nlon))
        divx[1:-1] = (u[1:-1] - np.roll(u[1:-1], 1, axis=1)) * le_lon[1:-1, None] / area[1:-1, None]
        divy[1:-1] = (v[1:] * le_lat[1:, None] - v[:-1] * le_lat[:-1, None]) / area[1:-1, None]
        divy[0] = v[0].sum() * le_lat[0] / nlon / area[0]
        divy[-1] = -v[-1].sum() * le_lat[-1] / nlon / area[-1]
        return [x[None] for x in (u, v, u, v, cflx, cfly, divx, divy)]

    def run(self, q, winds_at, steady=False, flux=None):
        """Advance the tracers q[l] over one period; winds_at(t) gives (u, v)
        at time t (called once when the winds are steady).  flux(q, wind, dt)
        returns the face fluxes (fx, fy) of one tracer; the oracle's
        ffsl_calc_tracer_hflx_cell by default."""
        flux = flux or (lambda q1, wind, dt_: self.o.ffsl_hflx(q1, *wind, dt_))
        dt, nlon = self.dt, self.nlon
        le_lon, le_lat, area = self.le_lon, self.le_lat, self.area
        wind = None
        for s in range(int(round(PERIOD / dt))):
            if wind is None or not steady:
                wind = self.batch(*winds_at((s + 0.5) * dt))
            fx, fy = zip(*(flux(q[l:l + 1], wind, dt) for l in range(len(q))))
            fx, fy = np.concatenate(fx), np.concatenate(fy)
            dx = (fx[:, 1:-1] - np.roll(fx[:, 1:-1], 1, axis=2)) * le_lon[None, 1:-1, None]
            dy = fy[:, 1:] * le_lat[None, 1:, None] - fy[:, :-1] * le_lat[None, :-1, None]
            qn = q.copy()
            qn[:, 1:-1] -= (dx + dy) / area[None, 1:-1, None] * dt
            qn[:, 0] -= (fy[:, 0].sum(axis=1) * le_lat[0] / nlon / area[0] * dt)[:, None]
            qn[:, -1] += (fy[:, -1].sum(axis=1) * le_lat[-1] / nlon / area[-1] * dt)[:, None]
            q = qn
        self.o.close()
        return q

    def l2(self, q, q0):
        d = q - q0
        return math.sqrt(np.sum(d * d * self.weight) / np.sum(q0 * q0 * self.weight))

    def mass_change(self, q, q0):
        return abs(np.sum((q - q0) * self.weight)) / np.sum(q0 * self.weight)


def distance(lon0, lat0, lon, lat):
    """Great-circle angle between (lon0, lat0) and the points (lon, lat)."""
    c = math.sin(lat0) * np.sin(lat) + math.cos(lat0) * np.cos(lat) * np.cos(lon - lon0)
    return np.arccos(np.clip(c, -1.0, 1.0))


def solid_rotation(nlon, nlat, dt, alpha=math.pi / 2, flux=None):
    tr = Transport(nlon, nlat, dt)
    u0 = 2 * math.pi * tr.cfg.radius / PERIOD
    lon_u, lat_u = np.meshgrid(tr.half_lon, tr.full_lat)
    lon_v, _ = np.meshgrid(tr.full_lon, tr.half_lat)
    u = u0 * (np.cos(lat_u) * math.cos(alpha) + np.sin(lat_u) * np.cos(lon_u) * math.sin(alpha))
    v = -u0 * np.sin(lon_v) * math.sin(alpha)
    lon_c, lat_c = np.meshgrid(tr.full_lon, tr.full_lat)
    r = distance(1.5 * math.pi, 0.0, lon_c, lat_c)
    R0 = 1.0 / 3.0
    bell0 = np.where(r < R0, H0 / 2 * (1 + np.cos(math.pi * r / R0)), 0.0)
    q0 = np.stack([bell0, np.ones_like(bell0)])
    q = tr.run(q0, lambda t: (u, v), steady=True, flux=flux)
    return tr, q, q0


def deformational_flow(nlon, nlat, dt, flux=None):
    tr = Transport(nlon, nlat, dt)
    k = 10 * tr.cfg.radius / PERIOD
    u_shape = np.sin(tr.half_lon)[None] ** 2 * np.sin(2 * tr.full_lat)[:, None]
    v_shape = np.sin(2 * tr.full_lon)[None] * np.cos(tr.half_lat)[:, None]

    def winds(t):
        c = k * math.cos(math.pi * t / PERIOD)
        return c * u_shape, c * v_shape

    lon, lat = np.meshgrid(tr.full_lon, tr.full_lat)
    centres = ((5 * math.pi / 6, 0.0), (7 * math.pi / 6, 0.0))
    x = np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)])
    gauss = np.zeros_like(lon)
    for lo, la in centres:
        xc = np.array([math.cos(la) * math.cos(lo), math.cos(la) * math.sin(lo), math.sin(la)])[:, None, None]
        gauss += 0.95 * np.exp(-5 * ((x - xc) ** 2).sum(0))
    r1, r2 = (distance(lo, la, lon, lat) for lo, la in centres)
    hill = lambda r: 0.1 + 0.9 * 0.5 * (1 + np.cos(math.pi * r / 0.5))
    cosine = np.where(r1 < 0.5, hill(r1), np.where(r2 < 0.5, hill(r2), 0.1))
    q0 = np.stack([gauss, cosine])
    q = tr.run(q0, winds, flux=flux)
    return tr, q, q0
