"""Known-answer runs of the FP64 oracle on the reference's own analytic test
cases (no GPU):

* the Rossby-Haurwitz wave of wavenumber 4 in shallow water
  (src/tests/swm/rossby_haurwitz_wave_test_mod.F90:14-86): mass conserved to
  round-off, total energy to its filter dissipation, the state's mirror
  symmetry about the equator and its four-fold symmetry in longitude kept to
  round-off, the wave's amplitude kept and its pattern moving east a little
  slower than Haurwitz's non-divergent speed
  nu = (R(3+R)w - 2 Omega) / ((1+R)(2+R)) (the shallow-water form adds
  divergence, which slows a Rossby wave);
* the zonal flow over an isolated mountain
  (src/tests/swm/mountain_zonal_flow_test_mod.F90:14-80): mass and total
  energy conserved, the fluid depth staying physical;
* the baroclinic-wave state (src/tests/baroclinic_wave_test_mod.F90:15-170)
  on the 26-level test coordinate: without the perturbation (the steady state
  of src/tests/steady_state_test_mod.F90) it stays steady, zonally uniform and
  symmetric about the equator to round-off for one day; with it, the first
  day stays smooth (no grid-scale surface-pressure noise).

The baroclinic runs use the oracle's OpenMP build: the same source and
floating-point flags as the parity build (no contraction, no fast-math),
which gives the same results with several threads."""
import math

import numpy as np
import pytest

from oracle import Oracle

from helpers import baroclinic_config, initial_state, load_state, swm_config

DAY = 86400.0


def lon_axes(nlon):
    dl = 2 * math.pi / nlon
    full = np.arange(nlon) * dl
    return full, full + 0.5 * dl


def run_swm(nlon, nlat, dt, ic, days=1.0):
    cfg = swm_config(nlon=nlon, nlat=nlat, dt=dt)
    o = Oracle(cfg)
    u, v, gz, gzs = ic(o, cfg)
    o.set_field("u_lon", u[None])
    o.set_field("v_lat", v[None])
    o.set_field("gz", gz[None])
    o.set_field("gzs", gzs)
    o.prepare()
    d0 = o.diagnose()
    o.step(int(round(days * DAY / dt)))
    d1 = o.diagnose()
    out = {f: o.get_field(f)[0] for f in ("u_lon", "v_lat", "gz")}
    out["full_lat"] = o.metric("full_lat", nlat)
    o.close()
    return cfg, (u, v, gz, gzs), out, d0, d1


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


def test_rossby_haurwitz_wave_one_day():
    cfg, (u0, v0, gz0, _), s, d0, d1 = run_swm(144, 73, 300.0, rossby_haurwitz)
    assert abs(d1["tm"] - d0["tm"]) / d0["tm"] < 1e-13
    assert abs(d1["te"] - d0["te"]) / d0["te"] < 2e-5
    gz, u, v = s["gz"], s["u_lon"], s["v_lat"]
    # mirror symmetry about the equator: gz, u even, v odd
    assert np.abs(gz - gz[::-1]).max() / np.abs(gz).max() < 1e-12
    assert np.abs(u - u[::-1]).max() / np.abs(u).max() < 1e-11
    assert np.abs(v + v[::-1]).max() / np.abs(v).max() < 1e-12
    # four-fold symmetry in longitude (nlon divisible by 4)
    q = cfg.nlon // 4
    assert np.abs(gz - np.roll(gz, q, axis=1)).max() / np.abs(gz).max() < 1e-12
    assert np.abs(u - np.roll(u, q, axis=1)).max() / np.abs(u).max() < 1e-11
    # the wave-4 component at 45 N: amplitude kept, eastward drift
    j = int(np.argmin(np.abs(s["full_lat"] - math.radians(45.0))))
    f0, f1 = np.fft.rfft(gz0[j])[4], np.fft.rfft(gz[j])[4]
    assert abs(abs(f1) / abs(f0) - 1) < 0.03
    shift = -np.angle(f1 / f0) / RH_R
    nu = (RH_R * (3 + RH_R) * RH_W - 2 * cfg.omega) / ((1 + RH_R) * (2 + RH_R)) * DAY
    assert 0.8 * nu < shift < nu, (math.degrees(shift), math.degrees(nu))


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


def test_mountain_zonal_flow_one_day():
    cfg, (_, _, _, gzs), s, d0, d1 = run_swm(144, 73, 300.0, mountain_zonal_flow)
    assert abs(d1["tm"] - d0["tm"]) / d0["tm"] < 1e-13
    assert abs(d1["te"] - d0["te"]) / d0["te"] < 5e-6
    depth = (s["gz"] - gzs) / cfg.g
    assert 3000.0 < depth.min() and depth.max() < 6100.0
    assert np.all(np.isfinite(s["u_lon"])) and np.abs(s["v_lat"]).max() < 40.0


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


def run_baroclinic_wave(perturb):
    cfg = baroclinic_config(nlon=72, nlat=37, nlev=26, dt=600.0)
    st = baroclinic_wave_state(cfg, perturb)
    o = Oracle(cfg, variant="omp")
    load_state(o, st)
    o.prepare()
    d0 = o.diagnose()
    o.step(int(DAY / 600.0))
    d1 = o.diagnose()
    out = {f: o.get_field(f) for f in ("phs", "u_lon", "v_lat")}
    o.close()
    return st, out, d0, d1


@pytest.mark.parametrize("perturb", [False, True], ids=["steady_state", "perturbed"])
def test_baroclinic_wave_first_day(perturb):
    st, s, d0, d1 = run_baroclinic_wave(perturb)
    assert abs(d1["tm"] - d0["tm"]) / d0["tm"] < 5e-13
    assert abs(d1["te"] - d0["te"]) / d0["te"] < 2e-7
    ps = s["phs"]
    assert np.sqrt(np.mean((ps - 1.0e5) ** 2)) < 30.0 and np.abs(ps - 1.0e5).max() < 100.0
    if not perturb:
        # steady: zonally uniform and symmetric about the equator to round-off
        assert np.abs(ps - ps[:, :1]).max() < 1e-7
        assert np.abs(ps - ps[::-1]).max() < 1e-7
        assert np.abs(s["v_lat"]).max() < 0.5
        assert np.sqrt(np.mean((s["u_lon"] - st["u_lon"]) ** 2)) < 0.2
    else:
        # smooth: the top quarter of the zonal spectrum of ps (wavelengths
        # under 2.7 grid spacings) carries < 1 % of the largest
        # planetary-scale amplitude
        F = np.abs(np.fft.rfft(ps - ps.mean(axis=1, keepdims=True), axis=1)).max(axis=0)
        assert F[3 * len(F) // 4:].max() < 0.01 * F[1:6].max()
