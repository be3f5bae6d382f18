"""The seeded synthetic initial states (gmc_make_ic) hold the properties the
benchmark workloads are described by (no GPU):

* shallow water at 1 degree: free surface 8000 m plus a sum of spherical
  harmonics of degree 1..8 whose largest excursion over the cell centres is
  100 m; a 2000 m Gaussian hill (radius 20 degrees) as topography; winds in
  geostrophic balance with the surface, tapered to zero at the equator;
* dry baroclinic at 0.5 degrees, 32 levels: a 35 sin^2(2 lat) m/s zonal jet,
  v = 0, temperatures 300 K plus N(0, 1 K) noise, a zonally uniform surface
  pressure in gradient-wind balance with the jet and an area mean of
  1000 hPa, and Gaussian-blob tracers in (0, 1];
* every state is a pure function of its seed."""
import math

import numpy as np
import pytest

import gmcore_gb300 as g
from gmcore_gb300 import abi
from oracle import Oracle

from helpers import swm_config


@pytest.fixture(scope="module")
def swm_1deg():
    cfg = swm_config(nlon=360, nlat=180, dt=60.0)
    return cfg, g.make_ic(cfg, 1, 20240601, 0.0)


@pytest.fixture(scope="module")
def baroclinic_half_degree():
    cfg = abi.default_config(nlon=720, nlat=360, nlev=32, baroclinic=1, dt_dyn=180.0,
                             vert_coord_template=abi.VCOORD_WRF_L32, time_scheme=abi.TIME_WRFRK3,
                             max_wave_speed=400.0, ntracer=4)
    return cfg, g.make_ic(cfg, 2, 20240601, 1.0)


def test_shallow_water_state(swm_1deg):
    cfg, st = swm_1deg
    h = st["gz"] / cfg.g                                           # 2-D: (nlat, nlon)
    assert abs(np.abs(h - 8000.0).max() - 100.0) < 1e-9
    hill = st["gzs"] / cfg.g
    assert 1900.0 < hill.max() <= 2000.0 and hill.min() >= 0.0
    u, v = st["u_lon"][0], st["v_lat"][0]
    assert np.all(u[0] == 0) and np.all(u[-1] == 0)
    assert 1.0 < np.abs(u).max() < 40.0 and 1.0 < np.abs(v).max() < 40.0
    # geostrophy at mid-latitudes: f u = -g dh/dy from the surface's own
    # centred difference between the neighbouring rows (1 degree apart)
    lat = g.mesh_metric(cfg, "full_lat")
    dy = cfg.radius * (lat[2:] - lat[:-2])
    mid = (np.abs(np.degrees(lat[1:-1])) > 20) & (np.abs(np.degrees(lat[1:-1])) < 70)
    f = 2 * cfg.omega * np.sin(lat[1:-1])
    taper = 1 - np.exp(-(lat[1:-1] / math.radians(5.0)) ** 2)
    hx = 0.5 * (h + np.roll(h, -1, axis=1))                        # h at the u points
    u_geo = -(cfg.g / f * taper)[:, None] * (hx[2:] - hx[:-2]) / dy[:, None]
    err = np.abs(u[1:-1][mid] - u_geo[mid]).max() / np.abs(u[1:-1][mid]).max()
    assert err < 0.02, err


def test_baroclinic_state(baroclinic_half_degree):
    cfg, st = baroclinic_half_degree
    nlat = cfg.nlat
    lat = g.mesh_metric(cfg, "full_lat")
    area = g.mesh_metric(cfg, "area_cell")
    phs = st["phs"]
    assert np.all(phs == phs[:, :1])                               # zonally uniform
    mean = np.sum(phs[:, 0] * area) / np.sum(area)
    assert abs(mean - 1.0e5) < 1e-6
    # gradient-wind balance (Rd T0 / a) dln(ps)/dlat = -(f u + u^2 tan(lat) / a)
    jet = np.array([35.0 * math.sin(2 * x) * math.sin(2 * x) for x in lat])
    a, T0 = cfg.radius, 300.0
    dlnps = (np.log(phs[2:, 0]) - np.log(phs[:-2, 0])) / (lat[2:] - lat[:-2])
    rhs = -(a / (cfg.Rd * T0)) * (2 * cfg.omega * np.sin(lat[1:-1]) * jet[1:-1] + jet[1:-1] ** 2 * np.tan(lat[1:-1]) / a)
    mid = np.abs(np.degrees(lat[1:-1])) < 80
    assert np.abs(dlnps[mid] - rhs[mid]).max() < 1e-3 * np.abs(rhs).max()
    u, v = st["u_lon"], st["v_lat"]
    assert np.array_equal(u[:, 1:-1], np.broadcast_to(jet[None, 1:-1, None], u[:, 1:-1].shape))
    assert np.all(u[:, [0, -1]] == 0) and np.all(v == 0) and np.all(st["gzs"] == 0)
    # temperatures from pt on the wrf_l32 levels
    o = Oracle(abi.default_config(nlon=36, nlat=19, nlev=32, baroclinic=1, vert_coord_template=abi.VCOORD_WRF_L32))
    try:
        hyai, hybi = o.metric("hyai", 33), o.metric("hybi", 33)
    finally:
        o.close()
    pl = np.array([hyai[k] * (cfg.hybrid_coord_p0 - cfg.ptop) + hybi[k] * (phs[:, 0] - cfg.ptop) + cfg.ptop
                   for k in range(33)])
    ph = 0.5 * (pl[:-1] + pl[1:])
    T = st["pt"] * (ph[:, :, None] / cfg.p0) ** (cfg.Rd / cfg.cpd)
    assert abs(T.mean() - 300.0) < 5e-3 and abs(T.std() - 1.0) < 5e-3
    q = st["q"]
    assert q.shape == (4, 32, nlat, cfg.nlon) and q.min() > 0.0 and q.max() <= 1.0
    assert all(q[t].max() > 0.8 for t in range(4))


def test_states_are_pure_functions_of_the_seed():
    cfg = swm_config()
    a, b, c = g.make_ic(cfg, 1, 5, 0.0), g.make_ic(cfg, 1, 5, 0.0), g.make_ic(cfg, 1, 6, 0.0)
    assert all(np.array_equal(a[k], b[k]) for k in a)
    assert not np.array_equal(a["gz"], c["gz"])
