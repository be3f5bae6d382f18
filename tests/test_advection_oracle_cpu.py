"""Known-answer check of the oracle's flux-form semi-Lagrangian transport
(ffsl_calc_tracer_hflx_cell, src/dynamics/adv/ffsl_mod.F90) with the
reference's own advection test: solid-body rotation of a cosine bell over the
poles for one revolution (src/tests/adv/solid_rotation_test_mod.F90).

Parameters follow that test: period 12 days, bell height h0 = 1000 and radius
R0 = a/3 centred at (3 pi/2, 0) (solid_rotation_test_mod.F90:16-20, 43-58),
rotation axis tilted by alpha = 90 degrees, u set on non-pole rows only,
m = 1, mfx = u, mfy = v (solid_rotation_test_mod.F90:83-101), and a background
tracer q0 = 1 beside the bell (solid_rotation_test_mod.F90:38, 48).  With
m = 1 the tracer update is the flux divergence of the FFSL face fluxes, with
the pole cells closed by the ring sums of the meridional fluxes.  The norms
are those of the reference's error tool (normalised L2 against the initial
field).  The checks: the bell's total is conserved to round-off, the
monotone limiter keeps it non-negative, the background stays 1 up to the
discrete divergence of the analytic wind, and the error falls by more than
second-order-like rates from 5 to 2.5 degrees."""
import math

import numpy as np
import pytest

from gmcore_gb300 import abi
from oracle import Oracle

PERIOD = 12 * 86400.0
H0 = 1000.0


def solid_rotation(nlon, nlat, dt, alpha=math.pi / 2):
    """One revolution; returns (bell, background, bell0, cell area)."""
    cfg = abi.default_config(nlon=nlon, nlat=nlat, nlev=1, baroclinic=0, dt_dyn=dt, dt_adv=dt,
                             limiter_type=abi.LIMITER_MONO)
    o = Oracle(cfg)
    try:
        a = cfg.radius
        dlon = 2 * math.pi / nlon
        full_lat, half_lat = o.metric("full_lat", nlat), o.metric("half_lat", nlat - 1)
        de_lon, le_lon = o.metric("de_lon", nlat), o.metric("le_lon", nlat)
        de_lat, le_lat = o.metric("de_lat", nlat - 1), o.metric("le_lat", nlat - 1)
        area = o.metric("area_cell", nlat)
        full_lon = np.arange(nlon) * dlon
        half_lon = full_lon + 0.5 * dlon
        u0 = 2 * math.pi * a / PERIOD
        lon_u, lat_u = np.meshgrid(half_lon, full_lat)
        lon_v, _ = np.meshgrid(full_lon, half_lat)
        u = u0 * (np.cos(lat_u) * math.cos(alpha) + np.sin(lat_u) * np.cos(lon_u) * math.sin(alpha))
        u[0], u[-1] = 0.0, 0.0
        v = -u0 * np.sin(lon_v) * math.sin(alpha)
        cflx = np.zeros_like(u)
        cflx[1:-1] = u[1:-1] * dt / de_lon[1:-1, None]
        cfly = v * dt / de_lat[:, None]
        divx = np.zeros((nlat, nlon))
        divy = np.zeros((nlat, nlon))
        divx[1:-1] = (u[1:-1] - np.roll(u[1:-1], 1, axis=1)) * le_lon[1:-1, None] / area[1:-1, None]
        divy[1:-1] = (v[1:] * le_lat[1:, None] - v[:-1] * le_lat[:-1, None]) / area[1:-1, None]
        divy[0] = v[0].sum() * le_lat[0] / nlon / area[0]
        divy[-1] = -v[-1].sum() * le_lat[-1] / nlon / area[-1]

        lon_c, lat_c = np.meshgrid(full_lon, full_lat)
        cosr = np.sin(lat_c) * math.sin(0.0) + np.cos(lat_c) * math.cos(0.0) * np.cos(lon_c - 1.5 * math.pi)
        r = a * np.arccos(np.clip(cosr, -1.0, 1.0))
        R0 = a / 3
        bell0 = np.where(r < R0, H0 / 2 * (1 + np.cos(math.pi * r / R0)), 0.0)
        q = np.stack([bell0, np.ones_like(bell0)])
        wind = [x[None] for x in (u, v, u, v, cflx, cfly, divx, divy)]
        for _ in range(int(round(PERIOD / dt))):
            fx, fy = zip(*(o.ffsl_hflx(q[l:l + 1], *wind, dt) for l in range(2)))
            fx, fy = np.concatenate(fx), np.concatenate(fy)
            dx = (fx[:, 1:-1] - np.roll(fx[:, 1:-1], 1, axis=2)) * le_lon[None, 1:-1, None]
            dy = fy[:, 1:] * le_lat[None, 1:, None] - fy[:, :-1] * le_lat[None, :-1, None]
            qn = q.copy()
            qn[:, 1:-1] -= (dx + dy) / area[None, 1:-1, None] * dt
            qn[:, 0] -= (fy[:, 0].sum(axis=1) * le_lat[0] / nlon / area[0] * dt)[:, None]
            qn[:, -1] += (fy[:, -1].sum(axis=1) * le_lat[-1] / nlon / area[-1] * dt)[:, None]
            q = qn
    finally:
        o.close()
    return q[0], q[1], bell0, np.broadcast_to(area[:, None], bell0.shape)


def l2_error(q, q0, w):
    d = q - q0
    return math.sqrt(np.sum(d * d * w) / np.sum(q0 * q0 * w))


@pytest.fixture(scope="module")
def runs():
    return {res: solid_rotation(*args) for res, args in ((5.0, (72, 37, 3600.0)), (2.5, (144, 73, 1800.0)))}


@pytest.mark.parametrize("res", [5.0, 2.5])
def test_solid_rotation_conserves_and_stays_monotone(runs, res):
    bell, background, bell0, w = runs[res]
    m0, m1 = np.sum(bell0 * w), np.sum(bell * w)
    assert abs(m1 - m0) / m0 < 1e-12
    assert bell.min() > -1e-10 * H0
    assert bell.max() <= H0 * (1 + 1e-12)
    assert np.abs(background - 1).max() < 1e-3


def test_solid_rotation_error_converges(runs):
    e5 = l2_error(*[runs[5.0][i] for i in (0, 2, 3)])
    e25 = l2_error(*[runs[2.5][i] for i in (0, 2, 3)])
    assert e25 < 0.1
    assert e25 < 0.35 * e5
