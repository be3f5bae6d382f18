"""The oracle's diagnosis of a state for history records (output_state /
orc_output_diag: calc_ph, calc_t, calc_gz_lev, calc_vor with the polar Stokes
rings, calc_div; operators_mod.F90:136-190, 354-431, 433-469, 585-680) against
a numpy restatement of the same formulas in the same operation order, on the
state after two steps of the 5-degree baroclinic case: div, vor and ph bit for
bit, t and z (libm pow and log on both sides) within 2 ulp-scale relative
error.  Rings are summed in the reference's order (zonal_sum: i = 1..nlon)."""
import numpy as np

import gmcore_gb300 as g
from gmcore_gb300 import abi
from oracle import Oracle

from helpers import load_state


def config():
    return abi.default_config(nlon=72, nlat=37, nlev=26, baroclinic=1, dt_dyn=600.0,
                              vert_coord_template=abi.VCOORD_TEST_L26, time_scheme=abi.TIME_WRFRK3,
                              max_wave_speed=400.0)


def ring(a):
    """Sum over longitude in order (the last axis), as zonal_sum does."""
    return np.cumsum(a, axis=-1)[..., -1]


east = lambda a: np.roll(a, -1, axis=-1)
west = lambda a: np.roll(a, 1, axis=-1)


def test_history_diagnostics_equal_restatement():
    cfg = config()
    o = Oracle(cfg)
    load_state(o, g.make_ic(cfg, 2, 17, 1.0))
    o.prepare()
    o.step(2)
    got = o.output_diag()
    nlon, nlat, nlev = cfg.nlon, cfg.nlat, cfg.nlev
    nh = nlat - 1
    u, v, pt = o.get_field("u_f"), o.get_field("v_f"), o.get_field("pt")
    m, ph_lev, gzs = o.get_field("m"), o.get_field("ph_lev"), o.get_field("gzs")
    full = {n: o.metric(n, nlat) for n in ("le_lon", "de_lon", "area_cell")}
    half = {n: o.metric(n, nh) for n in ("le_lat", "de_lat", "area_vtx", "half_tangent_wgt1", "half_tangent_wgt2")}
    o.close()

    # calc_div: interior rows, then the pole rings of v
    div = np.zeros((nlev, nlat, nlon))
    lel, ll, ac = full["le_lon"], half["le_lat"], full["area_cell"]
    for jj in range(1, nlat - 1):
        div[:, jj] = ((u[:, jj] * lel[jj] - west(u[:, jj]) * lel[jj]) +
                      (v[:, jj] * ll[jj] - v[:, jj - 1] * ll[jj - 1])) / ac[jj]
    div[:, 0] = (ring(v[:, 0]) * ll[0] / nlon / ac[0])[:, None]
    div[:, -1] = (ring(-v[:, -1]) * ll[-1] / nlon / ac[-1])[:, None]
    assert np.array_equal(got["div"], div)

    # calc_vor: interior half rows, then the polar rings of u_lat = mfx_lat / m_lat
    vor = np.zeros((nlev, nh, nlon))
    dl, dla, av = full["de_lon"], half["de_lat"], half["area_vtx"]
    for hh in range(nh):
        vor[:, hh] = (u[:, hh] * dl[hh] - u[:, hh + 1] * dl[hh + 1] + east(v[:, hh]) * dla[hh] -
                      v[:, hh] * dla[hh]) / av[hh]
    mfx = (m + east(m)) * 0.5 * u
    mfx[:, 0] = 0.0   # no zonal mass flux on the pole rows
    mfx[:, -1] = 0.0
    w1, w2 = half["half_tangent_wgt1"], half["half_tangent_wgt2"]

    def u_lat(hh):
        mf = w1[hh] * (west(mfx[:, hh]) + mfx[:, hh]) + w2[hh] * (west(mfx[:, hh + 1]) + mfx[:, hh + 1])
        return mf / ((m[:, hh] + m[:, hh + 1]) * 0.5)

    vor[:, 0] = (ring(-u_lat(0) * ll[0]) / nlon / ac[0])[:, None]
    vor[:, -1] = (ring(u_lat(nh - 1) * ll[nh - 1]) / nlon / ac[nh])[:, None]
    assert np.array_equal(got["vor"], vor)

    # calc_ph, calc_t
    ph = 0.5 * (ph_lev[:-1] + ph_lev[1:])
    assert np.array_equal(got["ph"], ph)
    t = pt * np.power(ph / cfg.p0, cfg.Rd / cfg.cpd)
    assert np.max(np.abs(got["t"] - t) / np.abs(t)) <= 4e-16

    # calc_gz_lev: each half level sums its layers down to the surface, in order
    dz = cfg.Rd * t * np.log(ph_lev[1:] / ph_lev[:-1])
    gz_lev = np.empty((nlev + 1, nlat, nlon))
    gz_lev[nlev] = gzs
    for k in range(nlev):
        acc = np.zeros((nlat, nlon))
        for l in range(k, nlev):
            acc = acc + dz[l]
        gz_lev[k] = gzs + acc
    z = 0.5 * (gz_lev[:-1] + gz_lev[1:]) / cfg.g
    assert np.max(np.abs(got["z"] - z)) <= 1e-13 * np.max(np.abs(z))


def test_shallow_water_history_diagnostics_equal_restatement():
    """Shallow water: z = gz / g of the state, div, and vor whose polar rings
    take the layer mass (gz - gzs) / g (calc_m, operators_mod.F90:527-531)."""
    cfg = abi.default_config(nlon=72, nlat=37, nlev=1, baroclinic=0, dt_dyn=600.0, time_scheme=abi.TIME_PC2)
    o = Oracle(cfg)
    load_state(o, g.make_ic(cfg, 1, 23, 1.0))
    o.prepare()
    o.step(3)
    got = o.output_diag()
    nlon, nlat = cfg.nlon, cfg.nlat
    nh = nlat - 1
    u, v, gz, gzs = o.get_field("u_f"), o.get_field("v_f"), o.get_field("gz"), o.get_field("gzs")
    full = {n: o.metric(n, nlat) for n in ("le_lon", "de_lon", "area_cell")}
    half = {n: o.metric(n, nh) for n in ("le_lat", "de_lat", "area_vtx", "half_tangent_wgt1", "half_tangent_wgt2")}
    o.close()
    gz, gzs = gz.reshape(1, nlat, nlon), gzs.reshape(1, nlat, nlon)
    assert np.array_equal(got["z"], gz / cfg.g)
    lel, ll, ac = full["le_lon"], half["le_lat"], full["area_cell"]
    div = np.zeros((1, nlat, nlon))
    for jj in range(1, nlat - 1):
        div[:, jj] = ((u[:, jj] * lel[jj] - west(u[:, jj]) * lel[jj]) +
                      (v[:, jj] * ll[jj] - v[:, jj - 1] * ll[jj - 1])) / ac[jj]
    div[:, 0] = (ring(v[:, 0]) * ll[0] / nlon / ac[0])[:, None]
    div[:, -1] = (ring(-v[:, -1]) * ll[-1] / nlon / ac[-1])[:, None]
    assert np.array_equal(got["div"], div)
    m = (gz - gzs) / cfg.g
    mfx = (m + east(m)) * 0.5 * u
    mfx[:, 0] = 0.0
    mfx[:, -1] = 0.0
    w1, w2 = half["half_tangent_wgt1"], half["half_tangent_wgt2"]

    def u_lat(hh):
        mf = w1[hh] * (west(mfx[:, hh]) + mfx[:, hh]) + w2[hh] * (west(mfx[:, hh + 1]) + mfx[:, hh + 1])
        return mf / ((m[:, hh] + m[:, hh + 1]) * 0.5)

    dl, dla, av = full["de_lon"], half["de_lat"], half["area_vtx"]
    vor = np.zeros((1, nh, nlon))
    for hh in range(nh):
        vor[:, hh] = (u[:, hh] * dl[hh] - u[:, hh + 1] * dl[hh + 1] + east(v[:, hh]) * dla[hh] -
                      v[:, hh] * dla[hh]) / av[hh]
    vor[:, 0] = (ring(-u_lat(0) * ll[0]) / nlon / ac[0])[:, None]
    vor[:, -1] = (ring(u_lat(nh - 1) * ll[nh - 1]) / nlon / ac[nh])[:, None]
    assert np.array_equal(got["vor"], vor)
