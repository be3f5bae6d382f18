"""The oracle's diagnostic operators against a separate numpy restatement of
the reference's operators_mod, on the prepared state (the run prologue's
all-pass operators_prepare leaves them in state(old)):

* calc_ph, calc_t (operators_mod.F90:136-190; hybrid_coord_calc_ph_lev,
  hybrid_coord_mod.F90:155-160; temperature, formula_mod.F90:24-31):
  ph_lev, ph_exn_lev = ph_lev^(Rd/cpd), t;
* calc_gz_lev (:433-469): gz_lev(k) = gzs + sum_{l=k}^{nlev} Rd t log(ratio),
  summed left to right for every k, the bottom level gzs;
* calc_m (:471-543): m, m_lev (one-sided at top and bottom), and its edge and
  vertex means (interp_mod.F90:233-275, 438-463);
* calc_mf (:545-610): mass fluxes and the tangential winds u_lat, v_lon;
* calc_ke with ke_scheme 2 (:234-352): cell KE blended with the four vertex
  KEs, the pole rows the ring mean of v^2 on the adjacent half row;
* calc_vor / calc_pv with pv_pole_stokes (:612-703);
* interp_pv_upwind with upwind_order_pv 3 (:738-795; upwind3,
  upwind_mod.F90:27-39), reading PV beyond the poles as fill_halo leaves it.

Expressions keep the reference's operation order (Fortran x**2 is x*x; ring
sums run sequentially over longitude) so that agreement is bit for bit,
with a tolerance of a few ulps for pow/log/sqrt."""
import math

import numpy as np
import pytest

from oracle import Oracle

from helpers import baroclinic_config, initial_state, load_state, swm_config

ULPS = 8 * np.finfo(float).eps
EPS = np.finfo(float).eps
POW = np.vectorize(math.pow)
LOG = np.vectorize(math.log)


def close(got, want, tol=ULPS):
    return float(np.abs(got - want).max() / np.abs(want).max()) <= tol


def ring(x):
    """Sequential sum over longitude (last axis), as zonal_sum on one rank."""
    return np.cumsum(x, axis=-1)[..., -1]


def prepared(cfg, seed=7):
    """The oracle after the run prologue on a seeded state, with a smooth
    meridional wind added (the seeded jets have v = 0)."""
    st = initial_state(cfg, seed)
    v = st["v_lat"]
    lon = np.arange(cfg.nlon) * 2 * np.pi / cfg.nlon
    lat = np.linspace(-np.pi / 2, np.pi / 2, cfg.nlat + 1)[1:-1]
    st["v_lat"] = v + 8.0 * np.cos(lat)[None, :, None] * np.sin(3 * lon + 0.5)[None, None, :] * np.ones((v.shape[0], 1, 1))
    o = Oracle(cfg)
    load_state(o, st)
    o.prepare()
    return o


# ---------------------------------------------------------------------------
# column diagnostics (baroclinic)
# ---------------------------------------------------------------------------
def columns(cfg, o):
    nlev = cfg.nlev
    hyai, hybi = o.metric("hyai", nlev + 1), o.metric("hybi", nlev + 1)
    test_l26 = cfg.vert_coord_template == 26
    lp = 0.0 if test_l26 else cfg.ptop            # local_ptop (hybrid_coord_mod.F90:78-90)
    phs = o.get_field("phs_f")
    ph_lev = np.array([hyai[k] * (cfg.hybrid_coord_p0 - lp) + hybi[k] * (phs - lp) + lp for k in range(nlev + 1)])
    kappa = cfg.Rd / cfg.cpd
    ph = 0.5 * (ph_lev[:-1] + ph_lev[1:])
    t = o.get_field("pt") * POW(ph / cfg.p0, kappa)
    gzs = o.get_field("gzs")
    gz_lev = np.zeros_like(ph_lev)
    gz_lev[-1] = gzs
    for k in range(nlev):
        dgz = np.zeros_like(phs)
        for l in range(k, nlev):
            dgz = dgz + cfg.Rd * t[l] * LOG(ph_lev[l + 1] / ph_lev[l])
        gz_lev[k] = gzs + dgz
    m_lev = np.zeros_like(ph_lev)
    m_lev[1:-1] = ph[1:] - ph[:-1]
    m_lev[0] = ph[0] - ph_lev[0]
    m_lev[-1] = ph_lev[-1] - ph[-1]
    return {"ph_lev": ph_lev, "ph_exn_lev": POW(ph_lev, kappa), "t": t, "gz_lev": gz_lev,
            "m": ph_lev[1:] - ph_lev[:-1], "m_lev": m_lev}


@pytest.mark.parametrize("nlev", [26, 32])
def test_column_diagnostics_match_restatement(nlev):
    cfg = baroclinic_config(nlev=nlev)
    o = prepared(cfg)
    try:
        for name, want in columns(cfg, o).items():
            got = o.get_field(name)
            assert got.shape == want.shape, name
            assert close(got, want), name
    finally:
        o.close()


# ---------------------------------------------------------------------------
# horizontal operators; arrays [k][j][i], 0-based, i = longitude
# ---------------------------------------------------------------------------
def prev(x):
    """x(i-1) with the longitude wrap."""
    return np.roll(x, 1, axis=-1)


def nxt(x):
    """x(i+1) with the longitude wrap."""
    return np.roll(x, -1, axis=-1)


def upwind3(f1, f2, f3, f4, wgt, sgn):
    c31, c32, c33 = 7.0 / 12.0, -1.0 / 12.0, 1.0 / 12.0
    return c31 * (f3 + f2) + c32 * (f4 + f1) + c33 * (f4 - f1 - 3 * (f3 - f2)) * wgt * sgn


def edge_pv(pv, un_or_ut, vt_or_vn, wgt, along_lat):
    """interp_pv_upwind, order 3: the blend of the upwind value and the mean
    by b = |tangent| / (|V| + eps); f1..f4 the four PV values along the line
    through the edge."""
    f1, f2, f3, f4 = pv
    t = vt_or_vn if not along_lat else un_or_ut       # tangential component
    n = un_or_ut if not along_lat else vt_or_vn
    if not along_lat:
        b = np.abs(t) / (np.sqrt(n * n + t * t) + EPS)
    else:
        b = np.abs(t) / (np.sqrt(t * t + n * n) + EPS)
    return b * upwind3(f1, f2, f3, f4, wgt, np.copysign(1.0, t)) + (1 - b) * 0.5 * (f2 + f3)


def horizontal(cfg, o):
    nlat, nhalf, nlon = cfg.nlat, cfg.nlat - 1, cfg.nlon
    M = {n: o.metric(n, nlat) for n in ("de_lon", "le_lon", "area_cell", "area_subcell1", "area_subcell2",
                                         "area_lon_west", "area_lon_east", "area_lon_north", "area_lon_south",
                                         "full_tangent_wgt1", "full_tangent_wgt2")}
    M.update({n: o.metric(n, nhalf) for n in ("de_lat", "le_lat", "area_vtx", "area_lat_west", "area_lat_east",
                                             "area_lat_north", "area_lat_south", "half_tangent_wgt1",
                                             "half_tangent_wgt2", "half_f")})
    col = lambda n: M[n][None, :, None]
    u, v, m = o.get_field("u_f"), o.get_field("v_f"), o.get_field("m")
    I = slice(1, nlat - 1)                      # full rows without the poles
    out = {}
    # calc_m's edge and vertex means, calc_mf
    m_lon = (m + nxt(m)) * 0.5
    m_lat = (m[:, :-1] + m[:, 1:]) * 0.5
    m_vtx = ((m[:, :-1] + nxt(m[:, :-1])) * col("area_subcell2")[:, :-1] +
             (m[:, 1:] + nxt(m[:, 1:])) * col("area_subcell1")[:, 1:]) / col("area_vtx")
    mfx = o.get_field("mfx_lon")                # pole rows as the oracle leaves them (zero weights)
    mfx[:, I] = m_lon[:, I] * u[:, I]
    mfy = m_lat * v
    mfx_lat = (col("half_tangent_wgt1") * (prev(mfx[:, :-1]) + mfx[:, :-1]) +
               col("half_tangent_wgt2") * (prev(mfx[:, 1:]) + mfx[:, 1:]))
    u_lat = mfx_lat / m_lat
    mfy_lon = (col("full_tangent_wgt1")[:, I] * (mfy[:, :-1] + nxt(mfy[:, :-1])) +
               col("full_tangent_wgt2")[:, I] * (mfy[:, 1:] + nxt(mfy[:, 1:])))
    v_lon = mfy_lon / m_lon[:, I]
    out.update(mfx_lon=(mfx[:, I], I), mfy_lat=(mfy, None), u_lat=(u_lat, None), v_lon=(v_lon, I))
    # calc_ke
    sq = lambda x: x * x
    ke = np.zeros_like(m)
    cell = (col("area_lon_west")[:, I] * sq(prev(u[:, I])) + col("area_lon_east")[:, I] * sq(u[:, I]) +
            col("area_lat_north")[:, :-1] * sq(v[:, :-1]) + col("area_lat_south")[:, 1:] * sq(v[:, 1:])
            ) / col("area_cell")[:, I]
    if cfg.ke_scheme == 2 and cfg.baroclinic:   # shallow water runs ke_scheme 1 (namelist_mod.F90:227-249)
        hs, hn = slice(0, nhalf - 1), slice(1, nhalf)          # half rows j-1 and j of full rows I
        lon_n, lon_s = col("area_lon_north"), col("area_lon_south")
        lat_e, lat_w, av = col("area_lat_east"), col("area_lat_west"), col("area_vtx")
        up, um, dn = u[:, 2:], u[:, I], u[:, :-2]               # full rows j+1, j, j-1
        kv1 = (lat_e[:, hn] * sq(prev(v[:, hn])) + lat_w[:, hn] * sq(v[:, hn]) +
               lon_n[:, I] * sq(prev(um)) + lon_s[:, 2:] * sq(prev(up))) / av[:, hn]
        kv2 = (lat_e[:, hs] * sq(prev(v[:, hs])) + lat_w[:, hs] * sq(v[:, hs]) +
               lon_n[:, :-2] * sq(prev(dn)) + lon_s[:, I] * sq(prev(um))) / av[:, hs]
        kv3 = (lat_e[:, hs] * sq(v[:, hs]) + lat_w[:, hs] * sq(nxt(v[:, hs])) +
               lon_n[:, :-2] * sq(dn) + lon_s[:, I] * sq(um)) / av[:, hs]
        kv4 = (lat_e[:, hn] * sq(v[:, hn]) + lat_w[:, hn] * sq(nxt(v[:, hn])) +
               lon_n[:, I] * sq(um) + lon_s[:, 2:] * sq(up)) / av[:, hn]
        w = cfg.ke_cell_wgt
        cell = (1.0 - w) * ((kv1 + kv4) * col("area_subcell2")[:, I] +
                            (kv2 + kv3) * col("area_subcell1")[:, I]) / col("area_cell")[:, I] + w * cell
    ke[:, I] = cell
    ke[:, 0] = (ring(sq(v[:, 0])) / nlon)[:, None]
    ke[:, -1] = (ring(sq(v[:, -1])) / nlon)[:, None]
    out["ke"] = (ke, None)
    # calc_vor, calc_pv (pv_pole_stokes)
    vor = (u[:, :-1] * col("de_lon")[:, :-1] - u[:, 1:] * col("de_lon")[:, 1:] +
           nxt(v) * col("de_lat") - v * col("de_lat")) / col("area_vtx")
    vor[:, 0] = (ring(-u_lat[:, 0] * M["le_lat"][0]) / nlon / M["area_cell"][0])[:, None]
    vor[:, -1] = (ring(u_lat[:, -1] * M["le_lat"][-1]) / nlon / M["area_cell"][-1])[:, None]
    pv = (vor + col("half_f")) / m_vtx
    out.update(vor=(vor, None), pv=(pv, None))
    # interp_pv_upwind: half rows beyond the poles are the first/last half
    # rows rotated by nlon/2 (fill_halo on one rank)
    P = np.concatenate([np.roll(pv[:, :1], nlon // 2, axis=-1), pv, np.roll(pv[:, -1:], nlon // 2, axis=-1)], axis=1)
    jf = np.arange(1, nlat - 1)
    f = [P[:, jf - 1], P[:, jf], P[:, jf + 1], P[:, jf + 2]]
    pv_lon = edge_pv(f, u[:, I], v_lon, cfg.upwind_wgt_pv, along_lat=False)
    g = [np.roll(pv, 2, axis=-1), prev(pv), pv, nxt(pv)]
    pv_lat = edge_pv(g, u_lat, v, cfg.upwind_wgt_pv, along_lat=True)
    out.update(pv_lon=(pv_lon, I), pv_lat=(pv_lat, None))
    return out


CASES = {
    "swm_5deg": lambda: swm_config(),
    "swm_1deg": lambda: swm_config(nlon=360, nlat=180, dt=60.0),
    "baroclinic_5deg_l26": lambda: baroclinic_config(),
    "baroclinic_4deg_wrf_l32": lambda: baroclinic_config(nlon=90, nlat=46, nlev=32, dt=600.0),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_horizontal_operators_match_restatement(case):
    cfg = CASES[case]()
    o = prepared(cfg)
    try:
        for name, (want, rows) in horizontal(cfg, o).items():
            got = o.get_field(name)
            if rows is not None:
                got = got[:, rows]
            assert got.shape == want.shape, name
            assert np.abs(want).max() > 0, name
            assert close(got, want), (case, name)
    finally:
        o.close()
