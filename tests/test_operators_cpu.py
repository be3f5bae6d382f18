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


def prepared(cfg, seed=7, u_wave=0.0):
    """The oracle after the run prologue on a seeded state, with a smooth
    meridional wind added and the winds sheared in the vertical (the seeded
    jets have v = 0, no shear and no zonal variation)."""
    st = initial_state(cfg, seed)
    shear = (1.0 + 0.03 * np.arange(cfg.nlev))[:, None, None]
    lon = np.arange(cfg.nlon) * 2 * np.pi / cfg.nlon
    st["u_lon"] = st["u_lon"] * shear * (1.0 + 0.2 * np.sin(2 * lon))[None, None, :]
    # optional wavenumber-2 zonal wind of both signs that keeps its strength
    # up to the poles (Courant numbers beyond one cell where rows are short)
    st["u_lon"] = st["u_lon"] + u_wave * np.sin(2 * (lon + np.pi / cfg.nlon))[None, None, :]
    v = st["v_lat"]
    lat = np.linspace(-np.pi / 2, np.pi / 2, cfg.nlat + 1)[1:-1]
    st["v_lat"] = v + 8.0 * np.cos(lat)[None, :, None] * np.sin(3 * lon + 0.5)[None, None, :] * shear
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
    "swm_5deg_coriolis2": lambda: swm_config(coriolis_scheme=2),
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


# ---------------------------------------------------------------------------
# tendencies of the forward pass (space_operators, gmcore_mod.F90:467-528)
# and the pressure-gradient force of the backward pass
# ---------------------------------------------------------------------------
def forward_tendencies(cfg, o):
    """calc_coriolis scheme 1 (:846-906), calc_grad_ke (:908-937),
    calc_grad_mf (:939-1006), calc_dphsdt (:1120-1143), calc_we_lev
    (:192-232, area-weighted edge means interp_mod.F90:308-436) and
    calc_wedudlev_wedvdlev (SB81, :1145-1216), from the pass's own
    diagnostics."""
    nlat, nhalf, nlon, nlev = cfg.nlat, cfg.nlat - 1, cfg.nlon, cfg.nlev
    M = {n: o.metric(n, nlat) for n in ("de_lon", "le_lon", "area_cell", "area_lon", "area_lon_west",
                                         "area_lon_east", "full_tangent_wgt1", "full_tangent_wgt2")}
    M.update({n: o.metric(n, nhalf) for n in ("de_lat", "le_lat", "area_lat", "area_lat_north", "area_lat_south",
                                             "half_tangent_wgt1", "half_tangent_wgt2")})
    col = lambda n: M[n][None, :, None]
    F = {n: o.get_field(n) for n in ("mfx_lon", "mfy_lat", "pv_lon", "pv_lat", "ke", "u_f", "v_f", "m")}
    mfx, mfy, pvx, pvy, ke = F["mfx_lon"], F["mfy_lat"], F["pv_lon"], F["pv_lat"], F["ke"]
    I = slice(1, nlat - 1)
    out = {}
    out["qhu"] = (col("half_tangent_wgt1") * (prev(mfx[:, :-1]) * (pvy + prev(pvx[:, :-1])) +
                                               mfx[:, :-1] * (pvy + pvx[:, :-1])) +
                  col("half_tangent_wgt2") * (prev(mfx[:, 1:]) * (pvy + prev(pvx[:, 1:])) +
                                               mfx[:, 1:] * (pvy + pvx[:, 1:]))) * 0.5, None
    pc = pvx[:, I]
    out["qhv"] = (col("full_tangent_wgt1")[:, I] * (mfy[:, :-1] * (pc + pvy[:, :-1]) +
                                                     nxt(mfy[:, :-1]) * (pc + nxt(pvy[:, :-1]))) +
                  col("full_tangent_wgt2")[:, I] * (mfy[:, 1:] * (pc + pvy[:, 1:]) +
                                                     nxt(mfy[:, 1:]) * (pc + nxt(pvy[:, 1:])))) * 0.5, I
    out["dkedlon"] = (nxt(ke[:, I]) - ke[:, I]) / col("de_lon")[:, I], I
    out["dkedlat"] = (ke[:, 1:] - ke[:, :-1]) / col("de_lat"), None
    out["dmfdlon"] = (mfx[:, I] - prev(mfx[:, I])) * col("le_lon")[:, I] / col("area_cell")[:, I], I
    dmfdlat = np.zeros((nlev, nlat, nlon))
    dmfdlat[:, I] = (mfy[:, 1:] * col("le_lat")[:, 1:] - mfy[:, :-1] * col("le_lat")[:, :-1]) / col("area_cell")[:, I]
    dmfdlat[:, 0] = (ring(mfy[:, 0]) * M["le_lat"][0] / nlon / M["area_cell"][0])[:, None]
    dmfdlat[:, -1] = (ring(-mfy[:, -1]) * M["le_lat"][-1] / nlon / M["area_cell"][-1])[:, None]
    out["dmfdlat"] = dmfdlat, None
    if cfg.coriolis_scheme == 2:      # qhu = mfx_lat pv_lat, qhv = mfy_lon pv_lon (:879, 899)
        mfx_lat = (col("half_tangent_wgt1") * (prev(mfx[:, :-1]) + mfx[:, :-1]) +
                   col("half_tangent_wgt2") * (prev(mfx[:, 1:]) + mfx[:, 1:]))
        mfy_lon = (col("full_tangent_wgt1")[:, I] * (mfy[:, :-1] + nxt(mfy[:, :-1])) +
                   col("full_tangent_wgt2")[:, I] * (mfy[:, 1:] + nxt(mfy[:, 1:])))
        out["qhu"] = mfx_lat * pvy, None
        out["qhv"] = mfy_lon * pvx[:, I], I
    if not cfg.baroclinic:            # shallow water (gmcore_mod.F90:503-518)
        out["du"] = out["qhv"][0] - out["dkedlon"][0], I
        out["dv"] = -out["qhu"][0] - out["dkedlat"][0], None
        dmfdlon = o.get_tend(0, "dmfdlon")
        dmfdlon[:, I] = out["dmfdlon"][0]
        out["dgz"] = -(dmfdlon + dmfdlat) * cfg.g, None
        return out
    dmfdlon = o.get_tend(0, "dmfdlon")          # pole rows as the pass leaves them
    dmfdlon[:, I] = out["dmfdlon"][0]
    dphs = np.zeros((nlat, nlon))
    for k in range(nlev):
        dphs = dphs - dmfdlon[k] - dmfdlat[k]
    out["dphs"] = dphs, None
    hybi = o.metric("hybi", nlev + 1)
    we = np.zeros((nlev + 1, nlat, nlon))
    mf = np.zeros((nlat, nlon))
    for k in range(1, nlev):
        mf = mf + dmfdlon[k - 1] + dmfdlat[k - 1]
        we[k] = -(hybi[k] * dphs) - mf
    out["we_lev"] = we, None
    we_lon = (col("area_lon_west")[:, I] * we[:, I] + col("area_lon_east")[:, I] * nxt(we[:, I])) / col("area_lon")[:, I]
    we_lat = (col("area_lat_north") * we[:, 1:] + col("area_lat_south") * we[:, :-1]) / col("area_lat")
    m = F["m"]
    m_lon, m_lat = ((m + nxt(m)) * 0.5)[:, I], (m[:, :-1] + m[:, 1:]) * 0.5

    def sb81(w, x, mm):
        r = np.zeros_like(x)
        r[1:-1] = (w[2:-1] * (x[2:] - x[1:-1]) + w[1:-2] * (x[1:-1] - x[:-2])) / mm[1:-1] / 2.0
        r[0] = (w[1] * (x[1] - x[0])) / mm[0] / 2.0
        r[-1] = (w[-2] * (x[-1] - x[-2])) / mm[-1] / 2.0
        return r
    out["wedudlev"] = sb81(we_lon, F["u_f"][:, I], m_lon), I
    out["wedvdlev"] = sb81(we_lat, F["v_f"], m_lat), None
    out["du"] = out["qhv"][0] - out["dkedlon"][0] - out["wedudlev"][0], I
    out["dv"] = -out["qhu"][0] - out["dkedlat"][0] - out["wedvdlev"][0], None
    return out


def pressure_gradient(cfg, o):
    """pgf_lin97_run, hydrostatic (pgf_lin97_mod.F90:20-105), or pgf_swm_run
    (pgf_swm_mod.F90:18-46)."""
    nlat, nhalf = cfg.nlat, cfg.nlat - 1
    de_lon, de_lat = o.metric("de_lon", nlat)[None, :, None], o.metric("de_lat", nhalf)[None, :, None]
    I = slice(1, nlat - 1)
    if not cfg.baroclinic:
        gz = o.get_field("gz_f")
        return {"pgf_lon": ((nxt(gz[:, I]) - gz[:, I]) / de_lon[:, I], I),
                "pgf_lat": ((gz[:, 1:] - gz[:, :-1]) / de_lat, None)}
    E, Z = o.get_field("ph_exn_lev"), o.get_field("gz_lev")

    def lin97(e0, e1, z0, z1, de):
        """Corners: 0 this side, 1 the other; [:-1] level k, [1:] level k+1."""
        dph1 = e1[1:] - e0[:-1]
        dph2 = e0[1:] - e1[:-1]
        dgz1 = z0[1:] - z1[:-1]
        dgz2 = z0[:-1] - z1[1:]
        return -(dph1 * dgz1 + dph2 * dgz2) / de / (dph1 + dph2)
    return {"pgf_lon": (lin97(E[:, I], nxt(E[:, I]), Z[:, I], nxt(Z[:, I]), de_lon[:, I]), I),
            "pgf_lat": (lin97(E[:, :-1], E[:, 1:], Z[:, :-1], Z[:, 1:], de_lat), None)}


@pytest.mark.parametrize("case", sorted(CASES))
def test_tendencies_match_restatement(case):
    cfg = CASES[case]()
    o = prepared(cfg)
    try:
        o.run_pass(0)
        for name, (want, rows) in forward_tendencies(cfg, o).items():
            got = o.get_field(name) if name == "we_lev" else o.get_tend(0, name)
            if rows is not None:
                got = got[:, rows]
            assert got.shape == want.shape, name
            assert np.abs(want).max() > 0, name
            assert close(got, want), (case, name, float(np.abs(got - want).max() / np.abs(want).max()))
        o.run_pass(1)
        for name, (want, rows) in pressure_gradient(cfg, o).items():
            got = o.get_tend(1, name)
            if rows is not None:
                got = got[:, rows]
            assert close(got, want), (case, name, float(np.abs(got - want).max() / np.abs(want).max()))
    finally:
        o.close()


# ---------------------------------------------------------------------------
# the dynamic mass batch: Courant numbers from RK4 departure points and the
# axis divergences (adv_batch_accum_uv_cell, adv_batch_mod.F90:218-377)
# ---------------------------------------------------------------------------
def batch_courant(cfg, o, dt, get=None):
    """get(name): the batch field reader (the mass batch by default)."""
    get = get or o.get_batch
    nlat, nhalf, nlon, nlev = cfg.nlat, cfg.nlat - 1, cfg.nlon, cfg.nlev
    R = cfg.radius
    dlon = (2 * math.pi - 0.0) / nlon
    half_lon = lambda l: (0.0 + (l - 1) * dlon) + 0.5 * dlon          # any index, halo included
    u, v = get("u"), get("v")
    fcos, hlat = o.metric("full_cos_lat", nlat), o.metric("half_lat", nhalf)
    de_lon, de_lat = o.metric("de_lon", nlat), o.metric("de_lat", nhalf)
    le_lon, le_lat, area = o.metric("le_lon", nlat), o.metric("le_lat", nhalf), o.metric("area_cell", nlat)
    I = slice(1, nlat - 1)
    # x: rows 2..nlat-1, faces i = 1..nlon; u at any face index by the wrap
    ii = np.arange(1, nlon + 1)[None, None, :].astype(float)
    cos = fcos[None, I, None]
    dx = de_lon[None, I, None]
    uI = u[:, I]
    uat = lambda l: np.take_along_axis(uI, (l - 1) % nlon, axis=-1)
    x0 = R * half_lon(ii) * cos

    def ux(x):
        l = np.floor(ii + (x - x0) / dx).astype(np.int64)
        return ((R * half_lon(l + 1) * cos - x) * uat(l) + (x - R * half_lon(l) * cos) * uat(l + 1)) / dx
    u1 = uI
    x1 = x0 + dt / 2 * u1
    u2 = ux(x1)
    x2 = x0 + dt / 2 * u2
    u3 = ux(x2)
    x3 = x0 + dt * u3
    u4 = ux(x3)
    cflx = (u1 + 2 * u2 + 2 * u3 + u4) / 6 * dt / dx
    # y: half rows 1..nhalf; outside 1..nhalf-1 the first stage's wind
    jj = np.arange(1, nhalf + 1)[None, :, None].astype(float)
    dy = de_lat[None, :, None]
    y0 = R * hlat[None, :, None]
    hl = lambda l: hlat[np.clip(l, 1, nhalf) - 1]

    def vy(y, v1):
        l = np.floor(jj + (y - y0) / dy).astype(np.int64) * np.ones_like(v1, dtype=np.int64)
        inside = (l >= 1) & (l <= nhalf - 1)
        lc = np.clip(l, 1, nhalf - 1)
        va = np.take_along_axis(v, lc - 1, axis=1)
        vb = np.take_along_axis(v, lc, axis=1)
        interp = ((R * hl(lc + 1) - y) * va + (y - R * hl(lc)) * vb) / dy
        return np.where(inside, interp, v1)
    v1 = v
    y1 = y0 + dt / 2 * v1
    v2 = vy(y1, v1)
    y2 = y0 + dt / 2 * v2
    v3 = vy(y2, v1)
    y3 = y0 + dt * v3
    v4 = vy(y3, v1)
    cfly = (v1 + 2 * v2 + 2 * v3 + v4) / 6 * dt / dy
    divx = (uI - prev(uI)) * le_lon[None, I, None] / area[None, I, None]
    divy = np.zeros((nlev, nlat, nlon))
    divy[:, I] = (v[:, 1:] * le_lat[None, 1:, None] - v[:, :-1] * le_lat[None, :-1, None]) / area[None, I, None]
    divy[:, 0] = (ring(v[:, 0]) * le_lat[0] / nlon / area[0])[:, None]
    divy[:, -1] = (ring(-v[:, -1]) * le_lat[-1] / nlon / area[-1])[:, None]
    return {"cflx": (cflx, I), "cfly": (cfly, None), "divx": (divx, I), "divy": (divy, None)}


@pytest.mark.parametrize("case", ["baroclinic_5deg_l26", "baroclinic_4deg_wrf_l32", "long_step"])
def test_batch_courant_numbers_match_restatement(case):
    if case == "long_step":   # departure points several cells away, winds of both signs
        cfg = baroclinic_config(dt=1200.0)
        o = prepared(cfg, u_wave=60.0)
    else:
        cfg = CASES[case]()
        o = prepared(cfg)
    try:
        o.run_pass(0)
        if case == "long_step":
            assert np.abs(o.get_batch("cflx")).max() > 1.0 and o.get_batch("u").min() < 0.0
        assert np.array_equal(o.get_batch("u")[:, 1:-1], o.get_field("u_f")[:, 1:-1])   # the dynamic batch copies
        for name, (want, rows) in batch_courant(cfg, o, cfg.dt_dyn).items():
            got = o.get_batch(name)
            if rows is not None:
                got = got[:, rows]
            assert got.shape == want.shape, name
            assert np.abs(want).max() > 0, name
            assert close(got, want), (case, name, float(np.abs(got - want).max() / np.abs(want).max()))
    finally:
        o.close()


# ---------------------------------------------------------------------------
# the polar filters applied by the run prologue (gmcore_mod.F90:109-122):
# u_f, v_f and phs_f / gz_f are the big filter of u_lon, v_lat, phs / gz
# (filter_on_lon_edge / _lat_edge / _cell, filter_mod.F90:25-163)
# ---------------------------------------------------------------------------
def filter_rows(o, x, lat, which=0):
    """tmp(i) = sum(wgt(:n,j) * x(i-hn:i+hn,j)), summed over the taps in
    order, on rows with more than one tap; other rows copied.  which: 0 big,
    1 small1, 2 small2."""
    y = x.copy()
    taps = o.filter_taps(which, lat)
    for j in range(x.shape[-2]):
        n = int(taps[j])
        if n <= 1:
            continue
        w, hn = o.filter_weights(which, lat, j + 1), (n - 1) // 2
        row = x[..., j, :]
        acc = np.zeros_like(row)
        for t in range(n):
            acc = acc + w[t] * np.roll(row, hn - t, axis=-1)     # x(i - hn + t)
        y[..., j, :] = acc
    return y


@pytest.mark.parametrize("case", sorted(CASES))
def test_prologue_filters_match_restatement(case):
    cfg = CASES[case]()
    o = prepared(cfg)
    try:
        pairs = [("u_lon", "u_f", 0), ("v_lat", "v_f", 1)]
        pairs.append(("phs", "phs_f", 0) if cfg.baroclinic else ("gz", "gz_f", 0))
        for src, dst, lat in pairs:
            x = o.get_field(src)
            want = filter_rows(o, x, lat)
            got = o.get_field(dst)
            assert not np.array_equal(want, x), dst          # some rows are filtered
            assert close(got, want), (case, dst, float(np.abs(got - want).max() / np.abs(want).max()))
    finally:
        o.close()


# ---------------------------------------------------------------------------
# the vertical Courant number of the mass batch: RK4 in eta with a level
# search, then the Lagrangian walk over whole layers (adv_batch_accum_we_lev,
# adv_batch_mod.F90:493-632; level spacings vert_coord_mod.F90:84-101)
# ---------------------------------------------------------------------------
def vertical_courant(cfg, o, dt, get=None):
    """get(name): the batch field reader (the mass batch by default)."""
    get = get or o.get_batch
    nlev = cfg.nlev
    hl, fl = [0.0] + list(o.metric("half_lev", nlev + 1)), [0.0] + list(o.metric("full_lev", nlev))   # 1-based
    full_dlev = [0.0] + [hl[k + 1] - hl[k] for k in range(1, nlev + 1)]
    half_dlev = [0.0] * (nlev + 2)
    for k in range(2, nlev + 1):
        half_dlev[k] = fl[k] - fl[k - 1]
    half_dlev[1] = fl[1] - hl[1]
    half_dlev[nlev + 1] = hl[nlev + 1] - fl[nlev]
    we, mlev = get("we"), get("m_lev")
    cflz = get("cflz").copy()                  # the boundary levels as the batch keeps them
    _, nlat, nlon = we.shape

    def find(k, z, w):
        if w > 0:
            for l in range(k, nlev + 1):
                if hl[l] <= z <= hl[l + 1]:
                    return l
        else:
            for l in range(k - 1, 0, -1):
                if hl[l] <= z <= hl[l + 1]:
                    return l
        raise AssertionError("cflz exceeds range")

    for j in range(nlat):
        for i in range(nlon):
            W = [0.0] + [float(x) for x in we[:, j, i]]
            Ml = [0.0] + [float(x) for x in mlev[:, j, i]]
            for k in range(2, nlev + 1):
                z0 = hl[k]
                w1 = W[k] / Ml[k] * half_dlev[k]
                z1 = z0 + dt / 2 * w1
                l = find(k, z1, w1)
                w2 = ((hl[l + 1] - z1) * W[l] / Ml[l] * half_dlev[l] +
                      (z1 - hl[l]) * W[l + 1] / Ml[l + 1] * half_dlev[l + 1]) / full_dlev[l]
                z2 = z0 + dt / 2 * w2
                l = find(k, z2, w2)
                w3 = ((hl[l + 1] - z2) * W[l] / Ml[l] * half_dlev[l] +
                      (z2 - hl[l]) * W[l + 1] / Ml[l + 1] * half_dlev[l + 1]) / full_dlev[l]
                z3 = z0 + dt * w3
                l = find(k, z3, w3)
                w4 = ((hl[l + 1] - z3) * W[l] / Ml[l] * half_dlev[l] +
                      (z3 - hl[l]) * W[l + 1] / Ml[l + 1] * half_dlev[l + 1]) / full_dlev[l]
                deta = (w1 + 2 * w2 + 2 * w3 + w4) / 6 * dt
                ks, ke, s = (k - 1, 1, -1) if deta < 0 else (k, nlev, 1)
                deta = abs(deta)
                for l in range(ks, ke + s, s):
                    deta = deta - full_dlev[l]
                    if deta < 0:
                        cflz[k - 1, j, i] = s * ((1 + deta / full_dlev[l]) + abs(l - ks))
                        break
    return cflz


@pytest.mark.parametrize("case", ["baroclinic_5deg_l26", "long_step"])
def test_vertical_courant_numbers_match_restatement(case):
    if case == "long_step":
        cfg = baroclinic_config(dt=1200.0)
        o = prepared(cfg, u_wave=60.0)
    else:
        cfg = CASES[case]()
        o = prepared(cfg)
    try:
        o.run_pass(0)
        assert np.array_equal(o.get_batch("we"), o.get_field("we_lev"))      # the dynamic batch copies
        want = vertical_courant(cfg, o, cfg.dt_dyn)
        got = o.get_batch("cflz")
        assert np.abs(want[1:-1]).max() > 0
        if case == "long_step":
            assert np.abs(got).max() > 1.0      # departure beyond the adjacent layer
        assert close(got, want), (case, float(np.abs(got - want).max() / np.abs(want).max()))
    finally:
        o.close()


# ---------------------------------------------------------------------------
# the vertical FFSL flux of pt and its divergence dptfdlev: linear ghost
# levels (operators_mod.F90:1085-1092), PPM cells with the monotone slope
# (ppm, slope_mono, ffsl_mod.F90:1147-1194), whole-layer sums plus the
# parabola's integral over the fractional part (vflx_ppm_cell, :883-941);
# no flux through the top and bottom interfaces
# ---------------------------------------------------------------------------
def slope_mono(fm1, f, fp1):
    df = (fp1 - fm1) * 0.5
    df_min = 2 * (f - np.minimum(np.minimum(fm1, f), fp1))
    df_max = 2 * (np.maximum(np.maximum(fm1, f), fp1) - f)
    return np.copysign(np.minimum(np.minimum(np.abs(df), df_min), df_max), df)


def ppm_cells(fm2, fm1, f, fp1, fp2):
    dfl, df, dfr = slope_mono(fm2, fm1, f), slope_mono(fm1, f, fp1), slope_mono(f, fp1, fp2)
    fl = 0.5 * (fm1 + f) + (dfl - df) / 6.0
    fr = 0.5 * (fp1 + f) + (df - dfr) / 6.0
    fl = f - np.copysign(np.minimum(np.abs(df), np.abs(fl - f)), df)
    fr = f + np.copysign(np.minimum(np.abs(df), np.abs(fr - f)), df)
    return fl, fr - fl, 6 * f - 3 * (fl + fr)


def vertical_flux_divergence(cfg, o):
    nlev = cfg.nlev
    pt = o.get_field("pt")
    g = np.zeros((nlev + 4,) + pt.shape[1:])          # level k at index k + 1, k = -1 .. nlev + 2
    g[2:nlev + 2] = pt
    g[1] = 2 * g[2] - g[3]
    g[0] = 2 * g[1] - g[2]
    g[nlev + 2] = 2 * g[nlev + 1] - g[nlev]
    g[nlev + 3] = 2 * g[nlev + 2] - g[nlev + 1]
    flux = vertical_flux(g, o.get_batch("we"), o.get_batch("cflz"))
    return flux[1:] - flux[:-1]


def vertical_flux(g, we, cflz):
    """vflx_ppm_cell: fluxes on the half levels of the field g given with two
    ghost levels each side (level k at index k + 1)."""
    nlev = g.shape[0] - 4
    fl, dq, q6 = ppm_cells(g[0:nlev], g[1:nlev + 1], g[2:nlev + 2], g[3:nlev + 3], g[4:nlev + 4])
    cell = lambda a, k: np.take_along_axis(a, (k - 1)[None], axis=0)[0]     # cell k (1-based), per column
    lev = lambda k: np.take_along_axis(g, (k + 1)[None], axis=0)[0]
    flux = np.zeros_like(we)
    for k in range(2, nlev + 1):
        c = cflz[k - 1]
        w = we[k - 1]
        ci = np.trunc(c).astype(np.int64)
        cf = c - ci
        pos = c > 0
        ku = np.where(pos, k - ci - 1, k - ci)
        s1 = np.where(pos, 1 - cf, 0.0)
        s2 = np.where(pos, 1.0, -cf)
        ds1, ds2, ds3 = s2 - s1, s2 * s2 - s1 * s1, s2 * s2 * s2 - s1 * s1 * s1
        total = np.zeros_like(c)                     # whole layers, in increasing level order
        for t in range(int(np.abs(ci).max())):
            first = np.where(pos, k - ci, k)         # k-ci .. k-1 (c > 0) or k .. k-ci-1 (c < 0)
            take = t < np.abs(ci)
            total = np.where(take, total + lev(np.where(take, first + t, k)), total)
        kc = np.clip(ku, 1, nlev)
        body = total + cell(fl, kc) * ds1 + 0.5 * cell(dq, kc) * ds2 + cell(q6, kc) * (ds2 / 2.0 - ds3 / 3.0)
        with np.errstate(divide="ignore", invalid="ignore"):     # c = 0 takes the zero branch
            flux[k - 1] = np.where(c == 0, 0.0, np.where(pos, w * body / c, -w * body / c))
    return flux


@pytest.mark.parametrize("case", ["baroclinic_5deg_l26", "baroclinic_4deg_wrf_l32", "long_step"])
def test_vertical_flux_divergence_matches_restatement(case):
    if case == "long_step":
        cfg = baroclinic_config(dt=1200.0)
        o = prepared(cfg, u_wave=60.0)
    else:
        cfg = CASES[case]()
        o = prepared(cfg)
    try:
        o.run_pass(0)
        want = vertical_flux_divergence(cfg, o)
        got = o.get_tend(0, "dptfdlev")
        assert np.abs(want).max() > 0
        assert close(got, want), (case, float(np.abs(got - want).max() / np.abs(want).max()))
    finally:
        o.close()


# ---------------------------------------------------------------------------
# the horizontal FFSL flux of pt and its divergence (calc_grad_ptf,
# operators_mod.F90:1008-1083; ffsl_calc_tracer_hflx_cell, ffsl_mod.F90:
# 318-413; hflx_ppm_cell, :778-881): inner advective fluxes of q, the
# intermediates qx, qy with the divergence corrections and the polar rings,
# then the outer fluxes of qy along x and qx along y with the mass fluxes
# ---------------------------------------------------------------------------
def lat_halo(x):
    """Two full rows beyond each pole, rotated by nlon/2 (fill_halo)."""
    h = x.shape[-1] // 2
    r = lambda j: np.roll(x[:, j:j + 1], h, axis=-1)
    return np.concatenate([r(2), r(1), x, r(-2), r(-3)], axis=1)


def hflx_ppm(u, v, mx, my, cflx, cfly):
    nlat = mx.shape[1]
    nlon = mx.shape[-1]
    cx = ppm_cells(np.roll(mx, 2, -1), np.roll(mx, 1, -1), mx, np.roll(mx, -1, -1), np.roll(mx, -2, -1))
    Y = lat_halo(my)
    cy = ppm_cells(Y[:, 0:nlat], Y[:, 1:nlat + 1], Y[:, 2:nlat + 2], Y[:, 3:nlat + 3], Y[:, 4:nlat + 4])
    # whole cells S first, then the parabola's terms, left to right as written
    integral = lambda S, fl, dq, q6, s1, s2: (S + fl * (s2 - s1) + 0.5 * dq * (s2 * s2 - s1 * s1) +
                                              q6 * ((s2 * s2 - s1 * s1) / 2.0 - (s2 * s2 * s2 - s1 * s1 * s1) / 3.0))
    # along x, rows 2 .. nlat-1, faces i = 1 .. nlon (Fortran indices)
    I = slice(1, nlat - 1)
    c = cflx[:, I]
    ci = np.trunc(c).astype(np.int64)
    cf = c - ci
    pos = c > 0
    fi = np.arange(1, nlon + 1)[None, None, :]
    cell = lambda a, m: np.take_along_axis(a[:, I], (m - 1) % nlon, axis=-1)
    iu = np.where(pos, fi - ci, fi - ci + 1)
    first = np.where(pos, fi + 1 - ci, fi + 1)
    S = np.zeros_like(c)
    for t in range(int(np.abs(ci).max())):
        take = t < np.abs(ci)
        S = np.where(take, S + cell(mx, np.where(take, first + t, 1)), S)
    s1, s2 = np.where(pos, 1 - cf, 0.0), np.where(pos, 1.0, -cf)
    body = integral(S, cell(cx[0], iu), cell(cx[1], iu), cell(cx[2], iu), s1, s2)
    fx = np.zeros_like(mx)
    with np.errstate(divide="ignore", invalid="ignore"):
        fx[:, I] = np.where(c == 0, 0.0, np.where(pos, u[:, I] * body / c, -u[:, I] * body / c))
    # along y, half rows j = 1 .. nhalf: upwind cell j (c > 0) or j + 1
    c = cfly
    pos = c > 0
    up = lambda a: np.where(pos, a[:, :-1], a[:, 1:])
    s1, s2 = np.where(pos, 1 - c, 0.0), np.where(pos, 1.0, -c)
    body = integral(0.0, up(cy[0]), up(cy[1]), up(cy[2]), s1, s2)
    with np.errstate(divide="ignore", invalid="ignore"):
        fy = np.where(c == 0, 0.0, np.where(pos, v * body / c, -v * body / c))
    return fx, fy


def ffsl_fluxes(cfg, o, q, B, mfx, mfy, dt, hflx=None):
    """ffsl_calc_tracer_hflx_cell: the outer fluxes (qmfx, qmfy) of q with
    batch B (u, v, cflx, cfly, divx, divy) and mass fluxes mfx, mfy."""
    nlat, nlon = cfg.nlat, cfg.nlon
    le_lon, le_lat, area = (o.metric("le_lon", nlat)[None, :, None], o.metric("le_lat", nlat - 1)[None, :, None],
                            o.metric("area_cell", nlat)[None, :, None])
    I = slice(1, nlat - 1)
    hflx = hflx or hflx_ppm
    fx, fy = hflx(B["u"], B["v"], q, q, B["cflx"], B["cfly"])
    qx, qy = q.copy(), q.copy()
    qx[:, I] = q[:, I] - 0.5 * ((fx[:, I] - prev(fx[:, I])) * le_lon[:, I] / area[:, I] - B["divx"][:, I] * q[:, I]) * dt
    qy[:, I] = q[:, I] - 0.5 * ((fy[:, 1:] * le_lat[:, 1:] - fy[:, :-1] * le_lat[:, :-1]) / area[:, I] -
                                B["divy"][:, I] * q[:, I]) * dt
    ps = (ring(fy[:, 0]) * le_lat[0, 0, 0] / nlon / area[0, 0, 0])[:, None]
    pn = (ring(fy[:, -1]) * le_lat[0, -1, 0] / nlon / area[0, -1, 0])[:, None]
    qy[:, 0] = q[:, 0] - 0.5 * (ps - B["divy"][:, 0] * q[:, 0]) * dt
    qy[:, -1] = q[:, -1] + 0.5 * (pn - B["divy"][:, -1] * q[:, -1]) * dt
    return hflx(mfx, mfy, qy, qx, B["cflx"], B["cfly"])


def horizontal_ffsl(cfg, o, dt):
    nlat, nlon = cfg.nlat, cfg.nlon
    le_lon, le_lat, area = (o.metric("le_lon", nlat)[None, :, None], o.metric("le_lat", nlat - 1)[None, :, None],
                            o.metric("area_cell", nlat)[None, :, None])
    B = {n: o.get_batch(n) for n in ("u", "v", "cflx", "cfly", "divx", "divy")}
    I = slice(1, nlat - 1)
    gx, gy = ffsl_fluxes(cfg, o, o.get_field("pt"), B, o.get_field("mfx_lon"), o.get_field("mfy_lat"), dt)
    dlon = (gx[:, I] - prev(gx[:, I])) * le_lon[:, I] / area[:, I]
    dlat = np.zeros((cfg.nlev, nlat, nlon))
    dlat[:, I] = (gy[:, 1:] * le_lat[:, 1:] - gy[:, :-1] * le_lat[:, :-1]) / area[:, I]
    dlat[:, 0] = (ring(gy[:, 0]) * le_lat[0, 0, 0] / nlon / area[0, 0, 0])[:, None]
    dlat[:, -1] = (ring(-gy[:, -1]) * le_lat[0, -1, 0] / nlon / area[0, -1, 0])[:, None]
    return {"dptfdlon": (dlon, I), "dptfdlat": (dlat, None)}


@pytest.mark.parametrize("case", ["baroclinic_5deg_l26", "baroclinic_4deg_wrf_l32", "long_step"])
def test_horizontal_ffsl_matches_restatement(case):
    if case == "long_step":   # whole-cell departures (|cflx| > 1) near the poles
        cfg = baroclinic_config(dt=1200.0)
        o = prepared(cfg, u_wave=60.0)
    else:
        cfg = CASES[case]()
        o = prepared(cfg)
    try:
        o.run_pass(0)
        for name, (want, rows) in horizontal_ffsl(cfg, o, cfg.dt_dyn).items():
            got = o.get_tend(0, name)
            if rows is not None:
                got = got[:, rows]
            assert np.abs(want).max() > 0, name
            assert close(got, want), (case, name, float(np.abs(got - want).max() / np.abs(want).max()))
    finally:
        o.close()


# ---------------------------------------------------------------------------
# update_state (time_schemes_mod.F90:120-242) over one Euler step (one
# forward-backward pair, step_forward_backward :102-118): phs and its big
# filter, pt through the layer mass with the small1 filter, u and v with the
# small2 filter, the v blend next to the poles (weight 0.6) and the big filter
# to u_f, v_f; the pass tendencies are the oracle's own (pinned above)
# ---------------------------------------------------------------------------
def euler_update(cfg, o, old, dt):
    nlat, nlev = cfg.nlat, cfg.nlev
    I = slice(1, nlat - 1)
    dphs, dpt = o.get_tend(0, "dphs"), o.get_tend(0, "dpt")
    du, dv = o.get_tend(1, "du"), o.get_tend(1, "dv")
    new = {}
    phs = old["phs"] + dt * dphs
    new["phs"] = phs
    new["phs_f"] = filter_rows(o, phs[None], 0)[0]
    hyai, hybi = o.metric("hyai", nlev + 1), o.metric("hybi", nlev + 1)
    lp = 0.0 if cfg.vert_coord_template == 26 else cfg.ptop
    ph_lev = np.array([hyai[k] * (cfg.hybrid_coord_p0 - lp) + hybi[k] * (new["phs_f"] - lp) + lp
                       for k in range(nlev + 1)])
    m_new = ph_lev[1:] - ph_lev[:-1]
    new["pt"] = filter_rows(o, old["pt"] * old["m"] + dt * dpt, 0, which=1) / m_new
    u = o.get_field("u_lon").copy()                  # pole rows: never updated
    u[:, I] = old["u_lon"][:, I] + dt * du[:, I]
    v = old["v_lat"] + dt * dv
    u = filter_rows(o, u, 0, which=2)
    v = filter_rows(o, v, 1, which=2)
    wgt = 0.6
    v[:, 0] = (1 - wgt) * v[:, 0] + wgt * v[:, 1]
    v[:, -1] = (1 - wgt) * v[:, -1] + wgt * v[:, -2]
    new["u_lon"], new["v_lat"] = u, v
    new["u_f"], new["v_f"] = filter_rows(o, u, 0), filter_rows(o, v, 1)
    return new


@pytest.mark.parametrize("case", ["baroclinic_5deg_l26", "baroclinic_4deg_wrf_l32"])
def test_update_state_matches_restatement(case):
    from gmcore_gb300 import abi
    # dt = 600 s: long enough that the small filters act on the polar rows
    kw = dict(nlon=90, nlat=46, nlev=32, dt=600.0) if "wrf" in case else dict(dt=600.0)
    cfg = baroclinic_config(time_scheme=abi.TIME_EULER, **kw)
    o = prepared(cfg)
    try:
        for which, lat in ((1, 0), (2, 0), (2, 1)):
            assert (o.filter_taps(which, lat) > 1).any()
        old = {f: o.get_field(f) for f in ("u_lon", "v_lat", "pt", "phs", "m")}
        o.step(1)
        for name, want in euler_update(cfg, o, old, cfg.dt_dyn).items():
            got = o.get_field(name)
            assert got.shape == want.shape, name
            assert close(got, want), (case, name, float(np.abs(got - want).max() / np.abs(want).max()))
    finally:
        o.close()


# ---------------------------------------------------------------------------
# diagnose (gmcore_mod.F90:213-341): the global integrals, each a sequential
# sum in the reference's loop order
# ---------------------------------------------------------------------------
def seq(*blocks):
    """Sum of the blocks' elements one after another, in row-major order."""
    return float(np.cumsum(np.concatenate([np.ravel(b) for b in blocks]))[-1])


def diagnostics(cfg, o):
    nlat, nhalf = cfg.nlat, cfg.nlat - 1
    I = slice(1, nlat - 1)
    ac = o.metric("area_cell", nlat)[None, :, None]
    alon, alat = o.metric("area_lon", nlat)[None, :, None], o.metric("area_lat", nhalf)[None, :, None]
    avtx = o.metric("area_vtx", nhalf)[None, :, None]
    F = {n: o.get_field(n) for n in ("u_lon", "v_lat", "mfx_lon", "mfy_lat", "m", "pv", "pv_lon", "pv_lat", "gzs")}
    m = F["m"]
    m_lon, m_lat = ((m + nxt(m)) * 0.5)[:, I], (m[:, :-1] + m[:, 1:]) * 0.5
    nlev = m.shape[0]
    tm = seq(m * ac)
    ke_lon = F["mfx_lon"][:, I] * 0.5 * F["u_lon"][:, I] * alon[:, I] * 2
    ke_lat = F["mfy_lat"] * 0.5 * F["v_lat"] * alat * 2
    te_ke = seq(*[b for k in range(nlev) for b in (ke_lon[k], ke_lat[k])])
    if cfg.baroclinic:
        te_ie = seq(m * cfg.cpd * o.get_field("t") * ac)
        te_pe = seq(F["gzs"] * o.get_field("phs") * ac[0])
        tpt = seq(m * o.get_field("pt") * ac)
    else:
        te_ie, tpt = 0.0, 0.0
        m1 = m[0]
        te_pe = seq((m1 * m1 * cfg.g * 0.5 + m1 * F["gzs"]) * ac[0])
    tav = seq(F["pv"] * avtx)
    pe_lon = m_lon * (F["pv_lon"][:, I] * F["pv_lon"][:, I]) * 0.5 * alon[:, I]
    pe_lat = m_lat * (F["pv_lat"] * F["pv_lat"]) * 0.5 * alat
    tpe = seq(*[b for k in range(nlev) for b in (pe_lon[k], pe_lat[k])])
    return {"tm": tm, "te": te_ke + te_ie + te_pe, "te_ke": te_ke, "te_ie": te_ie, "te_pe": te_pe,
            "tav": tav, "tpe": tpe, "tpt": tpt}


@pytest.mark.parametrize("case", sorted(CASES))
def test_diagnostics_match_restatement(case):
    cfg = CASES[case]()
    o = prepared(cfg)
    try:
        got = o.diagnose()
        want = diagnostics(cfg, o)
        for name, w in want.items():
            if w == 0.0:
                continue
            assert abs(got[name] - w) <= 4 * np.finfo(float).eps * abs(w), (case, name, got[name], w)
    finally:
        o.close()


# ---------------------------------------------------------------------------
# divergence damping (div_damp_run, div_damp_mod.F90:89-139; calc_div with
# the order-4 Laplacian of divergence, operators_mod.F90:354-431)
# ---------------------------------------------------------------------------
def divergence_damping(cfg, o):
    nlat, nhalf, nlon, nlev = cfg.nlat, cfg.nlat - 1, cfg.nlon, cfg.nlev
    I = slice(1, nlat - 1)
    row = lambda n, rows: o.metric(n, rows)[None, :, None]
    le_lon, de_lon, ac = row("le_lon", nlat), row("de_lon", nlat), row("area_cell", nlat)
    le_lat, de_lat = row("le_lat", nhalf), row("de_lat", nhalf)
    fcos, hcos = row("full_cos_lat", nlat), row("half_cos_lat", nhalf)
    u, v = o.get_field("u_f"), o.get_field("v_f")
    div = np.zeros((nlev, nlat, nlon))
    div[:, I] = ((u[:, I] * le_lon[:, I] - prev(u[:, I]) * le_lon[:, I]) +
                 (v[:, 1:] * le_lat[:, 1:] - v[:, :-1] * le_lat[:, :-1])) / ac[:, I]
    div[:, 0] = (ring(v[:, 0]) * le_lat[0, 0, 0] / nlon / ac[0, 0, 0])[:, None]
    div[:, -1] = (ring(-v[:, -1]) * le_lat[0, -1, 0] / nlon / ac[0, -1, 0])[:, None]
    c_lon = o.metric("div_c_lon", nlev * nlat).reshape(nlev, nlat)[:, :, None]
    c_lat = o.metric("div_c_lat", nlev * nhalf).reshape(nlev, nhalf)[:, :, None]
    u_lon, v_lat = o.get_field("u_lon"), o.get_field("v_lat")
    if cfg.div_damp_order == 4:
        d = np.zeros_like(div)          # pole rows are never set
        dc = div[:, I]
        d[:, I] = ((nxt(dc) - 2 * dc + prev(dc)) / (de_lon[:, I] * de_lon[:, I]) +
                   ((div[:, 2:] - dc) * hcos[:, 1:] / de_lat[:, 1:] -
                    (dc - div[:, :-2]) * hcos[:, :-1] / de_lat[:, :-1]) / le_lon[:, I] / fcos[:, I])
        u_lon[:, I] = u_lon[:, I] - c_lon[:, I] * (nxt(d[:, I]) - d[:, I]) / de_lon[:, I]
        v_lat = v_lat - c_lat * (d[:, 1:] - d[:, :-1]) / de_lat
    else:
        u_lon[:, I] = u_lon[:, I] + c_lon[:, I] * (nxt(div[:, I]) - div[:, I]) / de_lon[:, I]
        v_lat = v_lat + c_lat * (div[:, 1:] - div[:, :-1]) / de_lat
    return {"u_lon": u_lon, "v_lat": v_lat}


@pytest.mark.parametrize("case", ["swm_order2", "baroclinic_order2", "baroclinic_order4", "swm_order4"])
def test_divergence_damping_matches_restatement(case):
    order = 4 if case.endswith("4") else 2
    kw = dict(use_div_damp=1, div_damp_order=order, div_damp_coef2=1.0 / 128, div_damp_coef4=0.01)
    cfg = swm_config(**kw) if case.startswith("swm") else baroclinic_config(**kw)
    o = prepared(cfg)
    try:
        before = {f: o.get_field(f) for f in ("u_lon", "v_lat")}
        want = divergence_damping(cfg, o)
        o.run_pass(2)
        for name, w in want.items():
            got = o.get_field(name)
            assert not np.array_equal(w, before[name]), name
            assert close(got, w), (case, name, float(np.abs(got - w).max() / np.abs(w).max()))
    finally:
        o.close()


# ---------------------------------------------------------------------------
# the other PV edge interpolations: midpoint (interp_pv_midpoint,
# operators_mod.F90:705-736), first-order upwind (:738-770; upwind1,
# upwind_mod.F90:14-25) and TVD with its three limiters (interp_pv_tvd,
# :797-832; tvd, flux limiters, tvd_mod.F90:83-102; eps the default-kind
# literal 1.0e-6, rounded to float32 and widened)
# ---------------------------------------------------------------------------
TVD_EPS = float(np.float32(1.0e-6))


def tvd(cfl, fm1, f, fp1, fp2, limiter):
    r = np.where(cfl > 0, (f - fm1 + TVD_EPS) / (fp1 - f + TVD_EPS), (fp2 - fp1 + TVD_EPS) / (fp1 - f + TVD_EPS))
    if limiter == 0:
        C = np.ones_like(r)
    elif limiter == 1:
        C = (r + np.abs(r)) / (1 + np.abs(r))
    else:
        C = np.maximum(0.0, np.minimum(np.minimum(2.0 * r, 0.5 * (1 + r)), 2.0))
    return 0.5 * (fp1 + f - ((1 - C) * np.copysign(1.0, cfl) + cfl * C) * (fp1 - f))


def pv_edges_variant(cfg, o, scheme):
    from gmcore_gb300 import abi
    nlat, nlon = cfg.nlat, cfg.nlon
    I = slice(1, nlat - 1)
    pv, u, v = o.get_field("pv"), o.get_field("u_f"), o.get_field("v_f")
    ut, vt = o.get_field("u_lat"), o.get_field("v_lon")[:, I]
    P = np.concatenate([np.roll(pv[:, :1], nlon // 2, axis=-1), pv, np.roll(pv[:, -1:], nlon // 2, axis=-1)], axis=1)
    jf = np.arange(1, nlat - 1)
    fy = [P[:, jf - 1], P[:, jf], P[:, jf + 1], P[:, jf + 2]]          # pv(j-2) .. pv(j+1) along a column
    fx = [np.roll(pv, 2, axis=-1), prev(pv), pv, nxt(pv)]             # pv(i-2) .. pv(i+1) along a row
    if scheme == "midpoint":
        return 0.5 * (fy[2] + fy[1]), 0.5 * (fx[1] + fx[2])
    if scheme == "upwind1":
        w = cfg.upwind_wgt_pv
        up1 = lambda f1, f2, sgn: 0.5 * (f2 + f1) + -0.5 * (f2 - f1) * w * sgn
        b_lon = np.abs(vt) / (np.sqrt(u[:, I] * u[:, I] + vt * vt) + EPS)
        b_lat = np.abs(ut) / (np.sqrt(ut * ut + v * v) + EPS)
        return (b_lon * up1(fy[1], fy[2], np.copysign(1.0, vt)) + (1 - b_lon) * 0.5 * (fy[1] + fy[2]),
                b_lat * up1(fx[1], fx[2], np.copysign(1.0, ut)) + (1 - b_lat) * 0.5 * (fx[1] + fx[2]))
    dt = cfg.dt_dyn
    lim = cfg.tvd_limiter_type
    cfl_lon = vt * dt / o.metric("le_lon", nlat)[None, I, None]
    cfl_lat = ut * dt / o.metric("le_lat", nlat - 1)[None, :, None]
    return tvd(cfl_lon, *fy, lim), tvd(cfl_lat, *fx, lim)


@pytest.mark.parametrize("scheme", ["midpoint", "upwind1", "tvd_none", "tvd_van_leer", "tvd_mc"])
def test_pv_edge_variants_match_restatement(scheme):
    from gmcore_gb300 import abi
    kw = {"midpoint": dict(pv_scheme=abi.PV_MIDPOINT), "upwind1": dict(pv_scheme=abi.PV_UPWIND, upwind_order_pv=1),
          "tvd_none": dict(pv_scheme=abi.PV_TVD, tvd_limiter_type=abi.TVD_NONE),
          "tvd_van_leer": dict(pv_scheme=abi.PV_TVD, tvd_limiter_type=abi.TVD_VAN_LEER),
          "tvd_mc": dict(pv_scheme=abi.PV_TVD, tvd_limiter_type=abi.TVD_MC)}[scheme]
    cfg = baroclinic_config(**kw)
    o = prepared(cfg)
    try:
        want_lon, want_lat = pv_edges_variant(cfg, o, scheme.split("_")[0] if scheme.startswith("tvd") else scheme)
        got_lon, got_lat = o.get_field("pv_lon")[:, 1:-1], o.get_field("pv_lat")
        assert close(got_lon, want_lon), (scheme, float(np.abs(got_lon - want_lon).max()))
        assert close(got_lat, want_lat), (scheme, float(np.abs(got_lat - want_lat).max()))
    finally:
        o.close()


# ---------------------------------------------------------------------------
# ffsl_flux_type = 'van_leer': the limited linear profile in place of the
# parabola (hflx_van_leer_cell, vflx_van_leer_cell, ffsl_mod.F90:556-658)
# ---------------------------------------------------------------------------
def hflx_van_leer(u, v, mx, my, cflx, cfly):
    nlat, nlon = mx.shape[1], mx.shape[-1]
    I = slice(1, nlat - 1)
    c = cflx[:, I]
    ci = np.trunc(c).astype(np.int64)
    cf = c - ci
    pos = c > 0
    fi = np.arange(1, nlon + 1)[None, None, :]
    cell = lambda m: np.take_along_axis(mx[:, I], (m - 1) % nlon, axis=-1)
    iu = np.where(pos, fi - ci, fi - ci + 1)
    first = np.where(pos, fi + 1 - ci, fi + 1)
    S = np.zeros_like(c)
    for t in range(int(np.abs(ci).max())):
        take = t < np.abs(ci)
        S = np.where(take, S + cell(np.where(take, first + t, 1)), S)
    dm = slope_mono(cell(iu - 1), cell(iu), cell(iu + 1))
    fx = np.zeros_like(mx)
    with np.errstate(divide="ignore", invalid="ignore"):
        fx[:, I] = np.where(c == 0, 0.0, np.where(
            pos, u[:, I] * (cf * (cell(iu) + dm * 0.5 * (1 - cf)) + S) / c,
            u[:, I] * (cf * (cell(iu) - dm * 0.5 * (1 + cf)) - S) / c))
    Y = lat_halo(my)                                    # full row r at index r + 1 (r = -1 .. nlat + 2)
    c = cfly
    pos = c > 0
    ju = np.where(pos, np.arange(1, nlat)[None, :, None], np.arange(2, nlat + 1)[None, :, None]) * np.ones_like(c, dtype=np.int64)
    row = lambda r: np.take_along_axis(Y, r + 1, axis=1)
    dm = slope_mono(row(ju - 1), row(ju), row(ju + 1))
    fy = v * (row(ju) + dm * 0.5 * (np.copysign(1.0, c) - c))
    return fx, fy


def vertical_flux_van_leer(g, we, cflz):
    nlev = g.shape[0] - 4
    lev = lambda k: np.take_along_axis(g, (k + 1)[None], axis=0)[0]
    flux = np.zeros_like(we)
    for k in range(2, nlev + 1):
        c, w = cflz[k - 1], we[k - 1]
        ci = np.trunc(c).astype(np.int64)
        cf = c - ci
        pos = c > 0
        ku = np.where(pos, k - ci - 1, k - ci)
        first = np.where(pos, k - ci, k)
        S = np.zeros_like(c)
        for t in range(int(np.abs(ci).max())):
            take = t < np.abs(ci)
            S = np.where(take, S + lev(np.where(take, first + t, k)), S)
        dm = slope_mono(lev(ku - 1), lev(ku), lev(ku + 1))
        with np.errstate(divide="ignore", invalid="ignore"):
            flux[k - 1] = np.where(c == 0, 0.0, np.where(pos, w * (cf * (lev(ku) + dm * 0.5 * (1 - cf)) + S) / c,
                                                         w * (cf * (lev(ku) - dm * 0.5 * (1 + cf)) - S) / c))
    return flux


@pytest.mark.parametrize("case", ["van_leer", "van_leer_long_step"])
def test_van_leer_flux_divergences_match_restatement(case):
    from gmcore_gb300 import abi
    long = case.endswith("long_step")
    cfg = baroclinic_config(ffsl_flux_type=abi.FLUX_VAN_LEER, **(dict(dt=1200.0) if long else {}))
    o = prepared(cfg, u_wave=60.0 if long else 0.0)
    try:
        o.run_pass(0)
        nlat, nlon, nlev = cfg.nlat, cfg.nlon, cfg.nlev
        le_lon, le_lat, area = (o.metric("le_lon", nlat)[None, :, None], o.metric("le_lat", nlat - 1)[None, :, None],
                                o.metric("area_cell", nlat)[None, :, None])
        I = slice(1, nlat - 1)
        B = {n: o.get_batch(n) for n in ("u", "v", "cflx", "cfly", "divx", "divy")}
        gx, gy = ffsl_fluxes(cfg, o, o.get_field("pt"), B, o.get_field("mfx_lon"), o.get_field("mfy_lat"),
                             cfg.dt_dyn, hflx=hflx_van_leer)
        want = {"dptfdlon": (gx[:, I] - prev(gx[:, I])) * le_lon[:, I] / area[:, I]}
        dlat = np.zeros((nlev, nlat, nlon))
        dlat[:, I] = (gy[:, 1:] * le_lat[:, 1:] - gy[:, :-1] * le_lat[:, :-1]) / area[:, I]
        dlat[:, 0] = (ring(gy[:, 0]) * le_lat[0, 0, 0] / nlon / area[0, 0, 0])[:, None]
        dlat[:, -1] = (ring(-gy[:, -1]) * le_lat[0, -1, 0] / nlon / area[0, -1, 0])[:, None]
        want["dptfdlat"] = dlat
        pt = o.get_field("pt")
        g = np.zeros((nlev + 4,) + pt.shape[1:])
        g[2:nlev + 2] = pt
        g[1] = 2 * g[2] - g[3]
        g[0] = 2 * g[1] - g[2]
        g[nlev + 2] = 2 * g[nlev + 1] - g[nlev]
        g[nlev + 3] = 2 * g[nlev + 2] - g[nlev + 1]
        flux = vertical_flux_van_leer(g, o.get_batch("we"), o.get_batch("cflz"))
        want["dptfdlev"] = flux[1:] - flux[:-1]
        for name, w in want.items():
            got = o.get_tend(0, name)
            if name == "dptfdlon":
                got = got[:, I]
            assert close(got, w), (case, name, float(np.abs(got - w).max() / np.abs(w).max()))
    finally:
        o.close()
