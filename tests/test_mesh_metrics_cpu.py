"""The 1-D mesh metrics of the latitude-longitude C-grid against a separate
restatement of mesh_init_global (mesh_mod.F90:134-447, default options:
uniform latitudes, classic tangent weights):

* latitudes built by accumulating dlat from the south pole, snapped to 0
  within 1e-12 and mirrored for equatorial symmetry (:186-234), their sines
  and cosines with exact poles (:236-264);
* cell, sub-cell and vertex areas of the zonal strips (:266-283, 328);
* the areas of the triangles around each edge (:284-370).  The reference
  sums spherical angles in binary128 (calc_area, sphere_geometry_mod.F90:
  305-326); here each spherical excess is computed in 40-digit arithmetic by
  a different formula (Van Oosterom and Strackee's tan(E/2)) on the same
  vertices (x, y from double-precision sines and cosines multiplied in
  extended precision, z a double product, as cartesian_transform_1_r16
  forms them, :110-123).  Two properties of the reference's arithmetic are
  kept because they show at 1e-12: calc_area subtracts (n - 2) pi with the
  double-precision pi, so every triangle area carries R^2 (pi - pi_double);
  and the lune of a latitude arc (calc_area_with_last_small_arc, :328-390)
  is the polar sector minus the polar triangle, with the sector's longitude
  span from the vertices' recovered longitudes (atan2 of their coordinates)
  and its latitude sine z / R;
* edge lengths and distances (:372-391), classic tangent weights
  (:417-426) and Coriolis parameters (:436-441).

Closed forms must agree to 4 ulps, the triangle areas and what depends on
them to 1e-14 (measured: all 30 tables bit for bit at 5, 1 and 0.5
degrees)."""
import math

import numpy as np
import pytest

from oracle import Oracle

from helpers import swm_config

mpmath = pytest.importorskip("mpmath")
mp = mpmath.mp

PI = math.atan(1.0) * 4.0
PI2, PI05 = PI * 2, PI * 0.5
DEG = 180.0 / PI


def latitudes(nlat):
    """(full, half, full_deg, half_deg) latitudes."""
    nhalf = nlat - 1
    dlat = (PI05 - (-PI05)) / nhalf
    full, half = np.zeros(nlat), np.zeros(nhalf)
    full_deg, half_deg = np.zeros(nlat), np.zeros(nhalf)
    full[0], full_deg[0] = -PI05, -PI05 * DEG
    for j in range(1, nlat - 1):
        full[j] = full[j - 1] + dlat
        if abs(full[j]) < 1e-12:
            full[j] = 0.0
        full_deg[j] = full[j] * DEG
    full[-1], full_deg[-1] = PI05, PI05 * DEG
    for j in range(nhalf):
        half[j] = full[j] + 0.5 * dlat
        if abs(half[j]) < 1e-12:
            half[j] = 0.0
        half_deg[j] = half[j] * DEG
    for a, d in ((full, full_deg), (half, half_deg)):
        n = len(a)
        for j in range(n):
            if a[j] > 0:
                a[j] = -a[n - 1 - j]
                d[j] = -d[n - 1 - j]
    return full, half, full_deg, half_deg


def point(R, lon, lat):
    c = mpmath.mpf(math.cos(lat))
    return [mpmath.mpf(R) * c * mpmath.mpf(math.cos(lon)), mpmath.mpf(R) * c * mpmath.mpf(math.sin(lon)),
            mpmath.mpf(R * math.sin(lat))]


def unit(v):
    n = mpmath.sqrt(sum(x * x for x in v))
    return [x / n for x in v]


def great_triangle(R, a, b, c):
    """calc_area of the great-circle triangle abc: R^2 (E + pi - pi_double),
    the spherical excess E by Van Oosterom and Strackee."""
    a, b, c = unit(a), unit(b), unit(c)
    dot = lambda p, q: sum(x * y for x, y in zip(p, q))
    cross = [b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0]]
    num = abs(dot(a, cross))
    den = 1 + dot(a, b) + dot(b, c) + dot(c, a)
    excess = 2 * mpmath.atan2(num, den)
    return mpmath.mpf(R * R) * (excess + mpmath.pi - mpmath.mpf(PI))


def lon_lat(R, p):
    lon = mpmath.atan2(p[1], p[0])
    if lon < 0:
        lon += mpmath.mpf(PI2)
    return lon, mpmath.asin(p[2] / mpmath.mpf(R))


def triangle_with_latitude_arc(R, p0, p1, p2):
    """Area bounded by great arcs p0-p1, p0-p2 and the latitude arc p1-p2."""
    tri = great_triangle(R, p0, p1, p2)
    (_, lat0), (lon1, lat1), (lon2, _) = lon_lat(R, p0), lon_lat(R, p1), lon_lat(R, p2)
    if lat1 == 0:
        return tri
    dlon = lon2 - lon1 if lat0 > lat1 else lon1 - lon2
    if dlon < 0:
        dlon += mpmath.mpf(PI2)
    s1 = p1[2] / mpmath.mpf(R)
    poleward = lat0 * lat1 >= 0 and abs(lat0) > abs(lat1)
    q1, q2 = (p1, p2) if poleward else (p2, p1)
    pole = [0, 0, mpmath.mpf(R) if lat1 > 0 else -mpmath.mpf(R)]
    sector = mpmath.mpf(R * R) * dlon * ((1 - s1) if lat1 > 0 else (s1 + 1))
    lune = sector - great_triangle(R, pole, q1, q2)
    if lune < 0 and -lune > 1e-10:
        lune = 0
    return tri + lune if poleward else tri - lune


def restated(cfg):
    nlon, nlat = cfg.nlon, cfg.nlat
    nhalf = nlat - 1
    R, om = cfg.radius, cfg.omega
    mp.dps = 40
    dlon = (PI2 - 0.0) / nlon
    flon = [i * dlon for i in range(3)]
    hlon = [x + 0.5 * dlon for x in flon]
    full, half, full_deg, half_deg = latitudes(nlat)
    fc, fs = np.cos(full), np.sin(full)
    hc, hs = np.cos(half), np.sin(half)
    fc[0], fs[0], fc[-1], fs[-1] = 0.0, -1.0, 0.0, 1.0
    M = {n: np.zeros(nlat) for n in ("area_cell", "area_subcell1", "area_subcell2", "area_lon_west", "area_lon_east",
                                     "area_lon", "area_lon_north", "area_lon_south", "de_lon", "le_lon",
                                     "full_tangent_wgt1", "full_tangent_wgt2", "full_f")}
    M.update({n: np.zeros(nhalf) for n in ("area_vtx", "area_lat_west", "area_lat_east", "area_lat_north",
                                          "area_lat_south", "area_lat", "le_lat", "de_lat", "half_tangent_wgt1",
                                          "half_tangent_wgt2", "half_f")})
    for j in range(nlat):
        if j == 0:
            M["area_cell"][j] = R * R * dlon * (hs[j] + 1.0)
            M["area_subcell2"][j] = R * R * 0.5 * dlon * (hs[j] + 1.0)
        elif j == nlat - 1:
            M["area_cell"][j] = R * R * dlon * (1.0 - hs[j - 1])
            M["area_subcell1"][j] = R * R * 0.5 * dlon * (1.0 - hs[j - 1])
        else:
            M["area_cell"][j] = R * R * dlon * (hs[j] - hs[j - 1])
            M["area_subcell1"][j] = R * R * 0.5 * dlon * (fs[j] - hs[j - 1])
            M["area_subcell2"][j] = R * R * 0.5 * dlon * (hs[j] - fs[j])
            w = great_triangle(R, point(R, flon[0], full[j]), point(R, hlon[0], half[j - 1]),
                               point(R, hlon[0], half[j]))
            M["area_lon_west"][j] = M["area_lon_east"][j] = float(w)
            M["area_lon"][j] = M["area_lon_west"][j] + M["area_lon_east"][j]
            M["area_lon_north"][j] = float(triangle_with_latitude_arc(
                R, point(R, hlon[0], half[j]), point(R, flon[0], full[j]), point(R, flon[1], full[j])))
            M["area_lon_south"][j] = float(triangle_with_latitude_arc(
                R, point(R, hlon[0], half[j - 1]), point(R, flon[1], full[j]), point(R, flon[0], full[j])))
    for j in range(nhalf):
        M["area_vtx"][j] = R * R * dlon * (fs[j + 1] - fs[j])
        w = great_triangle(R, point(R, hlon[0], half[j]), point(R, flon[1], full[j]), point(R, flon[1], full[j + 1]))
        M["area_lat_west"][j] = M["area_lat_east"][j] = float(w)
        M["area_lat_north"][j] = float(triangle_with_latitude_arc(
            R, point(R, flon[1], full[j + 1]), point(R, hlon[0], half[j]), point(R, hlon[1], half[j])))
        M["area_lat_south"][j] = float(triangle_with_latitude_arc(
            R, point(R, flon[1], full[j]), point(R, hlon[1], half[j]), point(R, hlon[0], half[j])))
        if j == 0:
            M["area_lat_south"][j] = M["area_cell"][j]
        elif j + 1 == nlat - 1:
            M["area_lat_north"][j] = M["area_cell"][j + 1]
        M["area_lat"][j] = M["area_lat_north"][j] + M["area_lat_south"][j]
    for j in range(1, nlat - 1):
        M["de_lon"][j] = R * fc[j] * dlon
        M["le_lon"][j] = 2.0 * M["area_lon"][j] / M["de_lon"][j]
    for j in range(nhalf):
        M["le_lat"][j] = R * hc[j] * dlon
        M["de_lat"][j] = 2.0 * M["area_lat"][j] / M["le_lat"][j]
    # rows the scheme does not set keep the allocation fill, huge(1.0_r8)
    # (const_mod.F90:18, mesh_mod.F90:656)
    M["full_tangent_wgt1"][[0, -1]] = M["full_tangent_wgt2"][[0, -1]] = np.finfo(float).max
    for j in range(1, nlat - 1):
        M["full_tangent_wgt1"][j] = M["le_lat"][j - 1] / M["de_lon"][j] * 0.25
        M["full_tangent_wgt2"][j] = M["le_lat"][j] / M["de_lon"][j] * 0.25
    for j in range(nhalf):
        M["half_tangent_wgt1"][j] = M["le_lon"][j] / M["de_lat"][j] * 0.25
        M["half_tangent_wgt2"][j] = M["le_lon"][j + 1] / M["de_lat"][j] * 0.25
    M["full_f"] = 2.0 * om * fs
    M["half_f"] = 2.0 * om * hs
    M.update(full_lat=full, half_lat=half, full_cos_lat=fc, full_sin_lat=fs, half_cos_lat=hc, half_sin_lat=hs,
             full_lat_deg=full_deg, half_lat_deg=half_deg)
    return M


CLOSED = {"full_lat", "half_lat", "full_lat_deg", "half_lat_deg", "full_cos_lat", "full_sin_lat", "half_cos_lat", "half_sin_lat", "area_cell",
          "area_subcell1", "area_subcell2", "area_vtx", "de_lon", "le_lat", "full_f", "half_f"}


@pytest.mark.parametrize("nlon,nlat", [(72, 37), (360, 180), (720, 360)])
def test_mesh_metrics_match_restatement(nlon, nlat):
    cfg = swm_config(nlon=nlon, nlat=nlat, dt=60.0)
    want = restated(cfg)
    o = Oracle(cfg)
    try:
        for name, w in sorted(want.items()):
            got = o.metric(name, len(w))
            fill = w == np.finfo(float).max
            assert np.array_equal(got[fill], w[fill]), name
            got, w = got[~fill], w[~fill]
            scale = np.abs(w).max()
            err = float(np.abs(got - w).max() / scale)
            tol = 4 * np.finfo(float).eps if name in CLOSED else 1e-14
            assert err <= tol, (name, err)
    finally:
        o.close()


# Coefficient tables derived from the mesh.

def lon_damp_weights(deg_rows, lat0, interior):
    """lon_damp_init (lon_damp_mod.F90:43-68): exp((lat0 - |lat|)^2 ln(1e-3)
    / (lat0 - 80)^2), zero below 1e-6."""
    w = np.zeros(len(deg_rows))
    for j in interior:
        d, c = lat0 - abs(deg_rows[j]), lat0 - 80.0
        x = math.exp(d * d * math.log(1.0e-3) / (c * c))   # Fortran x**2 is x*x
        w[j] = 0.0 if x < 1.0e-6 else x
    return w


def test_zonal_smoother_weights_match_restatement():
    cfg = swm_config(nlon=720, nlat=360, dt=180.0)
    full, half, full_deg, half_deg = latitudes(cfg.nlat)
    o = Oracle(cfg)
    try:
        got_f = o.metric("lon_damp_wgt_full", cfg.nlat)
        got_h = o.metric("lon_damp_wgt_half", cfg.nlat - 1)
    finally:
        o.close()
    want_f = lon_damp_weights(full_deg, -full_deg[1], range(1, cfg.nlat - 1))
    want_h = lon_damp_weights(half_deg, -half_deg[0], range(cfg.nlat - 1))
    assert np.count_nonzero(want_f) > 0 and np.count_nonzero(want_h) > 0
    assert np.array_equal(got_f, want_f) and np.array_equal(got_h, want_h)


def div_damp_tables(cfg, o, M):
    """div_damp_init (div_damp_mod.F90:27-80) with the reference's pressures:
    vert_coord_calc_ph(k, p0) = hyam (p0_hybrid - ptop_local) + hybm (p0 -
    ptop_local) + ptop_local (hybrid_coord_mod.F90:146-152), where test_l26
    keeps ptop_local = 0 and resets the namelist ptop to p0_hybrid hyai(1)
    (hybrid_coord_test_mod.F90:145) and the wrf templates set ptop_local =
    ptop (hybrid_coord_mod.F90:78-90)."""
    nlat, nhalf, nlev = cfg.nlat, cfg.nlat - 1, cfg.nlev
    c_lon, c_lat = np.zeros((nlev, nlat)), np.zeros((nlev, nhalf))
    amp = np.ones(nlev)
    if cfg.baroclinic:
        hyai, hyam, hybm = o.metric("hyai", nlev + 1), o.metric("hyam", nlev), o.metric("hybm", nlev)
        test_l26 = cfg.vert_coord_template == 26
        local_ptop = 0.0 if test_l26 else cfg.ptop
        ptop = cfg.hybrid_coord_p0 * hyai[0] if test_l26 else cfg.ptop
        for k in range(nlev):
            ph = hyam[k] * (cfg.hybrid_coord_p0 - local_ptop) + hybm[k] * (cfg.p0 - local_ptop) + local_ptop
            amp[k] = max(1.0, 8 * (1 + math.tanh(math.log(ptop / ph))))
    for k in range(nlev):
        for j in range(1, nlat - 1):
            le, de = M["le_lon"][j], M["de_lon"][j]
            if cfg.div_damp_order == 4:
                c_lon[k, j] = cfg.div_damp_coef4 * (le * le) * (de * de)
            elif cfg.baroclinic:
                c_lon[k, j] = cfg.div_damp_coef2 * amp[k] * le * de
            else:
                c_lon[k, j] = cfg.div_damp_coef2 * le * de
        for j in range(nhalf):
            le, de = M["le_lat"][j], M["de_lat"][j]
            if cfg.div_damp_order == 4:
                c_lat[k, j] = cfg.div_damp_coef4 * (le * le) * (de * de)
            elif cfg.baroclinic:
                c_lat[k, j] = cfg.div_damp_coef2 * amp[k] * le * de
            else:
                c_lat[k, j] = cfg.div_damp_coef2 * le * de
    return c_lon, c_lat, amp


@pytest.mark.parametrize("case", ["swm_order2", "test_l26_order2", "wrf_l32_order2", "test_l26_order4"])
def test_divergence_damping_coefficients_match_restatement(case):
    from helpers import baroclinic_config
    kw = dict(use_div_damp=1, div_damp_order=4 if case.endswith("4") else 2, div_damp_coef2=1.0 / 128,
              div_damp_coef4=0.01)
    if case == "swm_order2":
        cfg = swm_config(nlon=72, nlat=37, dt=600.0, **kw)
    else:
        cfg = baroclinic_config(nlon=72, nlat=37, nlev=32 if "l32" in case else 26, dt=600.0, **kw)
    M = restated(cfg)
    o = Oracle(cfg)
    try:
        want_lon, want_lat, amp = div_damp_tables(cfg, o, M)
        got_lon = o.metric("div_c_lon", cfg.nlev * cfg.nlat).reshape(cfg.nlev, cfg.nlat)
        got_lat = o.metric("div_c_lat", cfg.nlev * (cfg.nlat - 1)).reshape(cfg.nlev, cfg.nlat - 1)
    finally:
        o.close()
    if case.endswith("order2") and case != "swm_order2":
        assert amp.max() > 1.0   # the upper levels are amplified
    for got, want in ((got_lon, want_lon), (got_lat, want_lat)):
        err = np.abs(got - want).max() / np.abs(want).max()
        assert err <= 4 * np.finfo(float).eps, (case, err)


@pytest.mark.parametrize("nlon,nlat", [(72, 37), (360, 180)])
def test_library_host_tables_match_restatement(nlon, nlat):
    """The library's own host entry points (gmc_mesh_metric, gmc_filter_taps,
    which build the grid from the library's normalised configuration) give
    the restated tables and the oracle's tap counts."""
    import gmcore_gb300 as g
    cfg = swm_config(nlon=nlon, nlat=nlat, dt=60.0)
    want = restated(cfg)
    for name, w in sorted(want.items()):
        got = g.mesh_metric(cfg, name)
        fill = w == np.finfo(float).max
        assert np.array_equal(got[fill], w[fill]), name
        assert np.array_equal(got[~fill], w[~fill]), name
    o = Oracle(cfg)
    try:
        for which in (0, 1, 2):
            for lat in (0, 1):
                assert np.array_equal(g.filter_taps(cfg, which, lat), o.filter_taps(which, lat)), (which, lat)
    finally:
        o.close()
