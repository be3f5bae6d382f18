"""Known-answer checks of the FP64 oracle and of the host-side grid set-up
(no GPU).  They pin the restatement with the reference's own invariants:
the area identities of debug_check_areas (src/utils/debug_mod.F90:33-111),
mass conservation of diagnose (gmcore_mod.F90:213-341), the steady
geostrophic flow test (tests/swm/steady_geostrophic_flow_test_mod.F90) with
the L1/L2 norms of tools/calc_errors.py, and the polar-filter halo width rule
(process_mod.F90:208-213)."""
import math

import numpy as np
import pytest

import gmcore_gb300 as g
from gmcore_gb300 import abi
from oracle import Oracle

from helpers import baroclinic_config, initial_state, load_state, swm_config


@pytest.mark.parametrize("nlon,nlat", [(360, 180), (72, 37), (720, 360)])
def test_area_identities(nlon, nlat):
    # debug_check_areas (src/utils/debug_mod.F90:33-111), same tolerances
    cfg = swm_config(nlon=nlon, nlat=nlat, dt=60.0)
    o = Oracle(cfg)
    R = cfg.radius
    total = 4 * math.pi * R * R
    nh = nlat - 1
    M = {n: o.metric(n, nlat) for n in ("area_cell", "area_subcell1", "area_subcell2", "area_lon",
                                        "area_lon_north", "area_lon_south")}
    M.update({n: o.metric(n, nh) for n in ("area_vtx", "area_lat", "area_lat_west", "area_lat_east")})
    assert abs(total - (M["area_cell"] * nlon).sum()) / total <= 1e-12
    assert abs(total - (M["area_vtx"] * nlon).sum()) / total <= 1e-12
    sub = M["area_subcell1"] + M["area_subcell2"]
    assert abs(total - (sub * nlon * 2).sum()) / total <= 1e-12
    assert np.all(np.abs(M["area_cell"] - 2 * sub) / M["area_cell"] <= 1e-12)
    vtx = 2 * (M["area_subcell2"][:-1] + M["area_subcell1"][1:])
    assert np.all(np.abs(M["area_vtx"] - vtx) / M["area_vtx"] <= 1e-12)
    inner = slice(1, nlat - 1)
    ns = M["area_lon_north"][inner] + M["area_lon_south"][inner]
    assert np.all(np.abs(ns - M["area_lon"][inner]) / M["area_lon"][inner] <= 1e-12)
    we = M["area_lat_west"] + M["area_lat_east"]
    assert np.all(np.abs(we - M["area_lat"]) / M["area_lat"] <= 1e-11)
    edge = (M["area_lon"][inner] * nlon).sum() + (M["area_lat"] * nlon).sum()
    assert abs(total - edge) / total <= 1e-9
    edge2 = (ns * nlon).sum() + (we * nlon).sum()
    assert abs(total - edge2) / total <= 1e-9


def test_host_metrics_match_analytic():
    cfg = swm_config(nlon=360, nlat=180, dt=60.0)
    R = cfg.radius
    dlon = 2 * math.pi / 360
    flat = g.mesh_metric(cfg, "full_lat")
    de_lon = g.mesh_metric(cfg, "de_lon")
    assert np.allclose(de_lon[1:-1], R * np.cos(flat[1:-1]) * dlon, rtol=1e-15)
    assert flat[0] == -math.pi / 2 and flat[-1] == math.pi / 2


@pytest.mark.parametrize("nlon,nlat,dt,expect", [(360, 180, 60.0, 17), (720, 360, 180.0, 189)])
def test_halo_width_rule(nlon, nlat, dt, expect):
    cfg = swm_config(nlon=nlon, nlat=nlat, dt=dt)
    taps = g.filter_taps(cfg, 0, 1)
    assert max(2, (taps.max() - 1) // 2) == expect


def test_steady_geostrophic_flow_stays_steady():
    # tests/swm/steady_geostrophic_flow_test_mod.F90 with alpha = 0
    cfg = swm_config(nlon=72, nlat=37, dt=600.0)
    o = Oracle(cfg)
    nlon, nlat = cfg.nlon, cfg.nlat
    R, om = cfg.radius, cfg.omega
    u0 = 2 * math.pi * R / (12 * 86400.0)
    gz0 = 2.94e4
    fcl, fsl = o.metric("full_cos_lat", nlat), o.metric("full_sin_lat", nlat)
    u = np.repeat((u0 * fcl)[:, None], nlon, axis=1)[None]
    gz = (gz0 - (R * om * u0 + u0 ** 2 * 0.5) * fsl[:, None] ** 2 * np.ones(nlon)[None, :])[None]
    o.set_field("u_lon", u)
    o.set_field("v_lat", np.zeros((1, nlat - 1, nlon)))
    o.set_field("gz", gz)
    o.set_field("gzs", np.zeros((nlat, nlon)))
    o.prepare()
    d0 = o.diagnose()
    o.step(144)   # one day
    d1 = o.diagnose()
    h0, h1 = gz[0], o.get_field("gz")[0]
    cl = np.cos(o.metric("full_lat", nlat))
    L1 = np.sum(np.sum(np.abs(h1 - h0), axis=1) * cl) / np.sum(np.sum(np.abs(h0), axis=1) * cl)
    L2 = np.sqrt(np.sum(np.sum((h1 - h0) ** 2, axis=1) * cl)) / np.sqrt(np.sum(np.sum(h0 ** 2, axis=1) * cl))
    assert L1 < 2e-4 and L2 < 2e-4, (L1, L2)
    assert abs(d1["tm"] - d0["tm"]) / d0["tm"] < 1e-13


@pytest.mark.parametrize("option", ["default", "tvd_pv", "van_leer_flux", "div_damp_4"])
def test_baroclinic_mass_conservation(option):
    """Total dry mass (diagnose tm, gmcore_mod.F90:234-240) is conserved to
    round-off by the default path and by each option off it."""
    from gmcore_gb300 import abi
    kw = {"default": {}, "tvd_pv": dict(pv_scheme=abi.PV_TVD, tvd_limiter_type=abi.TVD_MC),
          "van_leer_flux": dict(ffsl_flux_type=abi.FLUX_VAN_LEER),
          "div_damp_4": dict(use_div_damp=1, div_damp_order=4, div_damp_coef4=0.01)}[option]
    cfg = baroclinic_config(**kw)
    o = Oracle(cfg)
    load_state(o, initial_state(cfg))
    o.prepare()
    d0 = o.diagnose()
    # fourth-order damping with the reference's default coefficient is stable
    # only for a few steps at this 5 degree test resolution
    o.step(2 if option == "div_damp_4" else 6)
    d1 = o.diagnose()
    assert abs(d1["tm"] - d0["tm"]) / d0["tm"] < 1e-13


def test_baroclinic_rest_state_stays_at_rest():
    cfg = baroclinic_config(nlon=36, nlat=19)
    st = initial_state(cfg, noise_k=0.0)
    st["u_lon"][:] = 0.0
    st["phs"][:] = 1.0e5
    # isothermal 300 K column for uniform surface pressure
    o = Oracle(cfg)
    pt1 = np.ones_like(st["pt"])
    load_state(o, dict(st, pt=pt1))
    o.prepare()
    pl = o.get_field("ph_lev")[:, 0, 0]
    ph = 0.5 * (pl[:-1] + pl[1:])
    st["pt"] = 300.0 * (1e5 / ph[:, None, None]) ** (cfg.Rd / cfg.cpd) * np.ones_like(st["pt"])
    o = Oracle(cfg)
    load_state(o, st)
    o.prepare()
    o.step(5)
    assert np.abs(o.get_field("u_lon")).max() < 1e-10
    assert np.abs(o.get_field("v_lat")).max() < 1e-10


def test_tracer_mass_with_div_damp_and_cadence_runs():
    cfg = baroclinic_config(nlon=36, nlat=19, ntracer=1, use_div_damp=1, dt_adv=240.0)
    o = Oracle(cfg)
    load_state(o, initial_state(cfg))
    o.prepare()
    o.step(5)
    q = o.get_tracer(0)
    assert np.isfinite(q).all() and q.min() >= 0.0


def test_seeded_initial_state_is_deterministic():
    cfg = baroclinic_config(ntracer=2)
    a = g.make_ic(cfg, 2, 123, 1.0)
    b = g.make_ic(cfg, 2, 123, 1.0)
    c = g.make_ic(cfg, 2, 124, 1.0)
    for k in a:
        assert np.array_equal(a[k], b[k])
    assert not np.array_equal(a["pt"], c["pt"])
    # golden checksum of the generator (SplitMix64 + Box-Muller)
    assert abs(float(a["pt"].sum()) - float(b["pt"].sum())) == 0.0


@pytest.mark.parametrize("baroclinic", [False, True])
def test_space_operator_energy_identities(baroclinic):
    """debug_check_space_operators (debug_mod.F90:113-220): with the
    energy-conserving Coriolis scheme the Coriolis force does no work, the KE
    gradient's work cancels the KE flux divergence, mass and (baroclinic) pt
    flux divergences integrate to zero -- each to round-off relative to the sum
    of the magnitudes of its terms.  The non-conserving coriolis_scheme 2 must
    not satisfy the first identity."""
    from oracle import Oracle
    from helpers import baroclinic_config, initial_state, load_state, swm_config
    if baroclinic:
        cfg, steps = baroclinic_config(), 3
    else:
        cfg, steps = swm_config(), 0
    o = Oracle(cfg)
    load_state(o, initial_state(cfg))
    o.prepare()
    o.step(steps)
    r = o.space_identities()
    names = ("coriolis", "ke", "mass") + (("ptf",) if baroclinic else ())
    for name in names:
        val, scale = r[name]
        assert scale > 0, name
        assert abs(val) <= 1e-13 * scale, (name, val, scale)
    o.close()
    if baroclinic:
        cfg2 = baroclinic_config(coriolis_scheme=2)
        o = Oracle(cfg2)
        load_state(o, initial_state(cfg2))
        o.prepare()
        o.step(steps)
        val, scale = o.space_identities()["coriolis"]
        assert abs(val) > 1e-8 * scale
        o.close()


@pytest.mark.parametrize("pv_scheme", ["midpoint", "upwind1", "tvd"])
def test_coriolis_does_no_work_for_any_pv_interpolation(pv_scheme):
    """The energy-conserving Coriolis term (calc_coriolis scheme 1,
    operators_mod.F90:846-906) does no work whatever values the edge PV takes,
    so the identity of debug_check_space_operators holds for every
    interp_pv option (midpoint, first-order upwind, TVD with the van Leer
    limiter) and for the van Leer FFSL flux."""
    from oracle import Oracle
    from gmcore_gb300 import abi
    from helpers import baroclinic_config, initial_state, load_state
    kw = {"midpoint": dict(pv_scheme=abi.PV_MIDPOINT), "upwind1": dict(pv_scheme=abi.PV_UPWIND, upwind_order_pv=1),
          "tvd": dict(pv_scheme=abi.PV_TVD, tvd_limiter_type=abi.TVD_VAN_LEER,
                      ffsl_flux_type=abi.FLUX_VAN_LEER)}[pv_scheme]
    cfg = baroclinic_config(**kw)
    o = Oracle(cfg)
    load_state(o, initial_state(cfg))
    o.prepare()
    o.step(2)
    r = o.space_identities()
    for name in ("coriolis", "ke", "mass", "ptf"):
        val, scale = r[name]
        assert scale > 0, name
        assert abs(val) <= 1e-13 * scale, (pv_scheme, name, val, scale)
    o.close()


def test_openmp_build_matches_parity_build_with_tracers():
    """The OpenMP build of the oracle (the CPU baseline and the reference arm
    of the benchmark) copies tracers in and out level by level in parallel
    and must reproduce the parity build bit for bit, tracers included."""
    import os
    os.environ.setdefault("OMP_NUM_THREADS", "4")
    cfg = baroclinic_config(ntracer=2)
    st = initial_state(cfg)
    out = {}
    for variant in ("parity", "omp"):
        o = Oracle(cfg, variant=variant)
        load_state(o, st)
        for l in range(2):
            assert np.array_equal(o.get_tracer(l), st["q"][l]), (variant, l)
        o.prepare()
        o.step(4)
        out[variant] = [o.get_field(f) for f in ("u_lon", "v_lat", "pt", "phs")] + [o.get_tracer(l) for l in range(2)]
        o.close()
    for a, b in zip(out["parity"], out["omp"]):
        assert np.array_equal(a, b)
