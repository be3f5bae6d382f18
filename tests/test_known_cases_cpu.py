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

from cases import RH_R, RH_W, baroclinic_wave_state, mountain_zonal_flow, rossby_haurwitz
from helpers import baroclinic_config, load_state, swm_config

DAY = 86400.0


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


def test_mountain_zonal_flow_one_day():
    cfg, (_, _, _, gzs), s, d0, d1 = run_swm(144, 73, 300.0, mountain_zonal_flow)
    assert abs(d1["tm"] - d0["tm"]) / d0["tm"] < 1e-13
    assert abs(d1["te"] - d0["te"]) / d0["te"] < 5e-6
    depth = (s["gz"] - gzs) / cfg.g
    assert 3000.0 < depth.min() and depth.max() < 6100.0
    assert np.all(np.isfinite(s["u_lon"])) and np.abs(s["v_lat"]).max() < 40.0


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


def test_time_schemes_converge_to_one_solution():
    """euler, pc2 and wrfrk3 (time_schemes_mod.F90:244-288) advance the
    Rossby-Haurwitz wave for one hour with the polar filter off (its width
    depends on dt).  Each converges at first order in dt: every stage updates
    the winds with the pressure gradient of the mass the stage has just
    updated (step_forward_backward, :102-118), and that end-of-stage
    evaluation costs an order for all three.  All three converge to the same
    solution, which catches a stage that advances the wrong span of time."""
    from gmcore_gb300 import abi
    from cases import swm_state
    T = 3600.0
    run = {}
    for scheme in (abi.TIME_EULER, abi.TIME_PC2, abi.TIME_WRFRK3):
        for dt in (60.0, 30.0, 15.0):
            cfg = swm_config(dt=dt, time_scheme=scheme, max_wave_speed=0.0)
            o = Oracle(cfg)
            load_state(o, swm_state(cfg, rossby_haurwitz))
            o.prepare()
            o.step(int(round(T / dt)))
            run[scheme, dt] = np.concatenate([o.get_field(f).ravel() for f in ("u_lon", "v_lat")])
            o.close()
    diff = lambda a, b: float(np.abs(run[a] - run[b]).max())
    for scheme in (abi.TIME_EULER, abi.TIME_PC2, abi.TIME_WRFRK3):
        d60, d30 = diff((scheme, 60.0), (scheme, 30.0)), diff((scheme, 30.0), (scheme, 15.0))
        assert 1.8 < d60 / d30 < 2.2, (scheme, d60, d30)
    for scheme in (abi.TIME_PC2, abi.TIME_WRFRK3):
        e60, e30 = diff((scheme, 60.0), (abi.TIME_EULER, 60.0)), diff((scheme, 30.0), (abi.TIME_EULER, 30.0))
        assert 1.8 < e60 / e30 < 2.2, (scheme, e60, e30)
