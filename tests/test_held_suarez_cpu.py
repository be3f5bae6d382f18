"""The Held-Suarez test forcing of the oracle (test_case = 'held_suarez':
test_forcing_run after the integrator, gmcore_mod.F90:586; the forcing of
held_suarez_test_mod.F90:74-112) against a numpy restatement.  The forcing
acts on the new state after the dynamics of the step and before the tracer
and damping steps, so after one step the forced run equals the unforced run's
state with the forcing applied to it, bit for bit:

  u <- u - dt kv u  (rows 2 .. nlat-1),  v <- v - dt kv v,
  kv = kf max(0, (eta - sigma_b) / (1 - sigma_b)),
  pt <- pt - dt kt pt (1 - Teq / T),  kt = ka + (ks - ka) max(...) cos^4,
  Teq = max(200, (315 - 60 sin^2 - 10 ln(p/p0) cos^2) (p/p0)^kappa),

with the constants of held_suarez_test_mod.F90:18-24, p the full-level mean of
the half-level pressures and T the temperature of the unforced new state."""
import math

import numpy as np

from gmcore_gb300 import abi
from oracle import Oracle

from helpers import load_state

KF, KA, KS = 1.0 / 86400.0, 0.025 / 86400.0, 0.25 / 86400.0
SIG_B, DT_LAT, DPT_LEV, P0 = 0.7, 60.0, 10.0, 1.0e5


def config(forcing, dt=600.0):
    return abi.default_config(nlon=72, nlat=37, nlev=26, baroclinic=1, dt_dyn=dt,
                              vert_coord_template=abi.VCOORD_TEST_L26, time_scheme=abi.TIME_WRFRK3,
                              max_wave_speed=400.0, forcing=forcing)


def one_step(cfg, st):
    o = Oracle(cfg)
    load_state(o, st)
    o.prepare()
    o.step(1)
    out = {f: o.get_field(f) for f in ("u_lon", "v_lat", "pt", "t", "ph_lev", "phs")}
    eta = o.metric("full_lev", cfg.nlev)
    cos, sin = o.metric("full_cos_lat", cfg.nlat), o.metric("full_sin_lat", cfg.nlat)
    o.close()
    return out, eta, cos, sin


def test_forcing_after_one_step_equals_restatement():
    import gmcore_gb300 as g
    free_cfg = config(abi.FORCING_NONE)
    st = g.make_ic(free_cfg, 2, 11, 1.0)
    free, eta, cos, sin = one_step(free_cfg, st)
    hs_cfg = config(abi.FORCING_HELD_SUAREZ)
    forced, _, _, _ = one_step(hs_cfg, st)
    dt = hs_cfg.dt_dyn
    kappa = hs_cfg.Rd / hs_cfg.cpd
    nlev, nlat, nlon = hs_cfg.nlev, hs_cfg.nlat, hs_cfg.nlon
    u, v, pt, t = (free[k].copy() for k in ("u_lon", "v_lat", "pt", "t"))
    ph = 0.5 * (free["ph_lev"][:-1] + free["ph_lev"][1:])
    for k in range(nlev):
        sfac = max(0.0, (eta[k] - SIG_B) / (1.0 - SIG_B))
        kv = KF * sfac
        u[k, 1:nlat - 1] = u[k, 1:nlat - 1] - dt * kv * u[k, 1:nlat - 1]
        v[k] = v[k] - dt * kv * v[k]
        for j in range(nlat):
            c, s = cos[j], sin[j]
            c2 = c * c
            kt = KA + (KS - KA) * sfac * (c2 * c2)
            for i in range(nlon):
                p_p0 = ph[k, j, i] / P0
                teq = max(200.0, (315.0 - DT_LAT * (s * s) - DPT_LEV * math.log(p_p0) * c2) * math.pow(p_p0, kappa))
                pt[k, j, i] = pt[k, j, i] - dt * kt * pt[k, j, i] * (1.0 - teq / t[k, j, i])
    assert np.array_equal(forced["u_lon"], u)
    assert np.array_equal(forced["v_lat"], v)
    assert np.array_equal(forced["pt"], pt)
    assert np.array_equal(forced["phs"], free["phs"])   # the forcing leaves the mass alone
    # the friction acts only below sigma_b, the relaxation everywhere
    upper = eta < SIG_B
    assert np.array_equal(forced["u_lon"][upper], free["u_lon"][upper])
    assert not np.array_equal(forced["u_lon"][~upper], free["u_lon"][~upper])


def test_forcing_needs_the_baroclinic_model():
    import pytest
    from gmcore_gb300 import GmcError, Model
    cfg = abi.default_config(nlon=72, nlat=37, nlev=1, baroclinic=0, dt_dyn=600.0, forcing=abi.FORCING_HELD_SUAREZ)
    with pytest.raises(GmcError) as e:
        Model(cfg)
    assert e.value.code in (abi.GMC_EINVAL, abi.GMC_ECUDA)   # ECUDA first where no GPU exists
