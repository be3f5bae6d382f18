"""Smagorinsky damping of the oracle (use_smag_damp: damp_run,
damp_mod.F90:59-61; smag_damp_run, smag_damp_mod.F90:52-190) against a numpy
restatement.  The damping acts on the new state after the integrator and
before the tracer step, which leaves u and v alone, so after one step the
damped run's winds equal the undamped run's with the damping applied to them,
bit for bit: tension at cells (rows 2 .. nlat-1, zero on the pole rows the
reference never writes), shear at vertices, eddy viscosities at the u and v
points from the four values around them, and the viscous tendencies (only the
zonal term on the two half rows next to the poles)."""
import numpy as np

from gmcore_gb300 import abi
from oracle import Oracle

from helpers import load_state


def config(smag, coef=0.1):
    return abi.default_config(nlon=72, nlat=37, nlev=26, baroclinic=1, dt_dyn=600.0,
                              vert_coord_template=abi.VCOORD_TEST_L26, time_scheme=abi.TIME_WRFRK3,
                              max_wave_speed=400.0, use_smag_damp=smag, smag_damp_coef=coef)


def one_step(cfg, st):
    o = Oracle(cfg)
    load_state(o, st)
    o.prepare()
    o.step(1)
    out = {f: o.get_field(f) for f in ("u_lon", "v_lat", "pt", "phs")}
    nlat, nh = cfg.nlat, cfg.nlat - 1
    met = {n: o.metric(n, nlat) for n in ("de_lon", "le_lon", "full_cos_lat")}
    met.update({n: o.metric(n, nh) for n in ("de_lat", "le_lat", "half_cos_lat")})
    o.close()
    return out, met


def smag(u, v, m, coef, dt):
    """smag_damp_run restated; rows are 1-based in the comments, arrays 0-based."""
    nlev, nlat, nlon = u.shape
    nh = nlat - 1
    dx, ly, fc = m["de_lon"], m["le_lon"], m["full_cos_lat"]
    dy, lx, hc = m["de_lat"], m["le_lat"], m["half_cos_lat"]
    east = lambda a: np.roll(a, -1, axis=-1)
    west = lambda a: np.roll(a, 1, axis=-1)
    st = np.zeros_like(u)   # pole rows stay zero
    ss = np.zeros_like(v)
    for j in range(1, nlat - 1):   # full rows 2 .. nlat-1
        st[:, j] = (u[:, j] - west(u[:, j])) / dx[j] - (v[:, j] * hc[j] - v[:, j - 1] * hc[j - 1]) / ly[j] / fc[j]
    for j in range(nh):            # half rows 1 .. nhalf, between full rows j, j+1
        ss[:, j] = (east(v[:, j]) - v[:, j]) / lx[j] + (u[:, j + 1] * fc[j + 1] - u[:, j] * fc[j]) / dy[j] / hc[j]
    un, vn = u.copy(), v.copy()
    for j in range(1, nlat - 1):
        ls2 = coef / (1 / (dx[j] * dx[j]) + 1 / (ly[j] * ly[j])) * 1.0
        kmh = ls2 * np.sqrt(0.5 * (st[:, j] * st[:, j] + east(st[:, j]) * east(st[:, j])) +
                            0.5 * (ss[:, j] * ss[:, j] + ss[:, j - 1] * ss[:, j - 1]))
        du = kmh * ((west(u[:, j]) - 2 * u[:, j] + east(u[:, j])) / (dx[j] * dx[j]) +
                    ((u[:, j + 1] - u[:, j]) / dy[j] * hc[j] - (u[:, j] - u[:, j - 1]) / dy[j - 1] * hc[j - 1]) /
                    ly[j] / fc[j])
        un[:, j] = u[:, j] + dt * du
    for j in range(nh):
        ls2 = coef / (1 / (lx[j] * lx[j]) + 1 / (dy[j] * dy[j])) * 1.0
        kmh = ls2 * np.sqrt(0.5 * (st[:, j] * st[:, j] + st[:, j + 1] * st[:, j + 1]) +
                            0.5 * (ss[:, j] * ss[:, j] + west(ss[:, j]) * west(ss[:, j])))
        t = (west(v[:, j]) - 2 * v[:, j] + east(v[:, j])) / (lx[j] * lx[j])
        if 0 < j < nh - 1:
            t = t + ((v[:, j + 1] - v[:, j]) / ly[j + 1] * fc[j + 1] - (v[:, j] - v[:, j - 1]) / ly[j] * fc[j]) / dy[j] / hc[j]
        vn[:, j] = v[:, j] + dt * (kmh * t)
    return un, vn


def test_damping_after_one_step_equals_restatement():
    import gmcore_gb300 as g
    st = g.make_ic(config(0), 2, 13, 1.0)
    free, met = one_step(config(0), st)
    damped, _ = one_step(config(1, 0.2), st)
    u, v = smag(free["u_lon"], free["v_lat"], met, 0.2, 600.0)
    assert np.array_equal(damped["u_lon"], u)
    assert np.array_equal(damped["v_lat"], v)
    assert np.array_equal(damped["pt"], free["pt"]) and np.array_equal(damped["phs"], free["phs"])
    assert not np.array_equal(damped["u_lon"], free["u_lon"])
