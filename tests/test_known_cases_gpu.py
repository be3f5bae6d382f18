"""GPU step (FP64 form) vs the FP64 oracle on the reference's analytic
states: the Rossby-Haurwitz wave and the zonal flow over a mountain in
shallow water (src/tests/swm/rossby_haurwitz_wave_test_mod.F90,
mountain_zonal_flow_test_mod.F90) and the perturbed baroclinic wave on the
26-level test coordinate (src/tests/baroclinic_wave_test_mod.F90); and the
FFSL operator entry point (gmc_ffsl_hflx) driving the reference's advection
tests for a whole 12-day period (src/tests/adv/solid_rotation_test_mod.F90,
deform_test_mod.F90 case 2) against the same transport driven by the
oracle's fluxes.

Tolerances as for the seeded states: max-norm error <= 1e-12 after one step
and <= 1e-9 after a few hours.  Winds are measured against the wind scale
(the larger of max |u| and max |v|): the mountain flow and the baroclinic
wave start with v = 0, so their v after a step is small beside the round-off
that u carries."""
import numpy as np
import pytest

from gmcore_gb300 import Model
from oracle import Oracle

from cases import (baroclinic_wave_state, deformational_flow, mountain_zonal_flow, rossby_haurwitz,
                   solid_rotation, swm_state, transport_config)
from helpers import baroclinic_config, load_state, swm_config

pytestmark = pytest.mark.gpu

WINDS = {"u_lon", "v_lat", "u_f", "v_f"}


def errors(gpu, orc, fields):
    ref = {f: orc.get_field(f) for f in fields}
    wind = max(float(np.abs(ref[f]).max()) for f in fields if f in WINDS)
    out = {}
    for f in fields:
        scale = wind if f in WINDS else float(np.abs(ref[f]).max())
        out[f] = float(np.abs(gpu.get_field(f) - ref[f]).max()) / scale
    return out


def check_pair(cfg, st, fields, nsteps):
    orc = Oracle(cfg)
    gpu = Model(cfg)
    try:
        for obj in (orc, gpu):
            load_state(obj, st)
            obj.prepare()
            obj.step(1)
        e1 = errors(gpu, orc, fields)
        orc.step(nsteps - 1)
        gpu.step(nsteps - 1)
        en = errors(gpu, orc, fields)
    finally:
        gpu.close()
        orc.close()
    print(cfg.nlon, cfg.nlat, cfg.nlev, "1 step", e1, nsteps, "steps", en)
    assert max(e1.values()) <= 1e-12, e1
    assert max(en.values()) <= 1e-9, en


@pytest.mark.parametrize("ic", [rossby_haurwitz, mountain_zonal_flow], ids=["rossby_haurwitz", "mountain"])
def test_swm_case_matches_oracle(ic):
    cfg = swm_config(nlon=144, nlat=73, dt=300.0)
    check_pair(cfg, swm_state(cfg, ic), ("u_lon", "v_lat", "gz"), 48)


def test_baroclinic_wave_matches_oracle():
    cfg = baroclinic_config(nlon=72, nlat=37, nlev=26, dt=600.0)
    check_pair(cfg, baroclinic_wave_state(cfg, perturb=True), ("u_lon", "v_lat", "pt", "phs"), 12)


def device_flux(model):
    """flux(q, wind, dt) through gmc_ffsl_hflx on device buffers."""
    import torch

    def flux(q1, wind, dt):
        names = ("q", "u", "v", "mfx", "mfy", "cflx", "cfly", "divx", "divy")
        dev = {k: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
               for k, a in zip(names, (q1, *wind))}
        qmfx = torch.zeros_like(dev["q"])
        qmfy = torch.zeros_like(dev["v"])
        torch.cuda.synchronize()
        ptrs = {k: t.data_ptr() for k, t in dev.items()}
        ptrs.update(qmfx=qmfx.data_ptr(), qmfy=qmfy.data_ptr())
        model.ffsl_hflx(ptrs, dt)
        return qmfx.cpu().numpy(), qmfy.cpu().numpy()
    return flux


@pytest.mark.parametrize("case", [solid_rotation, deformational_flow], ids=["solid_rotation", "deformational_flow"])
def test_ffsl_transport_period_matches_oracle(case):
    pytest.importorskip("torch")
    nlon, nlat, dt = 72, 37, 3600.0
    model = Model(transport_config(nlon, nlat, dt))
    try:
        tr, qg, q0 = case(nlon, nlat, dt, flux=device_flux(model))
    finally:
        model.close()
    _, qo, _ = case(nlon, nlat, dt)
    err = [float(np.abs(qg[l] - qo[l]).max() / np.abs(qo[l]).max()) for l in range(len(qo))]
    mass = [tr.mass_change(qg[l], q0[l]) for l in range(len(qo))]
    print(case.__name__, "max-norm vs oracle after one period", err, "mass", mass)
    assert max(err) <= 1e-9, err
    assert max(mass) < 1e-12, mass
