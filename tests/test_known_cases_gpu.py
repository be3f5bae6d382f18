"""GPU step (FP64 form) vs the FP64 oracle on the reference's analytic
states: the Rossby-Haurwitz wave and the zonal flow over a mountain in
shallow water (src/tests/swm/rossby_haurwitz_wave_test_mod.F90,
mountain_zonal_flow_test_mod.F90) and the perturbed baroclinic wave on the
26-level test coordinate (src/tests/baroclinic_wave_test_mod.F90).

Tolerances as for the seeded states: max-norm error <= 1e-12 after one step
and <= 1e-9 after a few hours.  Winds are measured against the wind scale
(the larger of max |u| and max |v|): the mountain flow and the baroclinic
wave start with v = 0, so their v after a step is small beside the round-off
that u carries."""
import numpy as np
import pytest

from gmcore_gb300 import Model
from oracle import Oracle

from cases import baroclinic_wave_state, mountain_zonal_flow, rossby_haurwitz, swm_state
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
