"""Reference namelist options off the default path, GPU vs the FP64 oracle:
pv_scheme = 'tvd' with each tvd_limiter_type (interp_pv_tvd,
operators_mod.F90:797-832; tvd_mod.F90:44-84), ffsl_flux_type = 'van_leer'
(hflx/vflx_van_leer_cell, ffsl_mod.F90:556-658) and fourth-order divergence
damping (div_damp_mod.F90:65-76, 120-136; calc_div div2,
operators_mod.F90:412-425).

Tolerances as in the default-path parity tests: FP64 max-norm error relative
to the field maximum <= 1e-12 after one step, <= 1e-10 after several; the
mixed form within the mixed-form tolerances of the default path.
"""
import pytest

from gmcore_gb300 import Model, abi
from oracle import Oracle

from helpers import BC_FIELDS, SWM_FIELDS, baroclinic_config, compare, initial_state, load_state, rel_err, swm_config

pytestmark = pytest.mark.gpu


def run_pair(cfg, nsteps, cfg_gpu=None, seed=7):
    st = initial_state(cfg, seed)
    orc = Oracle(cfg)
    load_state(orc, st)
    orc.prepare()
    gpu = Model(cfg_gpu or cfg)
    load_state(gpu, st)
    gpu.prepare()
    orc.step(nsteps)
    gpu.step(nsteps)
    return gpu, orc


@pytest.mark.parametrize("limiter", [abi.TVD_NONE, abi.TVD_VAN_LEER, abi.TVD_MC])
def test_tvd_pv_shallow_water(limiter):
    cfg = swm_config(pv_scheme=abi.PV_TVD, tvd_limiter_type=limiter)
    gpu, orc = run_pair(cfg, 1)
    e1 = compare(gpu, orc, SWM_FIELDS)
    orc.step(9)
    gpu.step(9)
    e10 = compare(gpu, orc, SWM_FIELDS)
    print("tvd swm limiter", limiter, max(e1.values()), max(e10.values()))
    assert max(e1.values()) <= 1e-12, e1
    assert max(e10.values()) <= 1e-10, e10


@pytest.mark.parametrize("limiter", [abi.TVD_VAN_LEER, abi.TVD_MC])
def test_tvd_pv_baroclinic(limiter):
    cfg = baroclinic_config(pv_scheme=abi.PV_TVD, tvd_limiter_type=limiter)
    gpu, orc = run_pair(cfg, 1)
    e1 = compare(gpu, orc, BC_FIELDS)
    orc.step(4)
    gpu.step(4)
    e5 = compare(gpu, orc, BC_FIELDS)
    print("tvd baroclinic limiter", limiter, max(e1.values()), max(e5.values()))
    assert max(e1.values()) <= 1e-12, e1
    assert max(e5.values()) <= 1e-10, e5


@pytest.mark.parametrize("limiter", [abi.LIMITER_MONO, abi.LIMITER_PD, abi.LIMITER_NONE])
def test_van_leer_flux(limiter):
    cfg = baroclinic_config(ffsl_flux_type=abi.FLUX_VAN_LEER, limiter_type=limiter, ntracer=2, dt_adv=120.0)
    gpu, orc = run_pair(cfg, 1)
    e1 = compare(gpu, orc, BC_FIELDS)
    orc.step(4)
    gpu.step(4)
    e5 = compare(gpu, orc, BC_FIELDS)
    eq = max(rel_err(gpu.get_tracer(l), orc.get_tracer(l)) for l in range(2))
    print("van leer limiter", limiter, max(e1.values()), max(e5.values()), "q", eq)
    assert max(e1.values()) <= 1e-12, e1
    assert max(e5.values()) <= 1e-10, e5
    assert eq <= 1e-11, eq


@pytest.mark.parametrize("baroclinic", [False, True])
def test_div_damp_order4(baroclinic):
    if baroclinic:
        cfg, fields, n = baroclinic_config(use_div_damp=1, div_damp_order=4, div_damp_coef4=0.01), BC_FIELDS, 3
    else:
        cfg, fields, n = swm_config(use_div_damp=1, div_damp_order=4, div_damp_coef4=0.01), SWM_FIELDS, 5
    gpu, orc = run_pair(cfg, n)
    err = compare(gpu, orc, fields)
    print("div damp order 4 baroclinic", baroclinic, err)
    assert max(err.values()) <= 1e-11, err


def test_options_mixed_form():
    """TVD PV and van Leer fluxes together in the mixed form against the FP64
    oracle (fourth-order damping with the reference's default coefficient is
    not stable for long at this 5 degree test resolution, so it is checked
    separately above)."""
    kw = dict(pv_scheme=abi.PV_TVD, ffsl_flux_type=abi.FLUX_VAN_LEER, ntracer=1, dt_adv=120.0)
    cfg64 = baroclinic_config(precision=abi.PREC_FP64, **kw)
    cfg32 = baroclinic_config(precision=abi.PREC_MIXED, **kw)
    gpu, orc = run_pair(cfg64, 4, cfg_gpu=cfg32)
    err = compare(gpu, orc, BC_FIELDS)
    print("options mixed vs fp64 oracle", err)
    assert err["phs"] <= 1e-6 and err["pt"] <= 1e-5, err
    assert max(err.values()) <= 5e-3, err


def test_div_damp_order4_mixed_form():
    kw = dict(use_div_damp=1, div_damp_order=4, div_damp_coef4=0.01)
    cfg64 = baroclinic_config(precision=abi.PREC_FP64, **kw)
    cfg32 = baroclinic_config(precision=abi.PREC_MIXED, **kw)
    gpu, orc = run_pair(cfg64, 2, cfg_gpu=cfg32)
    err = compare(gpu, orc, BC_FIELDS)
    print("div damp order 4 mixed vs fp64 oracle", err)
    assert err["phs"] <= 1e-6 and err["pt"] <= 1e-5, err
    assert max(err.values()) <= 5e-3, err
