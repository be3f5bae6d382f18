"""GPU step vs the FP64 oracle on the same seeded initial state.

Tolerances (FP64 form): max-norm error relative to the field's maximum
<= 1e-12 after one step and <= 1e-9 after the longer runs; the two codes
evaluate the same expressions but differ in summation order of ring/column
sums, fused multiply-adds and libm vs CUDA transcendental rounding.
"""
import numpy as np
import pytest

from gmcore_gb300 import Model
from oracle import Oracle

from helpers import (BC_FIELDS, SWM_FIELDS, baroclinic_config, compare, initial_state, load_state,
                     swm_config)

pytestmark = pytest.mark.gpu


def run_pair(cfg, nsteps, seed=7):
    st = initial_state(cfg, seed)
    orc = Oracle(cfg)
    load_state(orc, st)
    orc.prepare()
    gpu = Model(cfg)
    load_state(gpu, st)
    gpu.prepare()
    orc.step(nsteps)
    gpu.step(nsteps)
    return gpu, orc


@pytest.mark.parametrize("nsteps,tol", [(1, 1e-12), (20, 1e-9)])
def test_swm_small(nsteps, tol):
    gpu, orc = run_pair(swm_config(), nsteps)
    err = compare(gpu, orc, SWM_FIELDS)
    print("swm 72x37", nsteps, err)
    assert max(err.values()) <= tol, err


def test_swm_c1_one_degree():
    # 1 degree, dt = 60 s, predict-correct: the shallow-water benchmark grid
    cfg = swm_config(nlon=360, nlat=180, dt=60.0)
    gpu, orc = run_pair(cfg, 1)
    err1 = compare(gpu, orc, SWM_FIELDS)
    orc.step(9)
    gpu.step(9)
    err10 = compare(gpu, orc, SWM_FIELDS)
    print("swm C1 1 step", err1, "10 steps", err10)
    assert max(err1.values()) <= 1e-12, err1
    assert max(err10.values()) <= 1e-10, err10


@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_swm_time_schemes(scheme):
    gpu, orc = run_pair(swm_config(time_scheme=scheme), 3)
    err = compare(gpu, orc, SWM_FIELDS)
    assert max(err.values()) <= 1e-11, err


@pytest.mark.parametrize("nsteps,tol", [(1, 1e-12), (10, 1e-9)])
def test_baroclinic_small(nsteps, tol):
    gpu, orc = run_pair(baroclinic_config(), nsteps)
    err = compare(gpu, orc, BC_FIELDS)
    print("baroclinic 72x37x26", nsteps, err)
    assert max(err.values()) <= tol, err


def test_baroclinic_wrf_l32():
    gpu, orc = run_pair(baroclinic_config(nlon=90, nlat=46, nlev=32, dt=600.0), 2)
    err = compare(gpu, orc, BC_FIELDS)
    print("baroclinic wrf_l32", err)
    assert max(err.values()) <= 1e-11, err


def test_diagnose_matches_oracle():
    gpu, orc = run_pair(baroclinic_config(), 2)
    dg, do = gpu.diagnose(), orc.diagnose()
    for k in ("tm", "te", "te_ke", "te_ie", "te_pe", "tav", "tpe", "tpt"):
        scale = max(abs(do[k]), 1e-300)
        assert abs(dg[k] - do[k]) / scale <= 1e-11 or abs(dg[k] - do[k]) <= 1e-12 * abs(do["te"]), (k, dg[k], do[k])


def run_pair_tracers(cfg, nsteps, seed=7):
    st = initial_state(cfg, seed)
    orc = Oracle(cfg)
    load_state(orc, st)
    orc.prepare()
    gpu = Model(cfg)
    load_state(gpu, st)
    gpu.prepare()
    orc.step(nsteps)
    gpu.step(nsteps)
    return gpu, orc


def tracer_err(gpu, orc, ntr):
    from helpers import rel_err
    return max(rel_err(gpu.get_tracer(l), orc.get_tracer(l)) for l in range(ntr))


@pytest.mark.parametrize("dt_adv_mult,nsteps", [(1, 4), (3, 8)])
def test_tracer_batch(dt_adv_mult, nsteps):
    # adv_run: advection starts at the second step and uses the static batch's
    # copy / add / average wind cadence (nstep = dt_adv / dt_dyn)
    cfg = baroclinic_config(ntracer=2, dt_adv=120.0 * dt_adv_mult)
    gpu, orc = run_pair_tracers(cfg, nsteps)
    e_q = tracer_err(gpu, orc, 2)
    err = compare(gpu, orc, BC_FIELDS)
    print("tracers dt_adv x", dt_adv_mult, "q", e_q, "dyn", max(err.values()))
    assert e_q <= 1e-11, e_q
    assert max(err.values()) <= 1e-10, err


def test_div_damp():
    cfg = baroclinic_config(use_div_damp=1)
    gpu, orc = run_pair(cfg, 3)
    err = compare(gpu, orc, BC_FIELDS)
    print("div damp", err)
    assert max(err.values()) <= 1e-11, err


def test_swm_div_damp():
    cfg = swm_config(use_div_damp=1)
    gpu, orc = run_pair(cfg, 5)
    err = compare(gpu, orc, SWM_FIELDS)
    assert max(err.values()) <= 1e-11, err


def test_mixed_precision_tracks_fp64():
    # FP32 bulk fields with FP64 rings, column sweeps and filter weights:
    # stays within a few 1e-5 of the FP64 oracle over a few steps
    cfg = baroclinic_config(precision=1, ntracer=1)
    cfg64 = baroclinic_config(precision=0, ntracer=1)
    st = initial_state(cfg64, 7)
    orc = Oracle(cfg64)
    load_state(orc, st)
    orc.prepare()
    gpu = Model(cfg)
    load_state(gpu, st)
    gpu.prepare()
    orc.step(4)
    gpu.step(4)
    err = compare(gpu, orc, BC_FIELDS)
    e_q = tracer_err(gpu, orc, 1)
    print("mixed vs fp64 oracle", err, "q", e_q)
    assert err["phs"] <= 1e-6 and err["pt"] <= 1e-5, err
    assert max(err.values()) <= 5e-3, err
    assert e_q <= 1e-3, e_q
