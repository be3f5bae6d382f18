"""The oracle stops where the reference stops, with the matching status code:
non-monotonic pressure levels at the prologue and after an update
(calc_m, operators_mod.F90:489-500), a zonal Courant number beyond the
longitude halo width (adv_batch_mod.F90:284-287) and a tracer row the zonal
fixer cannot fill (adv_mod.F90:236-258).  The GPU tests compare the library's
status with these on the same injected states."""
import pytest

from gmcore_gb300 import abi
from oracle import Oracle

import error_cases as ec
from helpers import load_state


def run_oracle(cfg, state, after_prepare=None, steps=1):
    o = Oracle(cfg)
    load_state(o, state)
    try:
        try:
            o.prepare()
        except RuntimeError as e:
            return "prepare", e
        if after_prepare:
            for name, a in after_prepare.items():
                o.set_field(name, a)
        try:
            o.step(steps)
        except RuntimeError as e:
            return "step", e
        return "ok", None
    finally:
        o.close()


def code_of(exc):
    # "oracle step failed (<code>): <message>"
    return int(str(exc).split("(")[1].split(")")[0])


def test_oracle_nonmonotonic_column_at_prologue():
    cfg = ec.config()
    where, e = run_oracle(cfg, ec.low_column(ec.base_state(cfg), cfg))
    assert where == "prepare" and code_of(e) == abi.GMC_ENONMONO
    assert "not monotonic" in str(e)


def test_oracle_nonmonotonic_column_after_update():
    cfg = ec.config()
    st = ec.base_state(cfg)
    bad = ec.low_column(st, cfg)
    where, e = run_oracle(cfg, st, after_prepare={"phs": bad["phs"]})
    assert where == "step" and code_of(e) == abi.GMC_ENONMONO


def test_oracle_zonal_courant_number_beyond_halo():
    cfg = ec.config()
    o = Oracle(cfg)
    hx = o.lon_halo_width
    o.close()
    # calc_mf's accum_uv_cell checks the mass batch already in the prologue
    where, e = run_oracle(cfg, ec.fast_band(ec.base_state(cfg), cfg, hx))
    assert where == "prepare" and code_of(e) == abi.GMC_ECFL
    assert "cflx" in str(e)


def test_oracle_zonal_courant_number_beyond_halo_after_prologue():
    cfg = ec.config()
    o = Oracle(cfg)
    hx = o.lon_halo_width
    o.close()
    st = ec.base_state(cfg)
    where, e = run_oracle(cfg, st, after_prepare={"u_lon": ec.fast_band(st, cfg, hx)["u_lon"]}, steps=2)
    assert where == "step" and code_of(e) == abi.GMC_ECFL


def test_oracle_unfillable_negative_tracer_row():
    cfg = ec.config(ntracer=2)
    where, e = run_oracle(cfg, ec.negative_row(ec.base_state(cfg), cfg), steps=2)
    assert where == "step" and code_of(e) == abi.GMC_ENEGTRACER


def test_oracle_seeded_state_runs_clean():
    cfg = ec.config(ntracer=2)
    where, e = run_oracle(cfg, ec.base_state(cfg), steps=2)
    assert where == "ok", e


@pytest.mark.parametrize("kind", [1, 2])
def test_oracle_initial_state_equals_library_generator(kind):
    import numpy as np

    import gmcore_gb300 as g
    import oracle
    if kind == 1:
        cfg = abi.default_config(nlon=72, nlat=37, nlev=1, baroclinic=0, dt_dyn=600.0)
    else:
        cfg = ec.config(ntracer=3)
    a, b = oracle.make_ic(cfg, kind, 123, 0.7), g.make_ic(cfg, kind, 123, 0.7)
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
