"""The library's status codes on states that make the step fail, injected on
the host through gmc_set_field (no device fault is provoked: every kernel
keeps its indexes in range for any value, and the error word is read after
the call).  Where the reference stops (non-monotonic pressure levels,
Courant number beyond the halo, unfillable negative tracer) the library
returns the oracle's code at the same call, prologue or step; a non-finite
state value, which the reference does not check, returns GMC_ENAN.  After an
error the context stays usable: the same context reports GMC_OK again once a
clean state is set and prepared."""
import numpy as np
import pytest

from gmcore_gb300 import GmcError, Model, abi
from oracle import Oracle

import error_cases as ec
from helpers import load_state

pytestmark = pytest.mark.gpu

PRECISIONS = [abi.PREC_FP64, abi.PREC_MIXED]


def outcome(obj, state, after_prepare=None, steps=1):
    """(where, code): where the call sequence stopped and its status."""
    load_state(obj, state)
    try:
        obj.prepare()
    except (GmcError, RuntimeError) as e:
        return "prepare", _code(e)
    for name, a in (after_prepare or {}).items():
        obj.set_field(name, a)
    try:
        obj.step(steps)
    except (GmcError, RuntimeError) as e:
        return "step", _code(e)
    return "ok", abi.GMC_OK


def _code(e):
    if isinstance(e, GmcError):
        return e.code
    return int(str(e).split("(")[1].split(")")[0])   # oracle: "... failed (<code>): ..."


def both(cfg, state, after_prepare=None, steps=1):
    m = Model(cfg)
    try:
        got = outcome(m, state, after_prepare, steps)
    finally:
        m.close()
    o = Oracle(cfg)   # FP64 whatever the form
    try:
        want = outcome(o, state, after_prepare, steps)
    finally:
        o.close()
    return got, want


@pytest.mark.parametrize("precision", PRECISIONS)
def test_nonmonotonic_column_at_prologue(precision):
    cfg = ec.config(precision=precision)
    got, want = both(cfg, ec.low_column(ec.base_state(cfg), cfg))
    assert want == ("prepare", abi.GMC_ENONMONO)
    assert got == want


@pytest.mark.parametrize("precision", PRECISIONS)
def test_nonmonotonic_column_after_update(precision):
    cfg = ec.config(precision=precision)
    st = ec.base_state(cfg)
    got, want = both(cfg, st, after_prepare={"phs": ec.low_column(st, cfg)["phs"]})
    assert want == ("step", abi.GMC_ENONMONO)
    assert got == want


@pytest.mark.parametrize("precision", PRECISIONS)
def test_courant_number_beyond_halo(precision):
    cfg = ec.config(precision=precision)
    m = Model(cfg)
    hx = m.lon_halo_width
    m.close()
    st = ec.base_state(cfg)
    got, want = both(cfg, ec.fast_band(st, cfg, hx))
    assert want == ("prepare", abi.GMC_ECFL)
    assert got == want
    got, want = both(cfg, st, after_prepare={"u_lon": ec.fast_band(st, cfg, hx)["u_lon"]}, steps=2)
    assert want == ("step", abi.GMC_ECFL)
    assert got == want


@pytest.mark.parametrize("precision", PRECISIONS)
def test_unfillable_negative_tracer(precision):
    cfg = ec.config(precision=precision, ntracer=2)
    got, want = both(cfg, ec.negative_row(ec.base_state(cfg), cfg), steps=2)
    assert want == ("step", abi.GMC_ENEGTRACER)
    assert got == want


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("field", ["u_lon", "v_lat", "pt", "phs"])
def test_non_finite_value_is_reported_and_context_recovers(precision, field):
    cfg = ec.config(precision=precision)
    st = ec.base_state(cfg)
    m = Model(cfg)
    load_state(m, st)
    m.prepare()
    bad = st[field].copy()
    bad[(0,) * (bad.ndim - 2) + (cfg.nlat // 4, 5)] = np.nan
    m.set_field(field, bad)
    with pytest.raises(GmcError) as e:
        m.step(1)
    assert e.value.code == abi.GMC_ENAN
    assert "non-finite" in str(e.value)
    # the same context runs a clean state afterwards
    load_state(m, st)
    m.prepare()
    m.step(2)
    assert np.isfinite(m.get_field("phs")).all()
    m.close()


def test_clean_state_runs_without_error():
    cfg = ec.config(ntracer=2)
    got, want = both(cfg, ec.base_state(cfg), steps=2)
    assert got == want == ("ok", abi.GMC_OK)


def test_calls_out_of_order_are_estate():
    # a step, or the tangent-linear model, before gmc_prepare: GMC_ESTATE, and
    # the context still prepares and steps afterwards
    cfg = ec.config()
    m = Model(cfg)
    load_state(m, ec.base_state(cfg))
    with pytest.raises(GmcError) as e:
        m.step(1)
    assert e.value.code == abi.GMC_ESTATE
    swm = abi.default_config(nlon=72, nlat=37, nlev=1, baroclinic=0, dt_dyn=600.0)
    s = Model(swm)
    with pytest.raises(GmcError) as e:
        s.tlm_step(1, {"u_lon": np.zeros((1, 37, 72)), "v_lat": np.zeros((1, 36, 72)), "gz": np.zeros((37, 72))})
    assert e.value.code == abi.GMC_ESTATE
    s.close()
    m.prepare()
    m.step(1)
    m.close()


def test_device_allocation_failure_is_enomem():
    # 8192 x 4000 x 64 levels in FP64 needs several hundred GB of device memory
    cfg = abi.default_config(nlon=8192, nlat=4000, nlev=64, baroclinic=1, dt_dyn=1.0,
                             vert_coord_template=abi.VCOORD_WRF_L64)
    with pytest.raises(GmcError) as e:
        Model(cfg)
    assert e.value.code == abi.GMC_ENOMEM
    # nothing is left behind: a small context works afterwards
    small = ec.config()
    m = Model(small)
    load_state(m, ec.base_state(small))
    m.prepare()
    m.step(1)
    m.close()
