"""The Held-Suarez test forcing (test_case = 'held_suarez', applied to the new
state after the integrator: test_forcing_run, gmcore_mod.F90:586;
held_suarez_test_mod.F90:74-112) on the GPU against the FP64 oracle: the FP64
form within 1e-12 after one step and 1e-10 after twelve (5 degrees, test_l26,
WRF-RK3, dt = 600 s), the mixed form within its stated tolerances, with tracers
and with every ensemble launch layout."""
import numpy as np
import pytest

from gmcore_gb300 import Model, abi, make_ic
from oracle import Oracle

from helpers import BC_FIELDS, compare, load_state, rel_err

pytestmark = pytest.mark.gpu


def config(precision, ntr=0, members=1):
    return abi.default_config(nlon=72, nlat=37, nlev=26, baroclinic=1, dt_dyn=600.0,
                              vert_coord_template=abi.VCOORD_TEST_L26, time_scheme=abi.TIME_WRFRK3,
                              max_wave_speed=400.0, ntracer=ntr, precision=precision, n_members=members,
                              forcing=abi.FORCING_HELD_SUAREZ)


def pair(cfg, st):
    orc, gpu = Oracle(cfg), Model(cfg)
    for obj in (orc, gpu):
        load_state(obj, st)
        obj.prepare()
    return orc, gpu


def test_fp64_against_oracle():
    cfg = config(abi.PREC_FP64, ntr=2)
    st = make_ic(cfg, 2, 5, 1.0)
    orc, gpu = pair(cfg, st)
    orc.step(1)
    gpu.step(1)
    e1 = compare(gpu, orc, BC_FIELDS)
    orc.step(11)
    gpu.step(11)
    e12 = compare(gpu, orc, BC_FIELDS)
    eq = max(rel_err(gpu.get_tracer(l), orc.get_tracer(l)) for l in range(2))
    print("held_suarez FP64 after 1 step", e1, "after 12", e12, "tracers", eq)
    assert max(e1.values()) <= 1e-12, e1
    assert max(e12.values()) <= 1e-10, e12
    assert eq <= 1e-10
    gpu.close()
    orc.close()


def test_mixed_form_within_stated_error():
    cfg = config(abi.PREC_MIXED)
    st = make_ic(cfg, 2, 5, 1.0)
    orc, gpu = pair(cfg, st)
    orc.step(4)
    gpu.step(4)
    e = compare(gpu, orc, ("u_lon", "v_lat", "pt", "phs"))
    print("held_suarez mixed after 4 steps", e)
    assert e["phs"] <= 1e-6 and e["pt"] <= 1e-5, e
    assert max(e.values()) <= 5e-3, e
    gpu.close()
    orc.close()


@pytest.mark.parametrize("layout", [0, 1])
def test_ensemble_members_equal_single_runs(layout):
    one = config(abi.PREC_MIXED)
    states = [make_ic(one, 2, 20 + m, 0.5) for m in range(2)]
    ens = Model(config(abi.PREC_MIXED, members=2))
    for m, st in enumerate(states):
        for k, a in st.items():
            ens.set_field(k, a, member=m)
    ens.set_member_layout(layout)
    ens.prepare()
    ens.step(3)
    for m, st in enumerate(states):
        single = Model(one)
        load_state(single, st)
        single.prepare()
        single.step(3)
        for f in ("u_lon", "v_lat", "pt", "phs"):
            assert np.array_equal(ens.get_field(f, member=m), single.get_field(f)), (layout, m, f)
        single.close()
    ens.close()
