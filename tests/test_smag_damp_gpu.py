"""Smagorinsky damping (use_smag_damp: damp_run, damp_mod.F90:59-61;
smag_damp_run, smag_damp_mod.F90:52-190) on the GPU against the FP64 oracle:
the FP64 form within 1e-12 after one step and 1e-10 after twelve (5 degrees,
test_l26, WRF-RK3, dt = 600 s), alone and after the Held-Suarez forcing and
fourth-order divergence damping, the mixed form within its stated
tolerances, and every ensemble launch layout equal to single runs."""
import numpy as np
import pytest

from gmcore_gb300 import Model, abi, make_ic
from oracle import Oracle

from helpers import BC_FIELDS, compare, load_state

pytestmark = pytest.mark.gpu


def config(precision, members=1, **kw):
    return abi.default_config(nlon=72, nlat=37, nlev=26, baroclinic=1, dt_dyn=600.0,
                              vert_coord_template=abi.VCOORD_TEST_L26, time_scheme=abi.TIME_WRFRK3,
                              max_wave_speed=400.0, precision=precision, n_members=members,
                              use_smag_damp=1, smag_damp_coef=0.1, **kw)


def run_pair(cfg, st, steps):
    orc, gpu = Oracle(cfg), Model(cfg)
    for obj in (orc, gpu):
        load_state(obj, st)
        obj.prepare()
    out = []
    for n in steps:
        orc.step(n)
        gpu.step(n)
        out.append(compare(gpu, orc, BC_FIELDS))
    gpu.close()
    orc.close()
    return out


@pytest.mark.parametrize("extra", [{}, {"forcing": abi.FORCING_HELD_SUAREZ, "use_div_damp": 1, "div_damp_order": 4}])
def test_fp64_against_oracle(extra):
    cfg = config(abi.PREC_FP64, **extra)
    e1, e12 = run_pair(cfg, make_ic(cfg, 2, 9, 1.0), (1, 11))
    print("smag FP64", extra, "after 1 step", e1, "after 12", e12)
    assert max(e1.values()) <= 1e-12, e1
    assert max(e12.values()) <= 1e-10, e12


def test_mixed_form_within_stated_error():
    cfg = config(abi.PREC_MIXED)
    (e,) = run_pair(cfg, make_ic(cfg, 2, 9, 1.0), (4,))
    print("smag mixed after 4 steps", e)
    assert e["phs"] <= 1e-6 and e["pt"] <= 1e-5, e
    assert max(e[f] for f in ("u_lon", "v_lat", "pt", "phs")) <= 5e-3, e


@pytest.mark.parametrize("layout", [0, 1])
def test_ensemble_members_equal_single_runs(layout):
    one = config(abi.PREC_MIXED)
    states = [make_ic(one, 2, 30 + m, 0.5) for m in range(2)]
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
