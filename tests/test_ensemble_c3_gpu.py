"""Batched ensembles of the C3 shape: 48 members at 2 degrees (180x90x26,
dt = 600 s) and 16 members at 1 degree (360x180x26, dt = 300 s), FP32 bulk
with FP64 reductions, members differing by seeded 0.1 K temperature noise,
240 steps: every member stays finite and conserves its mass, and members
stay distinct."""
import numpy as np
import pytest

import gmcore_gb300 as g
from gmcore_gb300 import abi


@pytest.mark.gpu
@pytest.mark.slow
@pytest.mark.parametrize("nlon,nlat,members,dt", [(180, 90, 48, 600.0), (360, 180, 16, 300.0)])
def test_ensemble_240_steps(nlon, nlat, members, dt):
    kw = dict(nlon=nlon, nlat=nlat, nlev=26, baroclinic=1, dt_dyn=dt, vert_coord_template=abi.VCOORD_TEST_L26,
              time_scheme=abi.TIME_WRFRK3, max_wave_speed=400.0, precision=abi.PREC_MIXED)
    base = abi.default_config(**kw)
    m = g.Model(abi.default_config(n_members=members, **kw))
    for mem in range(members):
        m.set_state(g.make_ic(base, 2, 500 + mem, 0.1), member=mem)
    m.prepare()
    tm0 = [m.diagnose(mem)["tm"] for mem in (0, members - 1)]
    m.step(240)
    tm1 = [m.diagnose(mem)["tm"] for mem in (0, members - 1)]
    ps = [m.get_field("phs", member=mem) for mem in (0, members - 1)]
    m.close()
    for p in ps:
        assert np.all(np.isfinite(p))
        assert 5e4 < p.min() and p.max() < 1.1e5
    assert not np.array_equal(ps[0], ps[1])
    for a, b in zip(tm0, tm1):
        assert abs(b - a) / a < 1e-8
