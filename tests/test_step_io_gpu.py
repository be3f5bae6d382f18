"""gmc_step_io, the coupled-step exchange: inputs set, nsteps steps, outputs
read back, with the transfers of registered host arrays overlapped with the
step.  Its results must equal, bit for bit, the same exchange made with
gmc_set_field / gmc_set_tracer, gmc_step and gmc_get_field / gmc_get_tracer,
for registered arrays (the overlapped path) and for pageable ones (the
sequential path), over several exchanges so that a stale or early transfer
would show in the next step."""
import numpy as np
import pytest

import gmcore_gb300 as g
from gmcore_gb300 import GmcError, abi

pytestmark = pytest.mark.gpu

FIELDS = ("u_lon", "v_lat", "pt", "phs")


def config(precision, ntr=3):
    return abi.default_config(nlon=144, nlat=73, nlev=26, baroclinic=1, dt_dyn=300.0,
                              vert_coord_template=abi.VCOORD_TEST_L26, time_scheme=abi.TIME_WRFRK3,
                              max_wave_speed=400.0, ntracer=ntr, precision=precision)


def model(cfg, st):
    m = g.Model(cfg)
    m.set_state(st)
    m.prepare()
    return m


def host_arrays(st, registered):
    make = g.page_aligned if registered else np.zeros
    host = {}
    for k in FIELDS + ("q",):
        host[k] = make(st[k].shape)
        host[k][...] = st[k]
    out = {k: make(host[k].shape) for k in FIELDS + ("q",)}
    return host, out


@pytest.mark.parametrize("precision", [abi.PREC_MIXED, abi.PREC_FP64])
@pytest.mark.parametrize("registered", [True, False])
@pytest.mark.parametrize("nsteps", [1, 2])
def test_exchange_equals_separate_calls(precision, registered, nsteps):
    cfg = config(precision)
    st = g.make_ic(cfg, 2, 7, 1.0)
    ref, ex = model(cfg, st), model(cfg, st)
    host, out = host_arrays(st, registered)
    regs = [host[k] for k in host] + [out[k] for k in out] if registered else []
    for a in regs:
        g.host_register(a)
    try:
        for _ in range(3):
            # perturb every input between exchanges, as a coupled driver would,
            # so that an input read before its transfer ends would show
            host["pt"] *= 1.0 + 1e-6
            host["u_lon"] *= 1.0 + 1e-6
            host["v_lat"] *= 1.0 - 1e-6
            host["phs"] += 0.5
            host["q"][0] *= 0.999
            for k in FIELDS:
                ref.set_field(k, host[k])
            for l in range(cfg.ntracer):
                ref.set_tracer(l, host["q"][l])
            ref.step(nsteps)
            want = {k: ref.get_field(k) for k in FIELDS}
            want_q = np.stack([ref.get_tracer(l) for l in range(cfg.ntracer)])
            ex.step_io([(k, host[k]) for k in FIELDS] + [(l, host["q"][l]) for l in range(cfg.ntracer)], nsteps,
                       [(k, out[k]) for k in FIELDS] + [(l, out["q"][l]) for l in range(cfg.ntracer)])
            for k in FIELDS:
                assert np.array_equal(out[k], want[k]), k
            assert np.array_equal(out["q"], want_q)
            for k in FIELDS + ("q",):
                host[k][...] = out[k]
        assert ex.stats()["steps"] == nsteps
    finally:
        for a in regs:
            g.host_unregister(a)
        ref.close()
        ex.close()


def test_exchange_rejects_a_bad_item_before_moving_anything():
    cfg = config(abi.PREC_MIXED)
    st = g.make_ic(cfg, 2, 7, 1.0)
    m = model(cfg, st)
    before = m.get_field("pt")
    with pytest.raises(GmcError) as e:
        m.step_io([("pt", before * 2.0), (7, np.zeros((cfg.nlev, cfg.nlat, cfg.nlon)))], 1, [])
    assert e.value.code == abi.GMC_EINVAL
    assert np.array_equal(m.get_field("pt"), before)
    with pytest.raises(GmcError):
        m.step_io([], 1, [("nonsense", np.zeros((cfg.nlat, cfg.nlon)))])
    # an unknown output name stops the call before its inputs are set
    with pytest.raises(GmcError):
        m.step_io([("pt", before * 2.0)], 1, [("nonsense", np.zeros((cfg.nlev, cfg.nlat, cfg.nlon)))])
    assert np.array_equal(m.get_field("pt"), before)
    m.close()
