"""History and restart files of a GPU context (gmc_restart_write,
gmc_restart_read, gmc_history_write; restart_mod.F90:54-251,
history_mod.F90:125-580), read back with scipy's netCDF reader:

* a restart holds the context's state bit for bit, and a context that reads
  it, prepares and steps continues the dynamics bit for bit like the context
  that never stopped (FP64 and mixed forms);
* a history file (two records, the second appended) holds the state and the
  tracers bit for bit, the integrals of gmc_diagnose, and ph, t, z, div and
  vor within FP64 rounding of the oracle's calc_ph / calc_t / calc_gz_lev /
  calc_div / calc_vor of the same state (the GPU contracts products into
  FMAs, evaluates pow and log with CUDA's libm and sums the pole rings in
  another order: relative tolerance 1e-12 of each field's largest value)."""
import numpy as np
import pytest

import gmcore_gb300 as g
from gmcore_gb300 import abi, GmcError
from oracle import Oracle

from helpers import load_state

pytestmark = pytest.mark.gpu
netcdf = pytest.importorskip("scipy.io").netcdf_file

DYN = ("u_lon", "v_lat", "pt", "phs")


def bc_config(precision, ntracer=2):
    return abi.default_config(nlon=72, nlat=37, nlev=26, baroclinic=1, dt_dyn=600.0,
                              vert_coord_template=abi.VCOORD_TEST_L26, time_scheme=abi.TIME_WRFRK3,
                              max_wave_speed=400.0, ntracer=ntracer, precision=precision)


def swm_config(precision):
    return abi.default_config(nlon=72, nlat=37, nlev=1, baroclinic=0, dt_dyn=600.0, time_scheme=abi.TIME_PC2,
                              precision=precision)


def started(cfg, st, steps):
    m = g.Model(cfg)
    m.set_state(st)
    m.prepare()
    if steps:
        m.step(steps)
    return m


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_restart_holds_the_state_and_continues_bit_for_bit(tmp_path, precision):
    cfg = bc_config(precision)
    a = started(cfg, g.make_ic(cfg, 2, 9, 1.0), 3)
    path = tmp_path / "run.r0.nc"
    a.restart_write(path, 1800.0, time_units="minutes")
    with netcdf(str(path), "r", mmap=False) as f:
        for name, key in (("u", "u_lon"), ("v", "v_lat"), ("pt", "pt"), ("phs", "phs"), ("gzs", "gzs")):
            assert np.array_equal(f.variables[name][0], a.get_field(key)), name
        for l in range(cfg.ntracer):
            assert np.array_equal(f.variables[f"q{l + 1}"][0], a.get_tracer(l))
        assert f.variables["time"][0] == 30.0
    b = g.Model(cfg)
    assert b.restart_read(path) == 1800.0
    for k in DYN + ("gzs",):
        assert np.array_equal(b.get_field(k), a.get_field(k)), k
    b.prepare()
    # the same file set through set_field / set_tracer: the reading context
    # must be that state exactly
    _, host = g.restart_read_host(cfg, path)
    c = g.Model(cfg)
    c.set_state(host)
    c.prepare()
    for m in (a, b, c):
        m.step(3)
    for k in DYN:
        assert np.array_equal(a.get_field(k), b.get_field(k)), k   # the dynamics never noticed the restart
        assert np.array_equal(c.get_field(k), b.get_field(k)), k
    for l in range(cfg.ntracer):
        assert np.array_equal(c.get_tracer(l), b.get_tracer(l))
    for m in (a, b, c):
        m.close()


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_history_records_against_the_oracle(tmp_path, precision):
    cfg = bc_config(precision)
    m = started(cfg, g.make_ic(cfg, 2, 11, 1.0), 2)
    path = tmp_path / "run.h0.nc"
    m.history_write(path, 1200.0, tracer_names="qa,qb")
    first = {k: m.get_field(k) for k in DYN}
    m.step(1)
    m.history_write(path, 1800.0, append=True, tracer_names="qa,qb")
    with netcdf(str(path), "r", mmap=False) as f:
        assert f.variables["time"][:].tolist() == [1200.0 / 3600, 1800.0 / 3600]
        assert np.array_equal(f.variables["pt"][0], first["pt"]) and np.array_equal(f.variables["u"][0], first["u_lon"])
        for name, key in (("u", "u_lon"), ("v", "v_lat"), ("pt", "pt"), ("phs", "phs")):
            assert np.array_equal(f.variables[name][1], m.get_field(key)), name
        assert np.array_equal(f.variables["qa"][1], m.get_tracer(0)) and np.array_equal(f.variables["qb"][1], m.get_tracer(1))
        d = m.diagnose()
        for k in ("te", "tpe", "te_ke", "te_ie", "te_pe"):
            assert f.variables[k][1] == d[k], k
        assert f.variables["tm"].typecode() == "f" and f.variables["tm"][1] == np.float32(d["tm"])
        assert np.array_equal(f.variables["zs"][:], m.get_field("gzs") / cfg.g)
        for k in ("ph", "vor", "div"):
            assert f.variables[k].typecode() == "f", k       # declared without dtype='r8' in the reference
        got = {k: np.asarray(f.variables[k][1], dtype=np.float64) for k in ("t", "z")}
        got32 = {k: np.asarray(f.variables[k][1]) for k in ("ph", "vor", "div")}
    # the oracle diagnoses the GPU's own state
    o = Oracle(cfg)
    load_state(o, {k: m.get_field(k) for k in DYN + ("gzs",)})
    o.prepare()
    for k in ("u_f", "v_f", "phs_f"):
        o.set_field(k, m.get_field(k))
    want = o.output_diag()
    o.close()
    for k, a in got.items():
        err = np.max(np.abs(a - want[k])) / np.max(np.abs(want[k]))
        assert err <= 1e-12, (k, err)
    for k, a in got32.items():   # stored as float32: equal to the rounded oracle value within one rounding
        assert np.allclose(a, want[k].astype(np.float32), rtol=1e-6, atol=1e-6 * np.max(np.abs(want[k]))), k
    m.close()


def test_shallow_water_history(tmp_path):
    cfg = swm_config(abi.PREC_FP64)
    m = started(cfg, g.make_ic(cfg, 1, 4, 1.0), 4)
    path = tmp_path / "swm.h0.nc"
    m.history_write(path, 2400.0, time_units="seconds")
    with netcdf(str(path), "r", mmap=False) as f:
        assert list(f.variables) == ["time", "lon", "lat", "ilon", "ilat", "tm", "te", "tpe", "u", "v", "z", "pv",
                                     "div", "zs"]
        assert f.variables["pv"].dimensions == ("time", "ilat", "ilon")
        assert np.array_equal(f.variables["pv"][0], m.get_field("pv")[0])
        assert np.array_equal(f.variables["u"][0], m.get_field("u_lon")[0])
        z, div = f.variables["z"][0], f.variables["div"][0]
    assert np.array_equal(z, m.get_field("gz") / cfg.g)
    o = Oracle(cfg)
    load_state(o, {k: m.get_field(k) for k in ("u_lon", "v_lat", "gz", "gzs")})
    o.prepare()
    for k in ("u_f", "v_f"):
        o.set_field(k, m.get_field(k))
    want = o.output_diag()["div"][0]
    assert np.max(np.abs(div - want)) <= 1e-12 * np.max(np.abs(want))
    m.close()


def test_restart_errors(tmp_path):
    cfg = bc_config(abi.PREC_MIXED)
    m = started(cfg, g.make_ic(cfg, 2, 9, 1.0), 0)
    before = m.get_field("pt")
    with pytest.raises(GmcError) as e:
        m.restart_read(tmp_path / "none.nc")
    assert e.value.code == abi.GMC_EIO
    other = bc_config(abi.PREC_MIXED, ntracer=0)
    g.restart_write_host(other, tmp_path / "nq.nc", 0.0, g.make_ic(other, 2, 1, 1.0))
    assert m.restart_read(tmp_path / "nq.nc") == 0.0              # tracers absent: kept
    assert not np.array_equal(m.get_field("pt"), before)
    with pytest.raises(GmcError) as e:
        m.history_write(tmp_path / "h.nc", 0.0, tracer_names="just_one")
    assert e.value.code == abi.GMC_EINVAL
    m.close()


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_background_writes_equal_synchronous_ones(tmp_path, precision):
    """A background write captures the state at the call: the steps taken
    while it runs do not reach the file, which equals, byte for byte, the file
    a synchronous write of the same state makes."""
    cfg = bc_config(precision)
    st = g.make_ic(cfg, 2, 13, 1.0)
    a, b = started(cfg, st, 2), started(cfg, st, 2)
    a.history_write(tmp_path / "bg.h0.nc", 1200.0, background=True)
    a.step(3)                                   # overlaps the write
    a.restart_write(tmp_path / "bg.r0.nc", 3000.0, background=True)   # waits for the history write first
    a.step(1)
    a.output_wait()
    b.history_write(tmp_path / "fg.h0.nc", 1200.0)
    b.step(3)
    b.restart_write(tmp_path / "fg.r0.nc", 3000.0)
    for name in ("h0", "r0"):
        assert (tmp_path / f"bg.{name}.nc").read_bytes() == (tmp_path / f"fg.{name}.nc").read_bytes(), name
    b.step(1)
    for k in DYN:
        assert np.array_equal(a.get_field(k), b.get_field(k)), k
    a.output_wait()                             # nothing in flight: OK
    a.close()
    b.close()


def test_background_write_failure_is_reported(tmp_path):
    cfg = bc_config(abi.PREC_MIXED)
    m = started(cfg, g.make_ic(cfg, 2, 9, 1.0), 1)
    m.history_write(tmp_path / "no_such_dir" / "h.nc", 0.0, background=True)
    m.step(1)
    with pytest.raises(GmcError) as e:
        m.output_wait()
    assert e.value.code == abi.GMC_EIO
    m.output_wait()                             # reported once
    # a failed background write is reported by the next file call
    m.restart_write(tmp_path / "no_such_dir" / "r.nc", 0.0, background=True)
    with pytest.raises(GmcError) as e:
        m.restart_write(tmp_path / "r.nc", 0.0)
    assert e.value.code == abi.GMC_EIO
    m.restart_write(tmp_path / "r.nc", 0.0)
    m.close()


@pytest.mark.parametrize("background", [False, True])
def test_ensemble_member_files_equal_single_runs(tmp_path, background):
    """Member 1 of a two-member context writes the restart and history files
    that a one-member context holding the same state writes, byte for byte."""
    one = bc_config(abi.PREC_MIXED)
    ens_cfg = bc_config(abi.PREC_MIXED)
    ens_cfg.n_members = 2
    states = [g.make_ic(one, 2, 40 + k, 0.5) for k in range(2)]
    ens = g.Model(ens_cfg)
    for k, st in enumerate(states):
        ens.set_state(st, member=k)
    ens.prepare()
    ens.step(2)
    single = started(one, states[1], 2)
    for name, call in (("r0", "restart_write"), ("h0", "history_write")):
        getattr(ens, call)(tmp_path / f"ens.{name}.nc", 1200.0, member=1, background=background)
        ens.output_wait()
        getattr(single, call)(tmp_path / f"one.{name}.nc", 1200.0)
        assert (tmp_path / f"ens.{name}.nc").read_bytes() == (tmp_path / f"one.{name}.nc").read_bytes(), name
    ens.close()
    single.close()


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_shallow_water_restart_continues_bit_for_bit(tmp_path, precision):
    cfg = swm_config(precision)
    a = started(cfg, g.make_ic(cfg, 1, 5, 1.0), 4)
    a.restart_write(tmp_path / "swm.r0.nc", 2400.0)
    b = g.Model(cfg)
    assert b.restart_read(tmp_path / "swm.r0.nc") == 2400.0
    b.prepare()
    a.step(5)
    b.step(5)
    for k in ("u_lon", "v_lat", "gz"):
        assert np.array_equal(a.get_field(k), b.get_field(k)), k
    a.close()
    b.close()
