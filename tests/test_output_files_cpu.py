"""History and restart files (restart_mod.F90:54-251, history_mod.F90:125-580)
without a GPU: the restart files the library writes from host arrays, read
by scipy's netCDF reader (an independent implementation of the classic
format), and netCDF files scipy writes, read by the library.  A state that
goes through a restart file and back continues, on the oracle, bit for bit
like the run that never stopped."""
import ctypes as C
import os

import numpy as np
import pytest

import gmcore_gb300 as g
from gmcore_gb300 import abi, GmcError
from oracle import Oracle

from helpers import load_state

netcdf = pytest.importorskip("scipy.io").netcdf_file


def bc_config(ntracer=2, **kw):
    return abi.default_config(nlon=72, nlat=37, nlev=26, baroclinic=1, dt_dyn=600.0,
                              vert_coord_template=abi.VCOORD_TEST_L26, time_scheme=abi.TIME_WRFRK3,
                              max_wave_speed=400.0, ntracer=ntracer, **kw)


def swm_config():
    return abi.default_config(nlon=72, nlat=37, nlev=1, baroclinic=0, dt_dyn=600.0, time_scheme=abi.TIME_PC2)


RESTART_BC = {"u": ("u_lon", ("time", "lev", "lat", "ilon"), "u wind component", "m s-1"),
              "v": ("v_lat", ("time", "lev", "ilat", "lon"), "v wind component", "m s-1"),
              "phs": ("phs", ("time", "lat", "lon"), "hydrostatic surface pressure", "Pa"),
              "pt": ("pt", ("time", "lev", "lat", "lon"), "potential temperature", "K"),
              "gzs": ("gzs", ("time", "lat", "lon"), "surface geopotential height", "m2 s-2")}


def test_baroclinic_restart_read_by_scipy(tmp_path):
    cfg = bc_config()
    st = g.make_ic(cfg, 2, 9, 1.0)
    path = tmp_path / "case.r0.nc"
    g.restart_write_host(cfg, path, 7200.0, st, time_units="hours", start_time="2001-02-03 04:05:06",
                         tracer_names=["qv", "o3"], restart_interval="1 days")
    raw = open(path, "rb").read(8)
    assert raw[:4] == b"CDF\x02" and int.from_bytes(raw[4:8], "big") == 1   # 64-bit offsets, one record
    with netcdf(str(path), "r", mmap=False) as f:
        assert f.version_byte == 2
        assert f.dimensions == {"time": None, "lon": 72, "lat": 37, "ilon": 72, "ilat": 36, "lev": 26, "ilev": 27}
        assert list(f.variables) == ["time", "lon", "lat", "ilon", "ilat", "lev", "ilev", "u", "v", "phs", "pt",
                                     "gzs", "qv", "o3"]
        assert f.time_step_size == 600.0 and f.restart_interval == b"1 days"
        for name, (key, dims, long_name, units) in RESTART_BC.items():
            v = f.variables[name]
            assert v.dimensions == dims and v.typecode() == "d", name
            assert v.long_name.decode() == long_name and v.units.decode() == units, name
            assert np.array_equal(v[0], st[key]), name
        assert np.array_equal(f.variables["qv"][0], st["q"][0]) and np.array_equal(f.variables["o3"][0], st["q"][1])
        t = f.variables["time"]
        assert t[0] == 2.0 and t.units == b"hours since 2001-02-03 04:05:06"
        lat, ilat = f.variables["lat"][:], f.variables["ilat"][:]
        assert lat[0] == -90.0 and lat[-1] == 90.0 and np.allclose(np.diff(lat), 5.0)
        assert np.allclose(ilat, 0.5 * (lat[1:] + lat[:-1]))
        assert np.allclose(f.variables["lon"][:], np.arange(72) * 5.0)
        assert np.allclose(f.variables["ilon"][:], np.arange(72) * 5.0 + 2.5)
        assert np.all(np.diff(f.variables["lev"][:]) > 0) and f.variables["ilev"][-1] == pytest.approx(1.0)
    t, back = g.restart_read_host(cfg, path, tracer_names="qv,o3")
    assert t == 7200.0
    for k, a in st.items():
        assert np.array_equal(back[k], a), k


def test_shallow_water_restart_round_trip(tmp_path):
    cfg = swm_config()
    st = g.make_ic(cfg, 1, 3, 1.0)
    path = tmp_path / "swm.r0.nc"
    g.restart_write_host(cfg, path, 86400.0 * 3, st, time_units="days")
    with netcdf(str(path), "r", mmap=False) as f:
        assert f.dimensions == {"time": None, "lon": 72, "lat": 37, "ilon": 72, "ilat": 36}
        assert f.variables["u"].dimensions == ("time", "lat", "ilon")
        assert f.variables["v"].dimensions == ("time", "ilat", "lon")
        assert f.variables["gz"].long_name == b"geopotential height"
        assert np.array_equal(f.variables["gz"][0], st["gz"]) and np.array_equal(f.variables["u"][0], st["u_lon"][0])
        assert f.variables["time"][0] == 3.0
    t, back = g.restart_read_host(cfg, path)
    assert t == 86400.0 * 3
    assert all(np.array_equal(back[k], st[k]) for k in st)


@pytest.mark.parametrize("version", [1, 2])
def test_restart_written_by_scipy_is_read(tmp_path, version):
    """A restart another netCDF writer made (CDF-1 or CDF-2, several record
    variables and two records, time in days, variables and attributes the
    library does not use) is read from its first record; a tracer the file
    lacks is left alone."""
    cfg = bc_config()
    st = g.make_ic(cfg, 2, 5, 1.0)
    path = str(tmp_path / "other.nc")
    with netcdf(path, "w", version=version) as w:
        w.title = "written by another netCDF writer"
        for d, n in (("time", None), ("lon", 72), ("lat", 37), ("ilon", 72), ("ilat", 36), ("lev", 26)):
            w.createDimension(d, n)
        tv = w.createVariable("time", "d", ("time",))
        tv.units = "days since 1990-01-01"
        tv[0] = 1.25
        tv[1] = 2.5
        extra = w.createVariable("unused", "f", ("lat", "lon"))
        extra.scale = np.float32(2.0)
        extra[:] = 1.0
        w.createVariable("counts", "i", ("time",))[:] = [3, 4]
        for name, (key, dims, _, _) in RESTART_BC.items():
            var = w.createVariable(name, "d", dims)
            var[0] = st[key] * 1.5
            var[1] = st[key] * 9.0   # a second record, not read
        qv = w.createVariable("q2", "d", ("time", "lev", "lat", "lon"))
        qv[0] = st["q"][1] * 2
        qv[1] = 0.0
    t, back = g.restart_read_host(cfg, path)
    assert t == 1.25 * 86400
    for name, (key, _, _, _) in RESTART_BC.items():
        assert np.array_equal(back[key], st[key] * 1.5), name
    assert np.isnan(back["q"][0]).all()                       # q1 absent: untouched
    assert np.array_equal(back["q"][1], st["q"][1] * 2)


def test_file_errors(tmp_path):
    cfg = bc_config()
    st = g.make_ic(cfg, 2, 5, 1.0)
    with pytest.raises(GmcError) as e:
        g.restart_write_host(cfg, tmp_path / "a.nc", 0.0, st, time_units="fortnights")
    assert e.value.code == abi.GMC_EINVAL
    with pytest.raises(GmcError) as e:
        g.restart_write_host(cfg, tmp_path / "a.nc", 0.0, st, tracer_names="only_one")
    assert e.value.code == abi.GMC_EINVAL
    with pytest.raises(GmcError) as e:
        g.restart_write_host(cfg, tmp_path / "no_such_dir" / "a.nc", 0.0, st)
    assert e.value.code == abi.GMC_EIO
    with pytest.raises(GmcError) as e:
        g.restart_read_host(cfg, tmp_path / "missing.nc")
    assert e.value.code == abi.GMC_EIO
    (tmp_path / "junk.nc").write_bytes(b"not a netCDF file at all")
    with pytest.raises(GmcError) as e:
        g.restart_read_host(cfg, tmp_path / "junk.nc")
    assert e.value.code == abi.GMC_EIO
    # a file of another grid is refused, not read into this one
    small = abi.default_config(nlon=36, nlat=19, nlev=26, baroclinic=1, dt_dyn=600.0,
                               vert_coord_template=abi.VCOORD_TEST_L26, max_wave_speed=400.0)
    g.restart_write_host(small, tmp_path / "small.nc", 0.0, g.make_ic(small, 2, 1, 1.0))
    with pytest.raises(GmcError) as e:
        g.restart_read_host(cfg, tmp_path / "small.nc")
    assert e.value.code == abi.GMC_EIO and "does not match this grid" in str(e.value)
    # a truncated file is refused
    full = open(tmp_path / "small.nc", "rb").read()
    (tmp_path / "cut.nc").write_bytes(full[: len(full) // 2])
    with pytest.raises(GmcError):
        g.restart_read_host(small, tmp_path / "cut.nc")


@pytest.mark.parametrize("steps_before", [2, 3])
def test_restart_continues_the_run_bit_for_bit_on_the_oracle(tmp_path, steps_before):
    """restart_write -> restart_read -> prepare continues the dynamics exactly
    as the uninterrupted run (the oracle restates the reference's run loop)."""
    cfg = bc_config()
    a = Oracle(cfg)
    load_state(a, g.make_ic(cfg, 2, 9, 1.0))
    a.prepare()
    a.step(steps_before)
    snap = {k: a.get_field(k) for k in ("u_lon", "v_lat", "pt", "phs", "gzs")}
    snap["q"] = np.stack([a.get_tracer(l) for l in range(cfg.ntracer)])
    g.restart_write_host(cfg, tmp_path / "r.nc", steps_before * cfg.dt_dyn, snap)
    t, back = g.restart_read_host(cfg, tmp_path / "r.nc")
    assert t == steps_before * cfg.dt_dyn
    b = Oracle(cfg)
    load_state(b, back)
    b.prepare()
    a.step(3)
    b.step(3)
    for f in ("u_lon", "v_lat", "pt", "phs"):
        assert np.array_equal(a.get_field(f), b.get_field(f)), f
    a.close()
    b.close()


def test_file_structs_match_the_header():
    assert C.sizeof(abi.FileOpts) == 5 * C.sizeof(C.c_void_p)   # four strings, an int32 and padding
    assert abi.FileOpts.background.offset == 4 * C.sizeof(C.c_void_p)
    assert C.sizeof(abi.RestartArrays) == 7 * C.sizeof(C.c_void_p)
    assert abi.STATUS_NAMES[abi.GMC_EIO] == "GMC_EIO"
