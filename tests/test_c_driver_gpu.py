"""A non-Python caller of the C ABI: tests/c_driver/step_driver.c, a plain C
host program built with gcc against include/gmcore_gpu.h and linked to the
library, runs the seeded state through create / set (halo'd column-major
arrays) / prepare / N steps / get / diagnose, each step one gmc_step_io
exchange through its registered halo'd arrays (the overlapped transfers with
row pitch and level stride), then writes a history record (in the background)
and a restart file.  Its output must match the FP64 oracle run on the same
state, as the Python-driven parity tests do, and its files must hold that
output."""
import os
import subprocess

import numpy as np
import pytest

from gmcore_gb300 import abi, make_ic
from oracle import Oracle

from helpers import load_state, rel_err

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_driver(tmp):
    from c_driver_build import build
    return build(tmp)


def run_driver(exe, tmp, kind, nlon, nlat, nlev, dt, scheme, ntr, prec, nsteps, seed):
    out = os.path.join(tmp, "state.bin")
    r = subprocess.run([exe, str(kind), str(nlon), str(nlat), str(nlev), str(dt), str(scheme), str(ntr), str(prec),
                        str(nsteps), str(seed), out], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return np.fromfile(out, dtype=np.float64)


@pytest.mark.parametrize("case", ["swm", "baroclinic"])
def test_c_driver_matches_oracle(tmp_path, case):
    tmp = str(tmp_path)
    exe = build_driver(tmp)
    if case == "swm":
        kind, nlon, nlat, nlev, dt, scheme, ntr, nsteps = 1, 72, 37, 1, 600.0, abi.TIME_PC2, 0, 6
        cfg = abi.default_config(nlon=nlon, nlat=nlat, nlev=1, baroclinic=0, dt_dyn=dt, time_scheme=scheme)
        names = [("u_lon", (nlev, nlat, nlon)), ("v_lat", (nlev, nlat - 1, nlon)), ("gz", (nlat, nlon))]
    else:
        kind, nlon, nlat, nlev, dt, scheme, ntr, nsteps = 2, 72, 37, 26, 120.0, abi.TIME_WRFRK3, 2, 4
        cfg = abi.default_config(nlon=nlon, nlat=nlat, nlev=nlev, baroclinic=1, dt_dyn=dt, time_scheme=scheme,
                                 vert_coord_template=nlev, max_wave_speed=400.0, ntracer=ntr)
        names = [("u_lon", (nlev, nlat, nlon)), ("v_lat", (nlev, nlat - 1, nlon)), ("pt", (nlev, nlat, nlon)),
                 ("phs", (nlat, nlon))]
    seed = 31
    raw = run_driver(exe, tmp, kind, nlon, nlat, nlev, dt, scheme, ntr, abi.PREC_FP64, nsteps, seed)
    got, off = {}, 0
    for name, shape in names:
        n = int(np.prod(shape))
        got[name] = raw[off:off + n].reshape(shape)
        off += n
    q = []
    for _ in range(ntr):
        n = nlev * nlat * nlon
        q.append(raw[off:off + n].reshape(nlev, nlat, nlon))
        off += n
    diag = raw[off:off + 8]
    assert off + 8 == raw.size

    orc = Oracle(cfg)
    load_state(orc, make_ic(cfg, kind, seed, 1.0))
    orc.prepare()
    orc.step(nsteps)
    errs = {name: rel_err(got[name], orc.get_field(name)) for name, _ in names}
    for l in range(ntr):
        errs[f"q{l}"] = rel_err(q[l], orc.get_tracer(l))
    d = orc.diagnose()
    orc.close()
    print(case, errs)
    assert max(errs.values()) <= 1e-11, errs
    assert abs(diag[0] - d["tm"]) <= 1e-11 * abs(d["tm"])
    # the history and restart files it wrote through the C ABI hold its final state
    from scipy.io import netcdf_file
    out = os.path.join(tmp, "state.bin")
    file_names = {"u_lon": "u", "v_lat": "v", "pt": "pt", "phs": "phs", "gz": "gz"}
    with netcdf_file(out + ".r0.nc", "r", mmap=False) as f:
        assert f.variables["time"][0] == dt * nsteps / 3600 and f.restart_interval == b"1 days"
        for name, shape in names:
            assert np.array_equal(f.variables[file_names[name]][0].reshape(shape), got[name]), name
        for l in range(ntr):
            assert np.array_equal(f.variables[f"q{l + 1}"][0], q[l])
    with netcdf_file(out + ".h0.nc", "r", mmap=False) as f:
        assert f.variables["te"][0] == diag[1] and f.variables["tpe"][0] == diag[6]
        assert np.array_equal(f.variables["u"][0].reshape(got["u_lon"].shape), got["u_lon"])
