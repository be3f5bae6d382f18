"""The C-ABI library loads, exports every function include/gmcore_gpu.h
declares, validates its arguments without a GPU, and the structure layouts
match the header."""
import ctypes as C
import os
import re

import pytest

import gmcore_gb300 as g
from gmcore_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "gmcore_gpu.h")).read()
    return sorted(set(re.findall(r"\b(gmc_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = g.load()
    names = header_functions()
    assert "gmc_step" in names and "gmc_create" in names
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(g.EXPORTED) | {n for n in names if hasattr(lib, n)}


def test_config_default_matches_python_mirror():
    lib = g.load()
    c = abi.Config()
    lib.gmc_config_default(C.byref(c))
    d = abi.default_config()
    for name, _ in abi.Config._fields_:
        assert getattr(c, name) == getattr(d, name), name


def test_invalid_configs_are_rejected_before_any_device_work():
    bad = [dict(nlon=7), dict(nlat=3), dict(nlev=2, baroclinic=0), dict(baroclinic=1, nlev=30, vert_coord_template=32),
           dict(time_scheme=9), dict(pv_scheme=7), dict(ntracer=2), dict(use_div_damp=1, div_damp_order=3),
           dict(dt_dyn=0.0), dict(pv_scheme=abi.PV_TVD, tvd_limiter_type=5), dict(ffsl_flux_type=4)]
    for kw in bad:
        cfg = abi.default_config(**kw)
        with pytest.raises(g.GmcError) as e:
            g.Model(cfg)
        assert e.value.code == abi.GMC_EINVAL, kw


def test_null_arguments():
    lib = g.load()
    assert lib.gmc_create(None, None) == abi.GMC_EINVAL
    assert lib.gmc_step(None, 1) == abi.GMC_EINVAL
    assert lib.gmc_prepare(None) == abi.GMC_EINVAL
    assert lib.gmc_last_error(None) == b"null context"
    # the file calls
    assert lib.gmc_restart_write(None, 0, b"x.nc", 0.0, None) == abi.GMC_EINVAL
    assert lib.gmc_restart_read(None, 0, b"x.nc", None, None) == abi.GMC_EINVAL
    assert lib.gmc_history_write(None, 0, b"x.nc", 0.0, 0, None) == abi.GMC_EINVAL
    assert lib.gmc_output_wait(None) == abi.GMC_EINVAL
    err = C.create_string_buffer(128)
    assert lib.gmc_restart_write_host(None, b"x.nc", 0.0, None, None, err, len(err)) == abi.GMC_EINVAL
    assert err.value == b"null configuration"
    cfg = abi.default_config(nlon=36, nlat=19, nlev=1, baroclinic=0, dt_dyn=600.0)
    assert lib.gmc_restart_write_host(C.byref(cfg), None, 0.0, None, None, err, len(err)) == abi.GMC_EINVAL
    assert lib.gmc_restart_read_host(C.byref(cfg), None, None, None, None, None, 0) == abi.GMC_EINVAL
    bad = abi.default_config(nlon=7, nlat=19, nlev=1, baroclinic=0, dt_dyn=600.0)
    assert lib.gmc_restart_read_host(C.byref(bad), b"x.nc", None, None, None, err, len(err)) == abi.GMC_EINVAL
    assert b"nlon" in err.value


def test_no_gpu_means_an_error_not_a_fallback():
    """Without a usable CUDA device a context cannot be created: gmc_create
    returns GMC_ECUDA with the CUDA runtime's message and no CPU path runs."""
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    from helpers import baroclinic_config, swm_config
    for cfg in (swm_config(), baroclinic_config()):
        with pytest.raises(g.GmcError) as e:
            g.Model(cfg)
        assert e.value.code == abi.GMC_ECUDA
        assert "cuda" in str(e.value).lower()
