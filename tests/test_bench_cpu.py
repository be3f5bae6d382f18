"""bench.py parses and its command line answers without a GPU (a syntax
error there would lose the measurement)."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_help_runs():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert "--impl" in r.stdout


def test_bench_byte_table_names_profiled_groups():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    for name in ("ffsl_x2", "ffsl_inner_y", "ffsl_hflx_y", "update_uv", "momentum_tend"):
        assert name in mod.KERNEL_BYTES, name


def test_page_aligned_arrays_own_their_pages():
    import mmap

    import numpy as np

    import gmcore_gb300 as g
    a, b = g.page_aligned((3, 5, 7)), g.page_aligned((11,))
    for x in (a, b):
        assert x.ctypes.data % mmap.PAGESIZE == 0
        assert x.dtype == np.float64 and not x.any()
    # the page after the end of one array is not the start of the other's
    end_a = a.ctypes.data + a.nbytes
    assert not (b.ctypes.data <= end_a < b.ctypes.data + b.nbytes)


def test_host_register_checks_its_argument_before_cuda():
    import numpy as np
    import pytest

    import gmcore_gb300 as g
    a = np.zeros((4, 6))[:, ::2]   # not contiguous
    with pytest.raises(ValueError):
        g.host_register(a)


def test_cpu_baseline_leg_loads_only_the_oracle():
    """The CPU baseline (and the reference arm built on it) builds its initial
    state with the oracle's own generator and times steps that advect the
    tracers; no library of the product is loaded in its process.  Run on a
    small grid in a fresh interpreter."""
    code = r'''
import importlib.util, json, sys
spec = importlib.util.spec_from_file_location("bench_mod", sys.argv[1])
b = importlib.util.module_from_spec(spec)
spec.loader.exec_module(b)
from gmcore_gb300 import abi
b.workload_config = lambda prec: abi.default_config(
    nlon=72, nlat=37, nlev=32, baroclinic=1, dt_dyn=180.0, vert_coord_template=abi.VCOORD_WRF_L32,
    time_scheme=abi.TIME_WRFRK3, max_wave_speed=400.0, ntracer=4, precision=prec)
class A:
    steps, warmup = 2, 1
r = b.cpu_baseline(A(), sample_steps=2, warm=1)
maps = open("/proc/self/maps").read()
print(json.dumps({"r": r, "product": "libgmcore_gpu" in maps, "oracle": "liboracle_omp" in maps}))
'''
    import json
    r = subprocess.run([sys.executable, "-c", code, os.path.join(ROOT, "bench.py")], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["oracle"] and not out["product"], out
    assert out["r"]["kind"] == "port" and out["r"]["value"] > 0
    assert "advects the tracers" in out["r"]["sample"]
