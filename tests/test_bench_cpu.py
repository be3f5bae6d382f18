"""bench.py parses and its command line answers without a GPU (the driver
runs it at round end; a syntax error there would lose the measurement)."""
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
