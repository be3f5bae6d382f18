"""The N > 1 path of bench.py (independent replicas, one process per GPU)
as two gloo ranks on CPU: the barrier and the maximum of the timed region
over ranks, the whole-job throughput of the replicas, and the reference arm
running on rank 0 alone (the other ranks return without work or output)."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import importlib.util, json, os, sys
spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(sys.argv[1], "bench.py"))
bench = importlib.util.module_from_spec(spec)
spec.loader.exec_module(bench)
ranks = bench.Ranks("gloo")
ranks.barrier()
rank_ms = 100.0 + 25.0 * bench.RANK          # this rank's timed region
max_ms = ranks.max(rank_ms)
ms_per_step, value = bench.replica_throughput(max_ms, 4, bench.WORLD)
ranks.barrier()
ranks.close()
if bench.RANK != 0:
    bench.run_reference(None)                # returns at once off rank 0
print(json.dumps({"rank": bench.RANK, "world": bench.WORLD, "max_ms": max_ms,
                  "ms_per_step": ms_per_step, "value": value}))
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_agree_on_the_slowest_replica():
    port = str(free_port())
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=port)
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT, ROOT], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err
        lines = [ln for ln in out.splitlines() if ln.strip()]
        assert len(lines) == 1, out         # nothing but this rank's own line
        outs.append(json.loads(lines[0]))
    for r in outs:
        assert r["world"] == 2
        assert r["max_ms"] == 125.0         # the slower rank's time on both ranks
        assert r["ms_per_step"] == 125.0 / 4
        # both replicas advanced 4 steps of 180 s in 125 ms
        assert abs(r["value"] - 2 * 4 * 180.0 / 0.125) < 1e-9


def test_single_process_ranks_are_no_ops():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_single", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    if mod.WORLD != 1:
        return
    r = mod.Ranks("gloo")
    r.barrier()
    assert r.max(3.5) == 3.5
    r.close()
    assert mod.replica_throughput(90.0, 2, 1) == (45.0, 2 * 180.0 / 0.09)
