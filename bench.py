"""Benchmark of the GMCORE dynamics step on GB300.

Workload (the headline configuration): hydrostatic dry baroclinic core at
0.5 degrees (720 x 360), 32 hybrid levels (wrf_l32), 4 FFSL tracers,
dt = 180 s, seeded synthetic initial state (isothermal 300 K, 35 m/s
balanced jet, 1 K temperature noise, Gaussian-blob tracers).  A step is one
time_integrate (three forward-backward stages, divergence-free default
options, tracer advection).

Metric: simulated days per wall-clock day (SDPD) of the mixed FP32/FP64 form,
with the FP64 form, their ratio and the surface-pressure difference reported
beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs N independent replicas (one per GPU, launched by torchrun); the
value is the whole-job total.  `--impl reference` times the FP64 CPU
restatement of the reference on the host cores instead.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
LOCAL_RANK = int(os.environ.get("LOCAL_RANK", "0"))
WORLD = int(os.environ.get("WORLD_SIZE", "1"))
RANK = int(os.environ.get("RANK", "0"))
if WORLD > 1:
    # one GPU per rank; the library uses the first visible device
    _vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    _phys = _vis.split(",")[LOCAL_RANK] if _vis else str(LOCAL_RANK)
    os.environ["CUDA_VISIBLE_DEVICES"] = _phys
    PHYS_GPU = _phys
else:
    _vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    PHYS_GPU = _vis.split(",")[0] if _vis else "0"
for _p in (ROOT, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

SEED = 20240601
DT = 180.0
NTRACER = 4
METRIC = "sim days/wall-day at 0.5°L32: mixed vs FP64 GPU at stated err; adjoint/fwd cost"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def workload_config(precision):
    from gmcore_gb300 import abi
    # time_scheme wrfrk3 (the reference default) and a 400 m/s polar-filter
    # design speed: an isothermal 300 K atmosphere carries Lamb waves at
    # ~347 m/s, faster than the default 300 m/s the filter widths assume.
    return abi.default_config(nlon=720, nlat=360, nlev=32, baroclinic=1, dt_dyn=DT,
                              vert_coord_template=abi.VCOORD_WRF_L32, time_scheme=abi.TIME_WRFRK3,
                              max_wave_speed=400.0, ntracer=NTRACER, precision=precision)


def workload_keys():
    """The `config` object of both arms' JSON lines: the workload only (the
    arithmetic each arm computes in is its `dtype`/`precision`)."""
    return {"workload": "hydrostatic baroclinic 0.5deg 720x360 L32 (wrf_l32), 4 FFSL tracers, dt=180 s",
            "time_scheme": "wrfrk3", "max_wave_speed": 400.0, "steps_per_sim_day": 480,
            "l2": "inputs larger than L2 (state ~1.5 GB mixed, ~3 GB FP64)"}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# Algorithmic (compulsory) bytes of one launch of each kernel group, in units
# of N s (N = nlon nlat nlev cells, s = bytes of a bulk value), N 8 (FP64
# level fields) and H 8 (FP64 surface fields): the fields the group must read
# and write once.  The FFSL kernels count their own inputs and outputs
# (ffsl_inner_y: q, v, cfly, divy -> qy; ffsl_x2: q, qy, u, mfx, cflx, divx ->
# qx, fx; ffsl_hflx_y: qx, mfy, cfly -> fy).
KERNEL_BYTES = {
    "mass_flux": (4, 0, 0.5), "tangent_winds": (4, 0, 0.5), "kinetic_energy": (3, 0, 0), "pv": (3, 0, 0.5),
    "pv_edges": (7, 0, 0), "batch_cfl": (6, 0, 0), "column_mass": (4, 0, 1.5),
    "ffsl_x2": (8, 0, 0), "ffsl_inner_y": (5, 0, 0), "ffsl_hflx_y": (4, 0, 0),
    "pt_tendency": (6, 0, 0), "momentum_tend": (10, 0, 0.5), "update_phs": (0, 0, 4.5), "update_pt": (3, 0, 1),
    "column_backward": (2, 1, 2), "update_uv": (9, 1, 0), "div_damp": (7, 0, 0), "tracer_accum": (4, 0, 0),
    "tracer_batch_cfl": (6, 0, 0), "tracer_batch_cflz": (3, 0, 0),
    "tracer_horizontal": (4, 0, 1), "tracer_vertical": (4, 0, 0.5), "tracer_lon_damp": (0.3, 0, 0),
    "surface_rel": (0, 0, 1.5),
}
# groups that launch more than one kernel (not a single kernel's roofline)
MULTI_KERNEL = {"tracer_accum", "div_damp"}


def algorithmic_bytes(name, cfg, s):
    n = cfg.nlon * cfg.nlat * cfg.nlev
    h = cfg.nlon * cfg.nlat
    a, b, c = KERNEL_BYTES.get(name, (0, 0, 0))
    return a * n * s + b * n * 8 + c * h * 8


def step_compulsory_bytes(cfg, s, ntracer):
    """Compulsory HBM bytes of one step when every intermediate stays on chip:
    per stage the dynamics read/write 16 bulk fields (3 stages), tracers 2 per
    tracer plus 10 shared batch fields, plus ~18 FP64 surface fields."""
    n = cfg.nlon * cfg.nlat * cfg.nlev
    h = cfg.nlon * cfg.nlat
    return n * s * (48 + 2 * ntracer + 10) + 18 * h * 8


def measured_traffic(name):
    """DRAM bytes per launch of a kernel group from the committed ncu launch
    list summary (profiles/kernel_traffic_c2_mixed.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "kernel_traffic_c2_mixed.json")) as f:
            return json.load(f)["groups"].get(name)
    except Exception:
        return None


def fp64_flops_per_cell(name):
    """FP64 FLOP per cell of one launch of a kernel group of the FP64 form, from
    the committed ncu op counts (profiles/fp64_flops_c2.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "fp64_flops_c2.json")) as f:
            return json.load(f)["groups"].get(name)
    except Exception:
        return None


def mixed_ops(name):
    """Warp instructions, FP32 instructions and FLOP per launch of a kernel
    group of the mixed form, from the committed ncu counts
    (profiles/mixed_ops_c2.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "mixed_ops_c2.json")) as f:
            return json.load(f)["groups"].get(name)
    except Exception:
        return None


def issue_roof(prof, ms_per_step, sm_mhz, fp32_peak):
    """The roof that binds the mixed form: instruction issue.  Warp
    instructions of one step (ncu counts per launch x the launches the
    in-bench profile saw over its 3 steps) against the GPU's issue rate (4
    warp instructions per SM per cycle at the SM clock sampled during the
    timed region), and the step's FP32 FLOP against the measured FP32 FMA
    peak."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    inst = f32i = flop = covered = 0.0
    total = sum(ms for ms, _ in prof.values()) / 3.0
    for name, (ms, cnt) in prof.items():
        o = mixed_ops(name)
        if o is None:
            continue
        inst += o["warp_inst_per_launch"] * cnt / 3.0
        f32i += o["fp32_inst_per_launch"] * cnt / 3.0
        flop += o["fp32_flop_per_launch"] * cnt / 3.0
        covered += ms / 3.0
    if not inst:
        return None
    peak_issue = sms * 4 * sm_mhz * 1e6
    s = ms_per_step / 1000.0
    return {"bound": "issue", "warp_inst_per_step": inst, "achieved_warp_inst_per_s": inst / s,
            "peak_warp_inst_per_s": peak_issue, "frac": inst / s / peak_issue,
            "issue_floor_ms_per_step": inst / peak_issue * 1000.0,
            "fp32_inst_share": f32i / 32.0 / inst,
            "fp32_flop_per_step": flop, "fp32_tflops": flop / s / 1e12, "fp32_peak_tflops": fp32_peak,
            "fp32_frac": flop / s / 1e12 / fp32_peak if fp32_peak else None,
            "kernel_time_covered": covered / total if total else None,
            "sms": sms, "sm_mhz": sm_mhz,
            "source": "profiles/mixed_ops_c2.json (ncu instruction and FP32 op counts per launch); "
                      "peak issue = SMs x 4 x sampled SM clock; FP32 peak = gmc_fp32_fma_peak (measured in this run)"}


def state_bytes(state):
    return sum(a.nbytes for a in state.values())


class Ranks:
    """Coordination of the replicas (one process per GPU, each advancing its
    own copy of the workload; no collective on the data path): a barrier
    around the timed region and the maximum of a time over ranks.  With one
    process both are no-ops."""

    def __init__(self, backend="nccl"):
        self.dist = None
        self.device = "cuda" if backend == "nccl" else "cpu"
        if WORLD > 1:
            import torch
            import torch.distributed as dist
            if backend == "nccl":
                torch.cuda.set_device(0)
            dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x):
        if self.dist is None:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def replica_throughput(max_ms, steps, world):
    """(ms per step, whole-job simulated days per wall-day) of `world`
    replicas that each advanced `steps` steps of DT seconds, the slowest in
    max_ms milliseconds."""
    return max_ms / steps, DT * steps / (max_ms / 1000.0) * world


def run_ours(args):
    import gmcore_gb300 as g
    from gmcore_gb300 import abi

    ranks = Ranks("nccl")
    barrier, max_over_ranks = ranks.barrier, ranks.max

    cfg = workload_config(abi.PREC_MIXED)
    cfg64 = workload_config(abi.PREC_FP64)
    st = g.make_ic(cfg, 2, SEED, 1.0)

    # ---- device-resident timing of the mixed form ----
    model = g.Model(cfg)
    model.set_state(st)
    model.prepare()
    model.step(args.warmup)
    clocks = ClockSampler(PHYS_GPU)
    barrier()
    clocks.start()
    model.step(args.steps)            # synchronous; CUDA events on the context stream
    barrier()
    clk = clocks.stop()
    stats = model.stats()
    dev_ms = max_over_ranks(stats["step_ms"])
    ms_per_step, value = replica_throughput(dev_ms, args.steps, WORLD)
    launches_per_step = stats["kernel_launches"] / args.steps
    # state after warmup + steps, compared with the FP64 form below
    mixed_state = {name: model.get_field(name) for name in ("phs", "u_lon", "v_lat", "pt")}

    if args.device_only:
        model.close()
        if RANK == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "sim days/wall-day", "n_gpus": WORLD,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
                              "device_only": True}), flush=True)
        ranks.close()
        return

    # ---- end to end through the C ABI with host buffers ----
    def paged(x):
        a = g.page_aligned(np.shape(x))
        a[...] = x
        return a

    def e2e_run(m, nsteps, registered, exchange=False):
        """Wall time of nsteps steps through the public calls with host float64
        arrays: each step sets u, v, pt, phs and the tracers from the host,
        steps once and reads them back; the result feeds the next step.
        registered: the arrays are page-locked once (gmc_host_register, outside
        the timed region) and gathered/scattered/converted by device kernels
        over the host link; otherwise they are pageable and staged on host cores
        through the library's pinned buffer.  exchange: the same exchange as one
        gmc_step_io call per step (tracer inputs move during the dynamics, the
        fields move back during the tracer advection)."""
        host = {k: paged(v) for k, v in st.items()}
        out = {k: g.page_aligned(v.shape) for k, v in host.items() if k != "q"}   # touched: no page faults when timed
        qout = g.page_aligned(host["q"].shape)
        pinned_arrays = list(host.values()) + list(out.values()) + [qout] if registered else []
        for a in pinned_arrays:
            g.host_register(a)
        try:
            barrier()
            t0 = time.perf_counter()
            for _ in range(nsteps):
                if exchange:
                    m.step_io([(k, host[k]) for k in ("u_lon", "v_lat", "pt", "phs")] +
                              [(l, host["q"][l]) for l in range(NTRACER)], 1,
                              [(k, out[k]) for k in ("u_lon", "v_lat", "pt", "phs")] +
                              [(l, qout[l]) for l in range(NTRACER)])
                else:
                    for name in ("u_lon", "v_lat", "pt", "phs"):
                        m.set_field(name, host[name])
                    for l in range(NTRACER):
                        m.set_tracer(l, host["q"][l])
                    m.step(1)
                    for name in ("u_lon", "v_lat", "pt", "phs"):
                        m.get_field(name, out=out[name])
                    for l in range(NTRACER):
                        m.get_tracer(l, out=qout[l])
                for name in ("u_lon", "v_lat", "pt", "phs"):
                    host[name], out[name] = out[name], host[name]
                host["q"], qout = qout, host["q"]
            barrier()
            t = max_over_ranks(time.perf_counter() - t0)
        finally:
            for a in pinned_arrays:
                g.host_unregister(a)
        return t, sum(host[k].nbytes for k in ("u_lon", "v_lat", "pt", "phs", "q"))

    e2e_steps = max(2, min(args.steps, 10))
    e2e_staged_s, _ = e2e_run(model, e2e_steps, registered=False)
    e2e_sep_s, _ = e2e_run(model, e2e_steps, registered=True)
    # the exchange's step graphs (one per tracer-cadence phase) are captured
    # by untimed exchanges first; then the median of three timed runs, so that
    # one run that meets a host stall does not stand for the path
    e2e_run(model, 12, registered=True, exchange=True)
    runs = [e2e_run(model, e2e_steps, registered=True, exchange=True) for _ in range(3)]
    e2e_s, h2d = sorted(runs)[1]
    e2e_value = DT * e2e_steps / e2e_s * WORLD
    e2e_sep_value = DT * e2e_steps / e2e_sep_s * WORLD
    e2e_staged_value = DT * e2e_steps / e2e_staged_s * WORLD

    # ---- per-kernel device timing for the roofline ----
    model.set_profiling(True)
    model.step(3)
    prof = model.kernel_profile()
    model.set_profiling(False)
    total = sum(ms for ms, _ in prof.values())
    singles = {k: v for k, v in prof.items() if k not in MULTI_KERNEL}
    top = max(singles.items(), key=lambda kv: kv[1][0])
    top_name, (top_ms, top_n) = top
    per_launch_ms = top_ms / top_n
    alg = algorithmic_bytes(top_name, cfg, 4)
    peak, peak_kind = measured_peaks()
    achieved = alg / (per_launch_ms / 1000.0) / 1e9
    traffic = measured_traffic(top_name)
    b_step = step_compulsory_bytes(cfg, 4, NTRACER)
    # DRAM bytes of a step from the ncu traffic per launch of each group (the
    # profiled run covers 3 steps): the redundancy over the compulsory bytes and
    # the kernel-time-weighted DRAM throughput of the step's kernels
    ncu_bytes = 0.0
    covered_ms = 0.0
    for name, (ms, cnt) in prof.items():
        tb = measured_traffic(name)
        if tb is not None:
            ncu_bytes += tb * cnt / 3.0
            covered_ms += ms / 3.0
    ncell = cfg.nlon * cfg.nlat * cfg.nlev
    roof_issue = issue_roof(prof, ms_per_step, clk.get("sm_mhz") or 2070.0, g.fp32_fma_peak())

    # ---- one simulated day (480 steps) of the mixed form, device-timed ----
    one_day = None
    if not args.quick:
        m1 = g.Model(cfg)
        m1.set_state(st)
        m1.prepare()
        m1.step(args.warmup)
        clocks_day = ClockSampler(PHYS_GPU)
        barrier()
        clocks_day.start()
        m1.step(480)
        barrier()
        clk_day = clocks_day.stop()
        day_ms = max_over_ranks(m1.stats()["step_ms"])
        m1.close()
        one_day = {"steps": 480, "device_s": day_ms / 1000.0, "ms_per_step": day_ms / 480,
                   "value": DT * 480 / (day_ms / 1000.0) * WORLD, "unit": "sim days/wall-day", "clocks": clk_day}
    model.close()

    # ---- FP64 form on the same initial state ----
    m64 = g.Model(cfg64)
    m64.set_state(st)
    m64.prepare()
    m64.step(args.warmup)
    barrier()
    m64.step(args.steps)
    barrier()
    ms64 = max_over_ranks(m64.stats()["step_ms"]) / args.steps
    errors = {}
    for name, a in mixed_state.items():
        d = a - m64.get_field(name)
        scale = 100.0 if name == "phs" else 1.0   # phs in hPa
        errors[name] = {"rms": float(np.sqrt(np.mean(d * d)) / scale), "max": float(np.max(np.abs(d)) / scale),
                        "unit": "hPa" if name == "phs" else ("K" if name == "pt" else "m/s")}
    ps_rms_hpa = errors["phs"]["rms"]
    # the FP64 form end to end through the same calls (like-for-like with the
    # FP64 CPU reference arm)
    e2e64_steps = 5
    e2e_run(m64, 1, registered=True, exchange=True)   # graph capture
    e2e64_s, _ = e2e_run(m64, e2e64_steps, registered=True, exchange=True)
    e2e64_value = DT * e2e64_steps / e2e64_s * WORLD
    # the FP64 form's roofline: FP64 issue (its kernels keep the FP64 pipe
    # busy, profiles/fp64_form_c2.md); the dominant kernel's FLOP per launch
    # over its in-bench launch time, against the FMA peak measured now
    m64.set_profiling(True)
    m64.step(1)
    prof64 = m64.kernel_profile()
    m64.set_profiling(False)
    m64.close()
    fp64_roof = None
    singles64 = {k: v for k, v in prof64.items() if k not in MULTI_KERNEL}
    top64, (t64, n64) = max(singles64.items(), key=lambda kv: kv[1][0])
    fpc = fp64_flops_per_cell(top64)
    if fpc is not None:
        peak64 = g.fp64_fma_peak()
        flop = fpc["fp64_flop_per_cell"] * ncell
        ach64 = flop / (t64 / n64 / 1000.0) / 1e12
        fp64_roof = {"bound": "fp64", "kernel": top64, "achieved": ach64, "peak": peak64, "unit": "TFLOP/s",
                     "frac": ach64 / peak64, "fp64_flop_per_launch": flop, "avg_launch_ms": t64 / n64,
                     "fp64_pipe_busy_pct_ncu": fpc["fp64_pipe_pct"],
                     "peak_source": "gmc_fp64_fma_peak (measured in this run)",
                     "flop_source": "profiles/fp64_flops_c2.json (ncu FP64 op counts)"}

    adj = adjoint_cost() if RANK == 0 else None
    ens = ensemble_throughput() if RANK == 0 else None
    files = file_io(cfg, st) if RANK == 0 and not args.quick else None

    c5 = c5_leg(args) if RANK == 0 and not args.quick else None

    cpu = None
    if RANK == 0 and WORLD == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args, sample_steps=3, warm=1)

    if RANK == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "sim days/wall-day",
            "n_gpus": WORLD,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_per_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 bulk + f64 (rings, column sweeps, integrals, filter weights)",
            "data": "synthetic (seeded isothermal 300 K + balanced 35 m/s jet + 1 K noise, 4 Gaussian-blob tracers)",
            "config": workload_keys(),
            "precision": "mixed",
            "parallelism": f"replicas x{WORLD}" if WORLD > 1 else "single GPU",
            "fp64": {"ms_per_step": ms64, "value": DT / (ms64 / 1000.0) * WORLD,
                     "mixed_speedup": ms64 / ms_per_step, "ps_rms_diff_hpa_after_steps": ps_rms_hpa,
                     "steps_compared": args.warmup + args.steps, "mixed_minus_fp64": errors,
                     "e2e": {"value": e2e64_value, "unit": "sim days/wall-day", "steps": e2e64_steps,
                             "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
                             "path": "the exchange path of e2e (gmc_step_io, registered arrays), FP64 form"},
                     "roofline": fp64_roof},
            "e2e": {"value": e2e_value, "unit": "sim days/wall-day", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": h2d, "steps": e2e_steps, "runs": "median of 3",
                    "path": "one gmc_step_io call per step (u, v, pt, phs and the tracers in, the same out; host "
                            "float64 arrays page-locked once with gmc_host_register): tracer inputs move during the "
                            "dynamics, the fields move back during the tracer advection",
                    "separate_calls_value": e2e_sep_value,
                    "separate_calls_path": "gmc_set_field/gmc_set_tracer + gmc_step(1) + gmc_get_field/gmc_get_tracer "
                                           "on the same registered arrays (device-side gather/convert)",
                    "pageable_value": e2e_staged_value,
                    "pageable_path": "same calls on pageable host arrays (host-side gather/convert into the "
                                     "library's pinned staging buffer)"},
            "gpu_launches": int(round(launches_per_step * args.steps)),
            "roofline": {"bound": "hbm", "kernel": top_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": alg, "avg_launch_ms": per_launch_ms,
                         "share_of_step": top_ms / total if total else None,
                         "traffic_source": "profiles/kernel_traffic_c2_mixed.json (ncu dram__bytes per launch)"},
            "step_roofline": {"compulsory_bytes_per_step": b_step, "achieved_gbs": b_step / (ms_per_step / 1000.0) / 1e9,
                              "frac": b_step / (ms_per_step / 1000.0) / 1e9 / peak,
                              "note": "all intermediates on chip; 16 N s per stage, 2 N s per tracer, 10 N s batch",
                              "ncu_dram_bytes_per_step": ncu_bytes,
                              "redundancy": ncu_bytes / b_step,
                              "kernel_time_weighted_dram_frac": (ncu_bytes / (covered_ms / 1000.0) / 1e9 / peak
                                                                 if covered_ms else None),
                              "issue": roof_issue},
            "cell_updates_per_s": ncell * args.steps / (dev_ms / 1000.0) * WORLD,
            "kernel_ms_per_step": {k: round(v[0] / 3.0, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
            "clocks": clk,
        }
        if adj is not None:
            line["adjoint"] = adj
        if ens is not None:
            line["ensemble"] = ens
        if cpu is not None:
            line["cpu_baseline"] = cpu
        if one_day is not None:
            line["one_day"] = one_day
        if files is not None:
            line["files"] = files
        if c5 is not None:
            line["c5"] = c5
        print(json.dumps(line), flush=True)
    ranks.close()


def file_io(cfg, st, reps=3):
    """History and restart files of the workload's state (0.5 deg L32, 4
    tracers, mixed form): wall time of gmc_restart_write, gmc_restart_read
    and gmc_history_write (best of `reps`; each moves the state over the host
    link, converts it to FP64 big-endian and writes or reads the netCDF file
    in the host's temporary directory), and the file sizes."""
    import shutil
    import tempfile
    import gmcore_gb300 as g
    m = g.Model(cfg)
    m.set_state(st)
    m.prepare()
    m.step(3)
    d = tempfile.mkdtemp(prefix="gmc_files_")
    r0, h0 = os.path.join(d, "c2.r0.nc"), os.path.join(d, "c2.h0.nc")

    def best(f):
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            f()
            ts.append(time.perf_counter() - t0)
        return min(ts)

    try:
        tw = best(lambda: m.restart_write(r0, 540.0))
        th = best(lambda: m.history_write(h0, 540.0))
        tr = best(lambda: m.restart_read(r0))
        rb, hb = os.path.getsize(r0), os.path.getsize(h0)
        m.prepare()
        # a history record every 6 simulated hours (120 steps of 180 s) in the
        # background, against the same steps without output: what the output
        # costs the run
        m.step(40)
        t0 = time.perf_counter()
        m.step(120)
        t_steps = time.perf_counter() - t0
        t0 = time.perf_counter()
        m.history_write(h0, 540.0, background=True)
        t_call = time.perf_counter() - t0
        m.step(120)
        m.output_wait()
        t_bg = time.perf_counter() - t0
    finally:
        m.close()
        shutil.rmtree(d, ignore_errors=True)
    return {"restart_bytes": rb, "restart_write_s": tw, "restart_write_gbs": rb / tw / 1e9,
            "restart_read_s": tr, "restart_read_gbs": rb / tr / 1e9,
            "history_bytes": hb, "history_write_s": th, "history_write_gbs": hb / th / 1e9,
            "history_background": {"call_returns_s": t_call, "steps": 120, "steps_alone_s": t_steps,
                                   "steps_with_write_s": t_bg, "output_cost_s": t_bg - t_steps},
            "where": "netCDF classic (CDF-2) files in the host's temporary directory, best of %d; background: "
                     "snapshot in HBM, the write on a host thread while 120 steps run" % reps}


def adjoint_cost():
    """Cost of the adjoint relative to the forward model on the shallow-water
    adjoint case (1 degree 360x180, predict-correct, dt = 60 s, 96 steps,
    checkpoint every 8 steps, FP64): wall time of gmc_adjoint (which runs the
    checkpointed forward sweep itself) over wall time of gmc_step(96)."""
    import gmcore_gb300 as g
    from gmcore_gb300 import abi
    cfg = abi.default_config(nlon=360, nlat=180, nlev=1, baroclinic=0, dt_dyn=60.0, time_scheme=abi.TIME_PC2)
    st = g.make_ic(cfg, 1, SEED, 0.0)
    nsteps, ckpt = 96, 8
    lam = {"u_lon": np.zeros((1, cfg.nlat, cfg.nlon)), "v_lat": np.zeros((1, cfg.nlat - 1, cfg.nlon)),
           "gz": np.ones((cfg.nlat, cfg.nlon))}

    # one context per kind, re-prepared before every call, as an assimilation
    # loop would do (device buffers and captured graphs persist)
    models = {}

    def timed(kind):
        m = models.get(kind)
        if m is None:
            m = models[kind] = g.Model(cfg)
        m.set_state(st)
        m.prepare()
        t0 = time.perf_counter()
        if kind == "fwd":
            m.step(nsteps)
        else:
            m.adjoint(nsteps, lam, ckpt_every=ckpt)
        return time.perf_counter() - t0

    timed("fwd"), timed("adj")   # warm-up (allocation, graph capture)
    fwd = min(timed("fwd") for _ in range(3))
    adj = min(timed("adj") for _ in range(3))
    for m in models.values():
        m.close()
    return {"config": "shallow water 1deg 360x180, pc2, dt=60 s, 96 steps, checkpoint every 8, fp64",
            "forward_ms": fwd * 1e3, "adjoint_ms": adj * 1e3, "adjoint_over_forward": adj / fwd,
            "note": "wall time per call on a re-prepared context; the adjoint includes its checkpointed forward sweep"}


def ensemble_throughput(steps=10, warmup=3):
    """Batched ensembles (mixed FP32/FP64, test_l26, wrfrk3): 48 members at
    2 degrees (180x90x26, dt = 600 s) and 16 members at 1 degree (360x180x26,
    dt = 300 s), members differing by seeded 0.1 K temperature noise, each
    ensemble one context (members on forked streams, steps replayed as CUDA
    graphs).  Device time per step of the whole ensemble and member
    simulated days per wall-day."""
    import gmcore_gb300 as g
    from gmcore_gb300 import abi
    out = []
    for nlon, nlat, members, dt in ((180, 90, 48, 600.0), (360, 180, 16, 300.0)):
        kw = dict(nlon=nlon, nlat=nlat, nlev=26, baroclinic=1, dt_dyn=dt, vert_coord_template=abi.VCOORD_TEST_L26,
                  time_scheme=abi.TIME_WRFRK3, max_wave_speed=400.0, precision=abi.PREC_MIXED)
        base = abi.default_config(**kw)
        m = g.Model(abi.default_config(n_members=members, **kw))
        for mem in range(members):
            m.set_state(g.make_ic(base, 2, SEED + mem, 0.1), member=mem)
        m.prepare()
        m.step(warmup)
        for _ in range(40):   # the launch-layout autotuner times its candidates on the first steps
            if m.stats()["layout_tuned"]:
                break
            m.step(1)
        m.step(steps)
        st = m.stats()
        ms = st["step_ms"] / steps
        m.close()
        out.append({"grid": f"{nlon}x{nlat}x26", "members": members, "dt": dt, "steps": steps,
                    "ms_per_step": ms, "member_sdpd": members * dt / (ms / 1000.0),
                    "member_layout": st["member_layout"], "layout_tuned": st["layout_tuned"]})
    return out


def cpu_baseline(args, sample_steps=3, warm=1):
    """FP64 CPU restatement of the reference (the oracle, OpenMP build) on
    the same workload, timed on the host cores.  Its initial state comes from
    the oracle's own build, so this leg loads no library of the product.  The
    first step after the prologue skips tracer advection (adv_mod.F90:166), so
    `warm` >= 1 untimed steps put every timed step on the full path."""
    from gmcore_gb300 import abi   # ctypes structures only
    import oracle as orc_mod
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    cfg = workload_config(abi.PREC_FP64)
    st = orc_mod.make_ic(cfg, 2, SEED, 1.0, variant="omp")
    o = orc_mod.Oracle(cfg, variant="omp")
    for name, a in st.items():
        if name == "q":
            for l in range(a.shape[0]):
                o.set_tracer(l, a[l])
        else:
            o.set_field(name, a)
    o.prepare()
    if warm:
        o.step(warm)
    t0 = time.perf_counter()
    o.step(sample_steps)
    dt_s = time.perf_counter() - t0
    o.close()
    return {"value": DT * sample_steps / dt_s, "unit": "sim days/wall-day", "cores": int(os.environ["OMP_NUM_THREADS"]),
            "kind": "port",
            "sample": f"{sample_steps} step(s) of the same 0.5deg L32 4-tracer workload after the run prologue and "
                      f"{warm} untimed step(s), so every timed step advects the tracers",
            "s_per_step": dt_s / sample_steps}


def run_reference(args):
    if RANK != 0:
        return
    cpu = cpu_baseline(args, sample_steps=args.steps, warm=max(1, args.warmup))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": cpu["value"],
        "unit": "sim days/wall-day",
        "n_gpus": WORLD,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": cpu["s_per_step"] * 1000.0,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded isothermal 300 K + balanced 35 m/s jet + 1 K noise, 4 Gaussian-blob tracers)",
        "config": workload_keys(),
        "precision": "fp64",
        "implementation": "FP64 C++ restatement of the reference, OpenMP on the host cores (the reference's "
                          "Fortran/MPI build cannot be compiled here)",
        "cpu_baseline": cpu,
        "e2e": {"value": cpu["value"], "unit": "sim days/wall-day", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def c5_leg(args, steps=10):
    """The high-resolution case (0.25 degrees 1440x720, 64 levels wrf_l64,
    8 FFSL tracers, dt = 60 s): the mixed form device-timed over `steps` steps
    after 3 warm-up steps, the FP64 form over 3 steps, and their RMS
    differences after those 3 steps (the mixed state is read after its warm-up
    steps)."""
    import gmcore_gb300 as g
    from gmcore_gb300 import abi

    def cfg_of(prec):
        return abi.default_config(nlon=1440, nlat=720, nlev=64, baroclinic=1, dt_dyn=60.0,
                                  vert_coord_template=abi.VCOORD_WRF_L64, time_scheme=abi.TIME_WRFRK3,
                                  max_wave_speed=400.0, ntracer=8, precision=prec)
    st = g.make_ic(cfg_of(abi.PREC_MIXED), 2, SEED, 1.0)
    fields = ("phs", "u_lon", "pt")
    m = g.Model(cfg_of(abi.PREC_MIXED))
    m.set_state(st)
    m.prepare()
    m.step(3)
    s_m = {f: m.get_field(f) for f in fields}
    m.step(steps)
    ms_m = m.stats()["step_ms"] / steps
    m.close()
    m = g.Model(cfg_of(abi.PREC_FP64))
    m.set_state(st)
    m.prepare()
    m.step(3)
    ms_d = m.stats()["step_ms"] / 3
    s_d = {f: m.get_field(f) for f in fields}
    m.close()
    n, h = 1440 * 720 * 64, 1440 * 720
    b_step = n * 4 * (48 + 2 * 8 + 10) + 18 * h * 8
    return {"workload": "hydrostatic baroclinic 0.25deg 1440x720 L64 (wrf_l64), 8 FFSL tracers, dt=60 s, wrfrk3, "
                        "max_wave_speed 400",
            "value": 60.0 / (ms_m / 1000.0), "unit": "sim days/wall-day", "steps": steps, "ms_per_step": ms_m,
            "cell_updates_per_s": n / (ms_m / 1000.0),
            "fp64": {"ms_per_step": ms_d, "value": 60.0 / (ms_d / 1000.0), "mixed_speedup": ms_d / ms_m},
            "mixed_minus_fp64_rms_after_3_steps": {f: float(np.sqrt(np.mean((s_m[f] - s_d[f]) ** 2))) for f in fields},
            "step_roofline": {"compulsory_bytes_per_step": b_step,
                              "frac": b_step / (ms_m / 1000.0) / 1e9 / measured_peaks()[0]}}


def run_c5(args):
    """The high-resolution case alone, as its own JSON line."""
    c5 = c5_leg(args, steps=args.steps)
    line = {"metric": "sim days/wall-day at 0.25°L64, 8 tracers: mixed vs FP64 GPU", "value": c5["value"],
            "unit": "sim days/wall-day", "n_gpus": 1, "steps": args.steps, "ms_per_step": c5["ms_per_step"],
            "higher_is_better": True, "dtype": "f32 bulk + f64 (rings, surface pressure, integrals)",
            "data": "synthetic (seeded)", "config": {"workload": c5["workload"]}, "c5": c5}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--device-only", action="store_true",
                    help="time only the device-resident mixed step (the case profiled under ncu)")
    ap.add_argument("--workload", choices=("c2", "c5"), default="c2",
                    help="c2: 0.5deg L32 4 tracers (headline); c5: 0.25deg L64 8 tracers")
    ap.add_argument("--quick", action="store_true",
                    help="leave out the one-day and 0.25deg legs (extra keys of the headline line)")
    args = ap.parse_args()
    if args.workload == "c5":
        run_c5(args)
        return
    if args.impl == "reference":
        if args.steps > 3:
            log("reference arm: each step of the CPU restatement takes seconds; timing", args.steps, "steps")
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
