"""Benchmark of the photon-tracing / photon-mapping waveform path on one GB300.

One step = one full pass of the hot path over one batch of photons, exactly what
``run_linear`` does: forward trace of N_f photons (photon maps), map build, backward trace
of N_b = N_f / 4 photons with a k = 100 nearest-neighbour gather at every backward event
into the time-binned waveform. The workload is the large single-instance configuration
(400 m, 20 m water, a = 0.10, b = 0.40, FF phase function, GGX alpha 0.10, albedo 0.20,
FOV 50 mrad, 0.05 ns bins, 1e8 forward photons, Philox seed 1).

Prints one JSON line (rank 0). ``--impl reference`` times the CPU restatement of the
reference's algorithm (the oracle, all host threads) on a bounded sample of the same
workload instead, and once, on a fixed subset, the reference's own ``run_linear`` and
``run_parallel`` (installed unmodified under ``baseline/_ref``).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "photons/s & waveform-grads/s on 1 GB300: batched+adjoint vs plain @≤1% L1"
UNIT = "photons/s"
ALG_BYTES_PER_GATHER = 16 + 100 * 32  # query record + k neighbour records (pos 12, dir 12, E 4, t 4)
# DRAM bytes per scatter-map query measured by ncu on the same kernel (dram__bytes_read.sum +
# dram__bytes_write.sum of one k_gather<1, 0> launch / its queries; 1e6-photon case of this scene)
DRAM_BYTES_PER_SCATTER_QUERY = 893
# Warp instructions per scatter-map query of the same capture (smsp__inst_executed.sum of one
# k_gather<1, 0> launch / its queries): the kernel is bound by instruction issue, so its issue
# rate is reported beside the HBM convention
INST_PER_SCATTER_QUERY = 4615


def workload_config(name: str):
    from pyalbsim_gb300.workloads import workload_config as wc

    return wc(name)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.device = device
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits"],
                    capture_output=True, text=True, timeout=5,
                ).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 2 + i and r[2 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# Flop-equivalents per interaction event of the tracer (FMA = 2, special-function op = 1),
# the convention its FP32 roofline is quoted in.
F_EVENT = 64


def fp32_peak_tflops():
    """FP32 peak of the GPU: SMs x 128 FP32 lanes x 2 flop per FMA x the maximum SM clock
    (MEASURED_PEAKS.json's sm_max_mhz when present). Derived, not measured: the measured-peak
    file carries no FP32 figure."""
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = 2070.0
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            mhz = float(json.load(fh).get("sm_max_mhz", mhz))
    except Exception:
        pass
    return sms * 128 * 2 * mhz * 1e6 / 1e12, f"derived: {sms} SMs x 128 FP32 lanes x 2 x {mhz:.0f} MHz"


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def measured(fn, *args):
    """One of the line's secondary measurements; a failure is recorded in its place, so the
    timed headline numbers are still printed."""
    try:
        return fn(*args)
    except Exception as e:  # noqa: BLE001 - reported in the JSON line
        return {"error": f"{type(e).__name__}: {e}"}


def cpu_oracle_rate(cfg, nf, nb, seed, threads):
    """(photons/s, seconds) of the oracle on nf forward + nb backward photons (its k-d tree
    neighbour search, the exact answer scipy's KDTree gives the reference)."""
    from oracle.oracle import oracle_run
    from pyalbsim_gb300.scene import build_scene

    scene = build_scene(cfg)
    t0 = time.perf_counter()
    oracle_run(scene, nf, nb, seed=seed, threads=threads)
    dt = time.perf_counter() - t0
    return (nf + nb) / dt, dt


def cpu_model() -> str:
    """Host CPU model (lscpu's model name; /proc/cpuinfo or the platform as fallbacks)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform

    return platform.processor() or platform.machine()


def cpu_baseline_port(cfg, ns, threads):
    """The oracle on two sample sizes of the workload (ns/2 and ns forward photons, a quarter
    as many backward): photons/s of the larger and the ratio of the two rates, which shows
    whether the figure is a per-photon rate or depends on the sample chosen."""
    small_rate, small_dt = cpu_oracle_rate(cfg, ns // 2, max(ns // 8, 1), 8, threads)
    rate, dt = cpu_oracle_rate(cfg, ns, max(ns // 4, 1), 7, threads)
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "model": cpu_model(),
            "sample": f"{ns} forward + {max(ns // 4, 1)} backward photons ({dt:.1f} s), oracle/alb_oracle.c "
                      "(exact k-d tree k-NN)",
            "rate_at_half_sample": small_rate, "rate_ratio_full_over_half": rate / small_rate}


def _reference_config(cfg):
    """The reference's own SimulationConfig with the same field values as ``cfg`` (a
    configuration of this package's drop-in classes; the extension fields, absent from the
    reference, must be unset)."""
    import dataclasses
    import importlib

    classes = {}
    for mod in ("laser", "scene", "sensor", "sea_floor", "sea_surface", "heatmap", "water", "simulation", "run"):
        m = importlib.import_module(f"alb_sim.config.{mod}")
        classes.update({n: getattr(m, n) for n in dir(m) if dataclasses.is_dataclass(getattr(m, n))})
    prof = importlib.import_module("alb_sim.utils.parameter_profile")
    classes.update({n: getattr(prof, n) for n in ("LinearParameter", "ExponentialParameter")})

    def conv(obj):
        if dataclasses.is_dataclass(obj):
            cls = classes[type(obj).__name__]
            names = {f.name for f in dataclasses.fields(cls) if f.init}
            for f in dataclasses.fields(obj):
                if f.name not in names and f.init and getattr(obj, f.name) is not None:
                    raise ValueError(f"{type(obj).__name__}.{f.name} has no counterpart in the reference")
            return cls(**{f.name: conv(getattr(obj, f.name)) for f in dataclasses.fields(obj) if f.name in names})
        if isinstance(obj, tuple):
            return tuple(conv(x) for x in obj)
        return obj

    return conv(cfg)


def reference_python_rates(cfg, nf_linear, nb_linear, nf_parallel, nb_parallel, processes):
    """The reference's own CPU path, installed unmodified under baseline/_ref, on a fixed
    subset of the workload: ``run_linear`` (one process) and ``run_parallel`` (``processes``
    worker processes, one forward and one backward batch each; ``multiprocess`` is not
    installed, so the standard library's ``multiprocessing`` stands in for it). Photons/s of
    each; the workload's 1e8 + 2.5e7 photons would take the time these rates extrapolate to."""
    import contextlib
    import io
    import multiprocessing

    ref = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isdir(os.path.join(ref, "alb_sim")):
        return {"unavailable": "the reference is not installed under baseline/_ref"}
    if ref not in sys.path:
        sys.path.insert(0, ref)
    sys.modules.setdefault("multiprocess", multiprocessing)
    from alb_sim.config.run import RunConfig
    from alb_sim.execution.linear import run_linear
    from alb_sim.execution.parallel import run_parallel

    rcfg = _reference_config(cfg)
    out = {"model": cpu_model(), "code": "alb_sim (baseline/_ref), unmodified", "extrapolated": True}
    rc = RunConfig(photons_per_batch_forward=nf_linear, photons_per_batch_backward=nb_linear, batches_forward=1,
                   batches_backward=1)
    t0 = time.perf_counter()
    with contextlib.redirect_stdout(io.StringIO()):
        run_linear(rcfg, rc, rng=np.random.default_rng(5))
    dt = time.perf_counter() - t0
    out["run_linear"] = {"value": (nf_linear + nb_linear) / dt, "unit": UNIT, "cores": 1, "seconds": dt,
                         "sample": f"{nf_linear} forward + {nb_linear} backward photons"}
    rc = RunConfig(processes=processes, photons_per_batch_forward=nf_parallel,
                   photons_per_batch_backward=nb_parallel, batches_forward=processes, batches_backward=processes)
    t0 = time.perf_counter()
    with contextlib.redirect_stdout(io.StringIO()):
        run_parallel(rcfg, rc, seed=None)  # a fixed seed would make every batch identical
    dt = time.perf_counter() - t0
    n = processes * (nf_parallel + nb_parallel)
    out["run_parallel"] = {"value": n / dt, "unit": UNIT, "cores": processes, "seconds": dt,
                           "sample": f"{processes} x ({nf_parallel} forward + {nb_parallel} backward) photons"}
    return out


def run_reference(args):
    """The reference's algorithm on the host cores (the C oracle, all threads)."""
    import torch.distributed as dist  # noqa: F401

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg = workload_config(args.workload)
    threads = os.cpu_count() or 1
    nf = args.ref_photons
    nb = max(nf // 4, 1)
    for _ in range(args.warmup):
        cpu_oracle_rate(cfg, max(nf // 10, 100), max(nb // 10, 25), 11, threads)
    rates, times = [], []
    for s in range(args.steps):
        r, dt = cpu_oracle_rate(cfg, nf, nb, 100 + s, threads)
        rates.append(r)
        times.append(dt)
    value = float(np.median(rates))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.median(times)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload_label, "sample_forward_photons": nf, "sample_backward_photons": nb},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "model": cpu_model(),
                         "sample": f"{nf} forward + {nb} backward photons of the workload per step, "
                                   "step-by-step C restatement of the reference with an exact k-d tree "
                                   "k-NN (oracle/alb_oracle.c)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_reference_python:
        # the reference's own Python path, once, on a fixed subset (not part of `value`)
        line["reference_python"] = measured(
            reference_python_rates, cfg, args.ref_linear_photons, max(args.ref_linear_photons // 4, 1),
            args.ref_parallel_photons, max(args.ref_parallel_photons // 4, 1), threads)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large", choices=["large", "small"])
    ap.add_argument("--photons", type=float, default=1e8, help="forward photons per step (backward = 1/4)")
    ap.add_argument("--ref-photons", type=int, default=40000)
    ap.add_argument("--ref-linear-photons", type=int, default=1000,
                    help="forward photons of the reference's own run_linear (at least k records per map)")
    ap.add_argument("--ref-parallel-photons", type=int, default=250,
                    help="forward photons per worker of the reference's own run_parallel")
    ap.add_argument("--no-reference-python", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=60000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-gradients", action="store_true")
    ap.add_argument("--grad-photons", type=float, default=1e7)
    ap.add_argument("--precise", action="store_true", help="float64-geometry tracer instead of the float32 one")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--sweep-every", type=int, default=32,
                    help="run every n-th instance of the 4096-instance sweep (1 = the whole sweep)")
    ap.add_argument("--sweep-only", action="store_true", help="print only the sweep measurement")
    args = ap.parse_args()
    args.workload_label = (
        "large single instance: 400 m, 20 m water a=0.10 b=0.40 FF, GGX alpha 0.10, albedo 0.20, "
        "FOV 50 mrad, 0.05 ns bins, k=100" if args.workload == "large" else
        "small: 400 m, 5 m water a=0.05 b=0.20 FF, GGX alpha 0.05, albedo 0.15, FOV 20 mrad, 0.1 ns bins, k=100"
    )
    if args.impl == "reference":
        return run_reference(args)
    if args.sweep_only:
        print(json.dumps({"batched_sweep": sweep_measure(args.sweep_every)}), flush=True)
        return None

    import torch

    from pyalbsim_gb300.replicas import aggregate_rate, max_over_ranks, rank_info, replica_seed

    world, rank, local = rank_info()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from pyalbsim_gb300.config.gpu import GpuRunOptions
    from pyalbsim_gb300.engine import GpuEngine

    cfg = workload_config(args.workload)
    nf = int(args.photons)
    nb = max(nf // 4, 1)
    # replicas: every rank traces its own photons (no data-path exchange)
    eng = GpuEngine(cfg, GpuRunOptions(device=local, precise=args.precise))

    def step(s):
        eng.ctx.reset()
        eng.n_forward = eng.n_backward = 0
        eng.forward(nf, replica_seed(1, rank, s))
        eng.build_maps()
        eng.backward(nb, replica_seed(1, rank, s))

    for w in range(args.warmup):
        step(w)
    eng.ctx.phase_times(reset=True)
    launches0 = eng.ctx.stats()["launches"]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record()
        for s in range(args.steps):
            step(args.warmup + s)
        ev1.record()
        torch.cuda.synchronize()
    ms = max_over_ranks(ev0.elapsed_time(ev1), device="cuda")
    gstats = eng.ctx.stats()
    launches = gstats.pop("launches") - launches0
    phases, gathers = eng.ctx.phase_times(reset=True)
    wf = eng.waveform_array(f64=True)
    ms_step = ms / args.steps
    value = aggregate_rate(nf + nb, world, ms_step)

    # roofline of the dominant kernel, the scatter-map gather k_gather<1, 0>: HBM-bound by the
    # algorithmic convention (3216 B per query), timed with CUDA events around its launches
    n_gathers = int(gathers.sum())
    sc_ms, sc_calls = phases["gather_scatter"]
    sc_queries = int(gathers[1])
    peak, peak_kind = measured_peak_hbm()
    achieved = (sc_queries * ALG_BYTES_PER_GATHER) / (sc_ms / 1e3) / 1e9 if sc_ms > 0 else 0.0
    q_per_launch = sc_queries / sc_calls if sc_calls else 0.0
    top = max(phases, key=lambda p: phases[p][0])
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (Philox streams; no dataset)",
        "config": {"workload": args.workload_label, "forward_photons": nf, "backward_photons": nb,
                   "parallelism": f"replicas x{world}", "l2": "working set of GBs per step, far above L2"},
        "phases_ms_per_step": {p: v[0] / args.steps for p, v in phases.items()},
        "gathers_per_step": int(n_gathers / args.steps),
        "gathers_per_s": world * (n_gathers / args.steps) / (ms_step / 1e3),
        "dominant_phase": top,
        "roofline": {"bound": "hbm", "kernel": "k_gather<1, 0> (scatter map, k-NN)", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak if peak else None,
                     "traffic": DRAM_BYTES_PER_SCATTER_QUERY * q_per_launch,
                     "algorithmic_bytes_per_launch": ALG_BYTES_PER_GATHER * q_per_launch,
                     "launches_per_step": sc_calls / args.steps, "peak_source": peak_kind,
                     "traffic_source": "ncu dram bytes per query of a 1e6-photon capture, scaled to a launch"},
        "gpu_launches": int(launches),
        # interaction events (scatters, surface crossings, seafloor hits) of the last step's
        # forward and backward traces over the mean step time
        "interaction_events": {
            "value": world * (gstats["forward_events"] + gstats["events"]) / (ms_step / 1e3), "unit": "events/s",
            "per_step": gstats["forward_events"] + gstats["events"]},
        "last_step_counters": gstats,
        "tracer_roofline": tracer_roofline(gstats, phases, args.steps),
        "gather_issue_roofline": measured(gather_issue_roofline, sc_queries, sc_ms),
        "clocks": clk.summary(),
        "waveform_total": float(wf.sum()),
    }
    # the timed context holds the full photon maps: free it before the end-to-end run,
    # which builds its own
    eng.close()
    eng = None
    if rank == 0:
        # CPU baseline: the oracle on a bounded sample of the same workload, all host threads
        threads = os.cpu_count() or 1
        line["cpu_baseline"] = cpu_baseline_port(cfg, args.cpu_sample, threads)
        if not args.no_e2e:
            line["e2e"] = measured(e2e_measure, cfg, nf, nb)
        if not args.no_sweep:
            line["batched_sweep"] = measured(sweep_measure, args.sweep_every)
        if not args.no_gradients:
            line["gradients"] = measured(gradients_measure, int(args.grad_photons))
            line["gradients_batched"] = measured(batched_gradients_measure)
            line["gradient_check"] = measured(gradient_check_measure)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def sm_count_and_clock():
    """(SMs, maximum SM clock in MHz): the device's SM count, MEASURED_PEAKS.json's clock."""
    import torch

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = 2070.0
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            mhz = float(json.load(fh).get("sm_max_mhz", mhz))
    except Exception:
        pass
    return sms, mhz


def gather_issue_roofline(queries, ms, sms_mhz=None):
    """The scatter-map gather against instruction issue, the bound its counters show: warp
    instructions per second (INST_PER_SCATTER_QUERY x queries over its CUDA-event time)
    against one issue per scheduler per cycle (SMs x 4 schedulers x the maximum SM clock)."""
    sms, mhz = sms_mhz if sms_mhz is not None else sm_count_and_clock()
    peak = sms * 4 * mhz * 1e6
    achieved = INST_PER_SCATTER_QUERY * queries / (ms / 1e3) if ms > 0 else 0.0
    return {"bound": "issue", "kernel": "k_gather<1, 0> (scatter map, k-NN)", "achieved": achieved, "peak": peak,
            "unit": "warp instructions/s", "frac": achieved / peak if peak else None,
            "instructions_per_query": INST_PER_SCATTER_QUERY,
            "source": "instructions per query from the ncu capture of a 1e6-photon launch; peak derived: "
                      f"{sms} SMs x 4 schedulers x {mhz:.0f} MHz"}


def tracer_roofline(gstats, phases, steps):
    """FP32 roofline of the forward trace: the last step's interaction events x F_EVENT over
    the forward trace's CUDA-event time per step, against the FP32 peak."""
    fwd_ms = phases["trace_fwd"][0] / steps
    peak, source = fp32_peak_tflops()
    achieved = gstats["forward_events"] * F_EVENT / (fwd_ms / 1e3) / 1e12 if fwd_ms > 0 else 0.0
    return {"bound": "fp32", "kernel": "k_trace_fast<0> (forward trace)", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak if peak else None, "events_per_s": gstats["forward_events"] / (fwd_ms / 1e3),
            "flop_per_event": F_EVENT, "peak_source": source}


def gradients_measure(nf: int):
    """Waveform gradients per second: the MSE between the waveform and a target simulated at
    depth 12 m, a 0.08, b 0.30, g 0.90 (HG), albedo 0.18, GGX alpha 0.08, differentiated
    with respect to all six parameters at the point 10% above, nf forward + nf/4 backward
    photons (Philox seed 3), the large scene's geometry. One gradient = one adjoint run (five
    columns) + one depth run (common-random-number forward difference against the adjoint
    run's own waveform). Baseline: central differences of plain runs (12 runs per gradient +
    1 for the value). Accuracy is measured
    separately, in expectation over seeds (``gradient_check_measure``): on one seed a central
    difference of a, b or the depth jumps with every integrator step and neighbour set that
    its step moves, so a single-seed comparison says nothing about either estimate."""
    import dataclasses

    import torch

    from pyalbsim_gb300.adjoint import WaveformFunction, with_parameters
    from pyalbsim_gb300.batch import surface_gate
    from pyalbsim_gb300.config.gpu import GpuRunOptions
    from pyalbsim_gb300.engine import GpuEngine
    from pyalbsim_gb300.workloads import large

    nb = max(nf // 4, 1)
    truth = np.array([12.0, 0.08, 0.30, 0.90, 0.18, float(np.sqrt(0.08))])
    base = with_parameters(large(hg=0.9), truth)
    # a 200 ns window from 10 ns before the surface return: the same bins at every depth
    base = dataclasses.replace(base, waveform_gate=surface_gate(base))
    opts = GpuRunOptions(precise=False)

    def plain(cfg, seed):
        eng = GpuEngine(cfg, opts)
        try:
            eng.forward(nf, seed)
            eng.build_maps()
            eng.backward(nb, seed)
            return eng.waveform_array(f64=True)
        finally:
            eng.close()

    target = torch.from_numpy(plain(base, 1003))
    p0 = 1.1 * truth
    point = with_parameters(base, p0)

    def loss_of(w):
        return float(((w - target.numpy()) ** 2).sum())

    plain(point, 3)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    w_plain = plain(point, 3)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    p = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    t0 = time.perf_counter()
    w = WaveformFunction.apply(p, base, nf, nb, 3, opts)
    loss = ((w - target) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    grad = p.grad.numpy().copy()
    names = ["depth", "a", "b", "g", "albedo", "roughness"]
    return {
        "value": 1.0 / t_grad, "unit": "waveform-gradients/s (6 parameters, MSE loss)",
        "photons_per_run": nf + nb, "s_per_gradient": t_grad, "s_per_plain_run": t_plain,
        "fd_baseline": {"value": 1.0 / (13 * t_plain), "unit": "waveform-gradients/s",
                        "runs_per_gradient": 13},
        "speedup_vs_fd": (13 * t_plain) / t_grad,
        "gradient": dict(zip(names, grad.tolist())),
        "loss": loss_of(w.detach().numpy()),
        "config": "target at depth 12, a 0.08, b 0.30, g 0.90, albedo 0.18, alpha 0.08; evaluated +10%; "
                  "400 m, FOV 50 mrad, 0.05 ns bins in a 200 ns window at the surface return, k = 100, "
                  "fast tracer",
        "waveform_l1_vs_plain": float(np.abs(w.detach().numpy() - w_plain).sum() / max(np.abs(w_plain).sum(), 1e-300)),
    }


CHANNEL_NAMES = ("bottom", "scatter", "surface_reflection", "transmission_up")


def _check_table(out):
    table = {}
    for name, r in out.items():
        table[name] = {
            CHANNEL_NAMES[c]: {"rel_diff": round(r["rel_diff"][c], 5), "se": round(r["rel_diff_se"][c], 5)}
            for c in range(4) if np.isfinite(r["rel_diff"][c])
        }
    return table


def gradient_check_measure(seeds: int = 128, photons: int = 1_000_000, config3_seeds: int = 16):
    """Accuracy of the gradient columns against common-random-number central differences, in
    expectation over seeds (paired standard errors), three ways:

    * ``by_parameter``: ``adjoint.difference_check`` on the small scene with an HG layer
      (5 m water, a 0.05, b 0.20, g 0.90, albedo 0.15, GGX alpha 0.05), 1e6 + 2.5e5 photons
      per run, Philox seeds 100.., relative half-steps a, b 5%, g 2%, albedo and roughness
      1e-3;
    * ``config3``: the same at the adjoint workload's geometry and point (the large scene,
      HG, depth 12 m, a 0.08, b 0.30, g 0.90, albedo 0.18, GGX alpha 0.08, each +10%, a 200 ns
      window at the surface return), relative half-steps 1e-3 for every parameter;
    * ``depth_forward_vs_central``: the forward depth difference the gradients use against
      the central one, small scene, the bias of the O(h) step."""
    import dataclasses

    import torch

    from pyalbsim_gb300.adjoint import CHECK_STEPS, PARAMS, depth_difference_bias, difference_check, with_parameters
    from pyalbsim_gb300.batch import surface_gate
    from pyalbsim_gb300.workloads import large, small

    cfg = small(hg=0.9)
    nb = photons // 4
    difference_check(cfg, photons // 10, nb // 10, seeds=[1, 2])  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = difference_check(cfg, photons, nb, seeds=list(range(100, 100 + seeds)))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    result = {
        "by_parameter": _check_table(out), "seeds": seeds, "photons_per_run": photons + nb, "wall_s": wall,
        "steps": {PARAMS[i]: h for i, h in CHECK_STEPS.items()},
        "config": "small scene: 400 m, 5 m water a=0.05 b=0.20 HG g=0.90, albedo 0.15, GGX alpha 0.05, "
                  "FOV 20 mrad, 0.1 ns bins, k = 100; fast tracer; rel_diff = mean(column total - CRN "
                  "central difference) / |mean difference| over seeds, se its paired standard error",
    }
    truth = np.array([12.0, 0.08, 0.30, 0.90, 0.18, float(np.sqrt(0.08))])
    c3 = with_parameters(large(hg=0.9), 1.1 * truth)
    c3 = dataclasses.replace(c3, waveform_gate=surface_gate(c3))
    steps3 = {i: 1e-3 for i in range(1, 6)}
    t0 = time.perf_counter()
    out3 = difference_check(c3, photons, nb, seeds=list(range(300, 300 + config3_seeds)), steps=steps3)
    result["config3"] = {"by_parameter": _check_table(out3), "seeds": config3_seeds,
                         "photons_per_run": photons + nb, "steps": {PARAMS[i]: h for i, h in steps3.items()},
                         "wall_s": time.perf_counter() - t0}
    t0 = time.perf_counter()
    db = depth_difference_bias(cfg, photons, nb, seeds=list(range(500, 500 + 32)))
    result["depth_forward_vs_central"] = {
        CHANNEL_NAMES[c]: {"rel_bias": round(db["rel_bias"][c], 5), "se": round(db["rel_bias_se"][c], 5)}
        for c in range(4) if np.isfinite(db["rel_bias"][c])}
    result["depth_forward_vs_central"].update(step_m=db["step_m"], seeds=32, wall_s=time.perf_counter() - t0)
    return result


def batched_gradients_measure(n_targets: int = 16, photons: int = 1_000_000, streams: int = 4):
    """Batched form: six-parameter gradients of n_targets Latin-hypercube instances (seed 4)
    at 1e6 + 2.5e5 photons, small scene with an HG layer and a 400 ns window. One
    alb_batch_run holds, per target, the adjoint instance and one plain instance at depth + h
    (the depth column's forward difference). Baseline: the plain single-instance run of every
    target through the engine, one after another (their mean time), 13 runs per
    central-difference gradient."""
    import torch

    from pyalbsim_gb300.adjoint import with_parameters
    from pyalbsim_gb300.batch import Instance, run_batch
    from pyalbsim_gb300.config.gpu import GpuRunOptions
    from pyalbsim_gb300.engine import GpuEngine
    from pyalbsim_gb300.inversion import gated_base, hypercube_targets

    base = gated_base()
    nb = photons // 4
    pts = 1.1 * hypercube_targets(n_targets, seed=4)
    pts[:, 3] = np.minimum(pts[:, 3], 0.99)

    def instances():
        out = []
        for i, p in enumerate(pts):
            out.append(Instance(with_parameters(base, p), photons, nb, 3000 + i, p))
            q = p.copy()
            q[0] += max(0.01 * p[0], 0.01)
            out.append(Instance(with_parameters(base, q), photons, nb, 3000 + i, q))
        return out

    mask = [k % 2 == 0 for k in range(2 * n_targets)]  # Jacobians for the adjoint instances only
    run_batch(instances()[:4], streams=streams, adjoint=True, jacobian_mask=mask[:4])  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, _, st, _, _ = run_batch(instances(), streams=streams, adjoint=True, jacobian_mask=mask)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0

    def plain(p):
        eng = GpuEngine(with_parameters(base, p), GpuRunOptions(precise=False))
        try:
            eng.forward(photons, 5)
            eng.build_maps()
            eng.backward(nb, 5)
            eng.waveform_array(f64=True)
        finally:
            eng.close()

    plain(pts[0])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for p in pts:
        plain(p)
    torch.cuda.synchronize()
    t_plain = (time.perf_counter() - t0) / n_targets
    rate = n_targets / t_batch
    return {
        "value": rate, "unit": "waveform-gradients/s (6 parameters)", "instances": n_targets,
        "photons_per_run": photons + nb, "streams": streams, "failed": int((st != 0).sum()),
        "s_per_batch": t_batch, "s_per_plain_run_mean": t_plain,
        "fd_baseline": {"value": 1.0 / (13 * t_plain), "unit": "waveform-gradients/s", "runs_per_gradient": 13},
        "speedup_vs_fd": rate * 13 * t_plain,
        "config": "small scene (400 m, 0.1 ns bins), HG layer, 400 ns window, k = 100; Latin-hypercube "
                  "parameters (seed 4) +10%; per target one adjoint instance + one depth + h instance "
                  "(forward difference), fast tracer",
    }


def sweep_measure(every: int = 32, streams: int = 8):
    """The batched Latin-hypercube sweep (4096 instances, seed 2: depth 1-40 m, a, b, g,
    albedo, GGX alpha, FOV 10-60 mrad; photons log-uniform in [1e5, 1e7] per instance, a
    quarter as many backward; 400 m, 0.1 ns bins, k-NN, HG water) through one
    ``alb_batch_run``: every ``every``-th instance (all 4096 with every=1). Wall time,
    traced photons per wall second, failed instances. Also the concurrency gain on small
    instances: 64 instances of 1e5 photons on one worker against ``streams`` workers."""
    import torch

    from pyalbsim_gb300.batch import hypercube_instances, run_batch
    from pyalbsim_gb300.workloads import small

    base = small(hg=0.9)
    inst = hypercube_instances(base, 4096, seed=2)[::every]
    run_batch(inst[:2], streams=2)  # warm-up
    torch.cuda.synchronize()
    _, _, st, _, wall = run_batch(inst, streams=streams)
    photons = sum(x.n_forward + x.n_backward for x in inst)
    codes = {-1: "invalid", -2: "too_few_records_for_k", -3: "capacity", -4: "cuda", -5: "iteration_cap"}
    failed = {codes.get(int(c), str(int(c))): int((st == c).sum()) for c in np.unique(st) if c != 0}
    out = {"instances": len(inst), "of": 4096, "photons": int(photons), "wall_s": wall,
           "value": photons / wall, "unit": "photons/s", "failed": int((st != 0).sum()), "failed_by_status": failed,
           "streams": streams}
    smalls = hypercube_instances(base, 64, seed=7, photons=(1e5, 1e5 + 1))
    t1 = run_batch(smalls, streams=1)[4]
    tn = run_batch(smalls, streams=streams)[4]
    out["small_instances"] = {"instances": 64, "photons_each": int(smalls[0].n_forward), "wall_s_1_worker": t1,
                              f"wall_s_{streams}_workers": tn, "gain": t1 / tn}
    return out


def e2e_measure(cfg, nf, nb, repeats: int = 3):
    """Throughput through the public drop-in call run_linear (context creation, table
    upload, traces, gathers and the host copy of the float32 waveforms inside the clock):
    the median of ``repeats`` calls, each one timed step, with every call's rate listed."""
    from pyalbsim_gb300.config import RunConfig
    from pyalbsim_gb300.execution.linear import run_linear
    from pyalbsim_gb300.scene import build_scene

    import contextlib
    import io

    rc = RunConfig(photons_per_batch_forward=nf, photons_per_batch_backward=nb, batches_forward=1, batches_backward=1)
    rates = []
    for r in range(repeats):
        t0 = time.perf_counter()
        with contextlib.redirect_stdout(io.StringIO()):
            w = run_linear(cfg, rc, rng=np.random.default_rng(1 + r))
        rates.append((nf + nb) / (time.perf_counter() - t0))
    scene = build_scene(cfg)
    h2d = len(scene.layers) * (3 * 18000 * 8 + 18000 * 8)  # phase theta, cdf, slope, weight tables
    d2h = sum(a.nbytes for a in w.values())
    return {"value": float(np.median(rates)), "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "runs": rates}


if __name__ == "__main__":
    main()
