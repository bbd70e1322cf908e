#!/usr/bin/env python3
"""Throughput benchmark of the Active Model B+ step on GB300.

Metric: Gsite-updates/s of the explicit-Euler AMB+ step at 4096^2 (and its
fraction of the HBM roofline at 8 B per site-update).

Workload (synthetic, seeded): 4096 x 4096 periodic, dt=1e-3, dx=dy=1,
a=-0.25 b=0 c=0.25 kappa=1 zeta=-1 lambda=0.5 T=0.05, phi = -0.4 + 0.01 N(0,1)
(numpy seed 2024), Philox noise, FP32 field with bf16 Kahan residual (f32c).
One bench step = one ``Integrator.run(inner)`` call (``inner`` Euler steps,
default 100) on device-resident buffers; the L2 is flushed (256 MiB write)
before every timed step.

Keys beyond the base contract:
  e2e          same metric through the C handle (amb_integrator_*) with pinned
               float64 host buffers: set_field + run(inner) + get_field per step.
  roofline     step kernel: 8 B x sites per launch / CUDA-event launch time,
               against MEASURED_PEAKS.json hbm_gbs.
  cpu_baseline the reference's CPU scheme (test/tjhung_ambplus.h compiled on the
               host, serial) on a bounded sample; the OpenMP oracle port beside it.
  clocks       nvidia-smi samples during the timed region.

``--impl reference`` times the reference's CPU implementation of the step
(test/tjhung_ambplus.h compiled into oracle/_ref; the oracle port where it is not built).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "active-model-bplus_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Gsite-updates/s 4096^2 (%HBM peak); surrogate vs plain time-to-t at S(k) tol"
UNIT = "Gsite-updates/s"
BYTES_PER_SITE = 8  # algorithmic: read phi (4 B) + write phi (4 B), FP32 path


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--inner", type=int, default=100)
    ap.add_argument("--precision", choices=["f32c", "f32", "f64"], default="f32c")
    ap.add_argument("--kernel", choices=["auto", "tile", "sliding"], default="auto")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--temperature", type=float, default=0.05)
    ap.add_argument("--ensemble", action="store_true",
                    help="measure the batched ensemble workload (256 replicas of uneven sizes) instead")
    ap.add_argument("--learned", action="store_true",
                    help="learned coarse stepper vs plain FP32: time to --t-end on a 512^2 AMB+ field")
    ap.add_argument("--t-end", type=float, default=1000.0)
    ap.add_argument("--learned-seeds", type=int, default=10,
                    help="noise seeds per arm of the learned-vs-plain comparison (default line and --learned)")
    ap.add_argument("--no-learned", action="store_true",
                    help="leave the learned-vs-plain comparison out of the default bench line")
    ap.add_argument("--weights", default=os.path.join(PKG, "activemodelbplus", "weights", "fluxnet_k50.npz"))
    ap.add_argument("--learned-steps", type=int, default=0,
                    help="time N macro steps of the learned stepper on the 512^2 field (after 40 untimed)")
    ap.add_argument("--learned-launches", type=int, default=0,
                    help="profiling: N forward passes of the learned stepper's network on a 512^2 field")
    ap.add_argument("--seg-rows", type=int, default=0,
                    help="with --kernel sliding: row-segment height (e.g. the autotuner's choice, for profiling)")
    ap.add_argument("--pairs", type=int, default=0,
                    help="with --kernel sliding: warp pairs per CTA; with --kernel tile: 256-thread groups per CTA")
    ap.add_argument("--persistent", action="store_true",
                    help="with --kernel tile: all steps of a run in one cooperative launch")
    ap.add_argument("--tile-rows", type=int, default=32, choices=[32, 28],
                    help="with --kernel tile: output tile height (32 x 32 or 28 x 32 tiles)")
    ap.add_argument("--fused", action="store_true",
                    help="with --kernel sliding: one warp per strip runs every stage (--pairs counts warps)")
    ap.add_argument("--launches", type=int, default=0,
                    help="profiling driver: run this many bare step launches through the C ABI and exit")
    ap.add_argument("--sweep", action="store_true",
                    help="precision/bandwidth sweep: f64, f32c and f32 from one field at each --sweep-sizes, "
                         "--sweep-steps steps; throughput and max/RMS/S(k) error against the FP64 run")
    ap.add_argument("--sweep-sizes", default="4096,8192")
    ap.add_argument("--sweep-steps", type=int, default=10000)
    return ap.parse_args(argv)


def workload(args):
    return dict(ny=args.size, nx=args.size, dt=1e-3, dx=1.0, dy=1.0, a=-0.25, b=0.0, c=0.25, kappa=1.0,
                lamb=0.5, zeta=-1.0, T=args.temperature, phi0=-0.4, amp=0.01, seed=2024)


def initial_field(w, rank=0):
    rng = np.random.default_rng(w["seed"] + rank)
    return w["phi0"] + w["amp"] * rng.standard_normal((w["ny"], w["nx"]))


def config_of(args, w):
    return {
        "workload": f"AMB+ {w['ny']}x{w['nx']} periodic, dt=1e-3, a=-0.25 b=0 c=0.25 kappa=1 zeta=-1 lambda=0.5 "
                    f"T={w['T']}, phi0=-0.4+0.01N(0,1), Philox noise",
        "ny": w["ny"], "nx": w["nx"], "precision": args.precision, "kernel": args.kernel,
        "inner_steps": args.inner, "l2": "flushed before every timed step (256 MiB write)",
        "parallelism": f"replicas{args.gpus}",
    }


# ------------------------------------------------------------------ clocks

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=5)

    def summary(self):
        if not self.lines:
            return None
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ helpers

def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _profile_record():
    path = os.path.join(ROOT, "profiles", "step_kernel_traffic.json")
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def measured_traffic(args):
    """Per-launch DRAM bytes of the step kernel from the committed ncu summary, if any."""
    return _profile_record().get(f"{args.precision}_{args.size}")


def issue_roofline(args, value: float, sm_mhz):
    """The step kernel's own binding limit: issue slots. With S thread-instruction slots per
    output site (ncu: smsp__inst_executed x 32 / sites, committed with the profile), the GPU can
    issue at most SMs x 4 schedulers x 32 lanes x clock / S site-updates per second; frac is the
    measured rate against that limit."""
    slots = _profile_record().get(f"{args.precision}_{args.size}_slots_per_site")
    if not slots:
        return None
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = float(sm_mhz) if sm_mhz else 2070.0
    limit = sms * 4 * 32 * mhz * 1e6 / slots / 1e9
    return {"slots_per_site": slots, "sm_mhz": mhz, "limit_gsites": limit, "frac": value / limit}


def _timed_sample(run, sites: int, seconds: float):
    """Steps of ``run(n)`` sized to take about ``seconds``; returns (steps, wall seconds)."""
    t0 = time.perf_counter()
    run(1)
    t1 = time.perf_counter() - t0
    nsteps = int(max(1, min(200, round(seconds / max(t1, 1e-6)))))
    t0 = time.perf_counter()
    run(nsteps)
    return nsteps, time.perf_counter() - t0


def _params(w):
    import oracle
    return oracle.Params(dt=w["dt"], dx=w["dx"], dy=w["dy"], a=w["a"], b=w["b"], c=w["c"], kappa=w["kappa"],
                         lamb=w["lamb"], zeta=w["zeta"], T=w["T"])


def cpu_reference_runner(w):
    """The reference's own CPU scheme (test/tjhung_ambplus.h, -Ofast, serial, with its drand48
    noise at D = T) on this workload, as ``run(nsteps)``; None where it is not built or the
    workload is outside the scheme (it needs b = 0, a = -c, dx = dy)."""
    import oracle
    if oracle.reference_lib(fast=True) is None or w["b"] != 0 or w["a"] != -w["c"] or w["dx"] != w["dy"]:
        return None
    field = initial_field(w)

    def run(n):
        return oracle.tjhung_run_noisy(field, n, w["dt"], w["dx"], w["c"], w["kappa"], w["lamb"], w["zeta"],
                                       w["T"], seed=1, fast=True)
    return run


def cpu_port_runner(w, threads: int):
    """The oracle port (oracle/amb_oracle.c, OpenMP over ``threads``) with Philox noise, as ``run(nsteps)``."""
    import oracle
    field = initial_field(w)
    p = _params(w)

    def run(n):
        return oracle.run(field, p, n, noise="philox" if w["T"] else "none", seed=1, nthreads=threads)
    return run


def cpu_baseline(w, seconds: float = 10.0):
    """Time the reference's CPU scheme on the same workload on the host (bounded sample, serial
    like the scheme itself); the OpenMP oracle port on all host cores is reported beside it."""
    sites = w["ny"] * w["nx"]
    threads = os.cpu_count() or 1
    out = None
    ref = cpu_reference_runner(w)
    if ref is not None:
        n, dt = _timed_sample(ref, sites, seconds)
        out = {"value": n * sites / dt / 1e9, "unit": UNIT, "cores": 1, "kind": "reference",
               "sample": f"{n} Euler steps of the {w['ny']}x{w['nx']} workload ({dt:.1f} s); "
                         f"test/tjhung_ambplus.h compiled -Ofast on this host, serial, its own drand48 noise"}
    n, dt = _timed_sample(cpu_port_runner(w, threads), sites, seconds)
    port = {"value": n * sites / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} Euler steps of the {w['ny']}x{w['nx']} workload ({dt:.1f} s); "
                      f"oracle/amb_oracle.c (OpenMP) with Philox noise"}
    if out is None:
        return port
    out["port"] = port
    return out


def fp64_path(w, stencil, model, field, nsteps: int = 20):
    """The FP64 path (the parity path, 1e-12 against the reference) on the same workload: nsteps
    in one Integrator.run, CUDA events, after 3 untimed steps."""
    import torch
    from activemodelbplus.integrator import Integrator
    sim = Integrator(field, stencil, model, precision="f64", seed=1)
    sim.run(3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    sim._launch(nsteps)
    e1.record()
    e1.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    sites = w["ny"] * w["nx"]
    return {"value": nsteps * sites / sec / 1e9, "unit": UNIT, "dtype": "f64",
            "sample": f"{nsteps} steps of the {w['ny']}x{w['nx']} workload, tile kernel (512-thread CTAs), CUDA events"}


def reference_gpu_baseline(w, nsteps: int = 20):
    """The reference's own CUDA integrator (FP64, 3 launches per step) on this GPU, timed with
    CUDA events over nsteps of its run loop on the same workload."""
    import oracle
    if not oracle.ReferenceGpuIntegrator.available():
        return {"unavailable": "reference cubin not built (oracle/build.py needs the reference checkout)"}
    p = oracle.Params(dt=w["dt"], dx=w["dx"], dy=w["dy"], a=w["a"], b=w["b"], c=w["c"], kappa=w["kappa"],
                      lamb=w["lamb"], zeta=w["zeta"], T=w["T"])
    ref = oracle.ReferenceGpuIntegrator(initial_field(w), p, seed=1)
    try:
        ref.time_steps(3)
        ms = ref.time_steps(nsteps)
    finally:
        ref.close()
    sites = w["ny"] * w["nx"]
    return {"value": nsteps * sites / (ms / 1e3) / 1e9, "unit": UNIT, "dtype": "f64",
            "sample": f"{nsteps} steps of src/integrator.cu's run loop (step + calculate_forces + "
                      f"calculate_local_currents) at {w['ny']}x{w['nx']}, CUDA events"}


# ------------------------------------------------------------------ arms

def run_reference_arm(args, w, rank, world):
    """The reference's CPU implementation of the step: test/tjhung_ambplus.h compiled on this host
    (serial: the scheme is single-threaded and keeps its noise generator in global state), or the
    OpenMP oracle port on all host threads where the scheme is not built. Each step is one Euler
    step of the bench workload."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    ref = cpu_reference_runner(w)
    if ref is not None:
        kind, cores, desc = "reference", 1, "test/tjhung_ambplus.h -Ofast, serial, its own drand48 noise"
        run = ref
    else:
        kind, cores, desc = "port", threads, "oracle/amb_oracle.c, OpenMP, Philox noise"
        run = cpu_port_runner(w, threads)
    for _ in range(args.warmup):
        run(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run(1)
    dt = time.perf_counter() - t0
    sites = w["ny"] * w["nx"]
    value = args.steps * sites / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(config_of(args, w), inner_steps=1, precision="f64 (CPU)"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"each step = 1 Euler step of the {w['ny']}x{w['nx']} workload; {desc}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)


def max_over_ranks(dist, values, device):
    """Element-wise maximum of per-rank timings across the process group (identity without one)."""
    if dist is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t]


def job_throughput(world: int, steps: int, inner: int, sites: int, seconds: float) -> float:
    """Whole-job Gsite-updates/s: every rank advances its own replica (weak scaling), the
    slowest rank's time counts."""
    return world * steps * inner * sites / seconds / 1e9


def run_ours(args, w, rank, world, dist):
    import torch
    from activemodelbplus.integrator import Integrator, Model, Stencil, _native as N

    dev = torch.device("cuda", torch.cuda.current_device())
    stencil = Stencil(w["dt"], w["dx"], w["dy"])
    model = Model(w["a"], w["b"], w["c"], w["kappa"], w["lamb"], w["zeta"], w["T"])
    field = initial_field(w, rank)
    sites = w["ny"] * w["nx"]
    launch = None
    if args.kernel == "sliding" and (args.seg_rows or args.pairs or args.fused):
        launch = {"seg_rows": args.seg_rows, "pairs_per_cta": args.pairs, "fused": args.fused}
    elif args.kernel == "tile" and (args.pairs or args.persistent or args.tile_rows != 32):
        launch = {"pairs_per_cta": args.pairs, "persistent": args.persistent, "tile_rows": args.tile_rows}
    sim = Integrator(field, stencil, model, precision=args.precision, seed=1000 + rank, kernel=args.kernel,
                     launch=launch)
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        sim.run(args.inner)
    barrier()

    step_ms, kern_ms = [], []
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    with ClockSampler(dev.index) as clocks:
        barrier()
        for k in range(args.steps):
            flush.fill_(float(k))
            ev[0].record()
            sim._events = (ev[1], ev[2])
            sim.run(args.inner)
            ev[3].record()
            ev[3].synchronize()
            step_ms.append(ev[0].elapsed_time(ev[3]))
            kern_ms.append(ev[1].elapsed_time(ev[2]))
        sim._events = None
        barrier()
    total_ms = sum(step_ms)
    launch_ms = sum(kern_ms) / (args.steps * args.inner)
    total_ms, launch_ms = max_over_ranks(dist, [total_ms, launch_ms], dev)
    value = job_throughput(world, args.steps, args.inner, sites, total_ms / 1e3)

    # e2e through the C handle with pinned float64 host buffers
    e2e = None
    if not args.no_e2e:
        L = N.lib()
        prec = {"f64": N.AMB_F64, "f32": N.AMB_F32, "f32c": N.AMB_F32C}[args.precision]
        host_in = torch.from_numpy(field).pin_memory()
        host_out = torch.empty_like(host_in).pin_memory()
        h = ctypes.c_void_p()
        s, m = N.stencil_struct(stencil), N.model_struct(model)
        rc = L.amb_integrator_create(host_in.data_ptr(), w["ny"], w["nx"], ctypes.byref(s), ctypes.byref(m), prec,
                                     2000 + rank, ctypes.byref(h))
        if rc:
            raise RuntimeError(N.last_error())
        try:
            def e2e_step():
                for rc in (L.amb_integrator_set_field(h, host_in.data_ptr()), L.amb_integrator_run(h, args.inner),
                           L.amb_integrator_get_field(h, host_out.data_ptr())):
                    if rc:
                        raise RuntimeError(N.last_error())
            for _ in range(args.warmup):
                e2e_step()
            barrier()
            wall = 0.0
            for k in range(args.steps):
                flush.fill_(float(k))
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                e2e_step()
                wall += time.perf_counter() - t0
            wall = max_over_ranks(dist, [wall], dev)[0]
            e2e = {"value": job_throughput(world, args.steps, args.inner, sites, wall), "unit": UNIT,
                   "h2d_bytes_per_step": int(host_in.numel() * 8), "d2h_bytes_per_step": int(host_out.numel() * 8)}
        finally:
            L.amb_integrator_destroy(h)

    if rank != 0:
        return
    peak, peak_kind = peaks()
    bytes_per_site = BYTES_PER_SITE if args.precision != "f64" else 16
    achieved = bytes_per_site * sites / (launch_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "f64" else "f32", "data": "synthetic",
        "config": dict(config_of(args, w), kernel_config=sim.kernel_config or launch),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback 6.8 TB/s", "traffic": measured_traffic(args),
                     "kernel": "AMB+ fused step", "launch_us": launch_ms * 1e3,
                     "algorithmic_bytes_per_launch": bytes_per_site * sites},
        "e2e": e2e,
        "gpu_launches": args.steps * (args.inner + 1),
        "clocks": clocks.summary(),
    }
    csum = line["clocks"] or {}
    line["roofline"]["issue"] = issue_roofline(args, value, csum.get("sm_mhz"))
    if not args.no_cpu and world == 1:
        line["cpu_baseline"] = cpu_baseline(w)
        line["reference_gpu"] = reference_gpu_baseline(w)
        line["fp64"] = fp64_path(w, stencil, model, field)
    if not args.no_learned and world == 1 and os.path.exists(args.weights):
        # the metric's second half: learned surrogate vs plain FP32 time to t = 10^3 at 512^2,
        # --learned-seeds noise seeds per arm (default ten: about two minutes; both arms are
        # deterministic, so the errors are those of the committed comparison record)
        res, _ = learned_comparison(args, args.learned_seeds)
        line["learned_time_to_t"] = learned_summary(res)
    print(json.dumps(line), flush=True)


def run_launches(args, w):
    """Bare step launches (amb_step_f32_ex / amb_step_f64) on a device field, for profilers."""
    import torch
    from activemodelbplus.integrator import _native as N
    L = N.lib()
    field = initial_field(w)
    dtype = torch.float64 if args.precision == "f64" else torch.float32
    a = torch.from_numpy(field).to(device="cuda", dtype=dtype)
    b = torch.empty_like(a)
    s = N.amb_stencil(w["dt"], w["dx"], w["dy"])
    m = N.amb_model(w["a"], w["b"], w["c"], w["kappa"], w["lamb"], w["zeta"], w["T"])
    stream = torch.cuda.current_stream().cuda_stream
    if args.precision == "f64":
        cfg = N.amb_kernel_config(1, 0, args.pairs, (N.AMB_FLAG_PERSISTENT if args.persistent else 0)
                                  | (N.AMB_FLAG_TILE_ROWS_28 if args.tile_rows == 28 else 0))
        rc = L.amb_step_f64_ex(ctypes.byref(s), ctypes.byref(m), 1, w["ny"], w["nx"], a.data_ptr(), b.data_ptr(), 0,
                               args.launches, None, ctypes.byref(cfg), stream, None)
    else:
        res = torch.zeros(a.shape, dtype=torch.int16, device="cuda") if args.precision == "f32c" else None
        cfg = N.amb_kernel_config({"auto": 0, "tile": 1, "sliding": 2}[args.kernel], args.seg_rows, args.pairs,
                                  (N.AMB_FLAG_PERSISTENT if args.persistent else 0)
                                  | (N.AMB_FLAG_FUSED if args.fused else 0)
                                  | (N.AMB_FLAG_TILE_ROWS_28 if args.tile_rows == 28 else 0))
        rc = L.amb_step_f32_ex(ctypes.byref(s), ctypes.byref(m), 1, w["ny"], w["nx"], a.data_ptr(), b.data_ptr(),
                               res.data_ptr() if res is not None else None, 0, args.launches, None, ctypes.byref(cfg),
                               stream, None)
    torch.cuda.synchronize()
    if rc:
        raise RuntimeError(N.last_error())
    print(json.dumps({"launches": args.launches, "size": w["ny"], "precision": args.precision}))


def run_sweep(args):
    """Precision/bandwidth sweep on the bench workload's parameters (zeta=-1, lambda=0.5, T=0.05,
    phi0=-0.4+0.01N(0,1), numpy seed 2024) at each size: the same field and Philox key run
    --sweep-steps steps in FP64 (the path pinned to the reference at 1e-12), in FP32 with the
    bf16-compensated update (f32c) and in plain FP32, each timed with CUDA events around one
    Integrator.run (the autotuner runs in the constructor, outside the timed region). Prints one
    JSON line per (size, precision): Gsite-updates/s, algorithmic GB/s (16 B/site FP64, 8 B/site
    FP32) and its fraction of the measured HBM copy bandwidth, and against the FP64 end state the
    max and RMS |delta phi|, the relative L2 error of S(k) over the notebook's bins and the
    relative error of the S(k) mean wavenumber."""
    import copy
    import torch
    from activemodelbplus.analysis import mean_wavenumber, structure_factor
    from activemodelbplus.integrator import Integrator, Model, Stencil
    peak, peak_kind = peaks()
    for size in [int(v) for v in args.sweep_sizes.split(",")]:
        a2 = copy.copy(args)
        a2.size = size
        w = workload(a2)
        field = initial_field(w)
        stencil = Stencil(w["dt"], w["dx"], w["dy"])
        model = Model(w["a"], w["b"], w["c"], w["kappa"], w["lamb"], w["zeta"], w["T"])
        ref = None
        for prec in ("f64", "f32c", "f32"):
            sim = Integrator(field, stencil, model, precision=prec, seed=w["seed"])
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with ClockSampler(torch.cuda.current_device()) as clocks:
                e0.record()
                sim.run(args.sweep_steps)
                e1.record()
                torch.cuda.synchronize()
            sec = e0.elapsed_time(e1) / 1e3
            end = sim.field_tensor.double().clone()
            cfg = getattr(sim, "kernel_config", None)
            del sim
            gsite = size * size * args.sweep_steps / sec / 1e9
            bps = 16 if prec == "f64" else 8
            line = {"sweep": True, "size": size, "precision": prec, "steps": args.sweep_steps, "seconds": sec,
                    "gsite_per_s": gsite, "gbs_algorithmic": gsite * bps, "hbm_frac": gsite * bps / peak,
                    "peak_gbs": peak, "peak_source": peak_kind, "kernel_config": cfg, "clocks": clocks.summary()}
            k, S, _ = structure_factor(end, w["dx"], w["dy"], phi0=w["phi0"])
            if ref is None:
                ref = (end, S, mean_wavenumber(k, S))
            else:
                d = end - ref[0]
                m = np.isfinite(S) & np.isfinite(ref[1])
                line.update({"max_abs_err_vs_f64": float(d.abs().max()),
                             "rms_err_vs_f64": float(d.square().mean().sqrt()),
                             "sk_rel_l2_err_vs_f64": float(np.linalg.norm(S[m] - ref[1][m]) / np.linalg.norm(ref[1][m])),
                             "kavg_rel_err_vs_f64": abs(mean_wavenumber(k, S) - ref[2]) / ref[2]})
            print(json.dumps(line), flush=True)
        del ref
        torch.cuda.empty_cache()


def run_ensemble(args):
    """Batched ensemble: 256 replicas, sizes drawn from {128,192,256,384,512,768,1024}^2, zeta in
    [-4,4], lambda in [-1,1], phi0 in [-0.6,0.6], T in [0,0.1], a=-0.25 c=0.25 kappa=1, dt=1e-3,
    f32c, numpy seed 7. One bench step = one Ensemble.run(inner) (one launch per time step over all
    replicas, replayed from a captured CUDA graph)."""
    import torch
    from activemodelbplus.integrator import Ensemble, Model, Stencil
    rng = np.random.default_rng(7)
    sizes = rng.choice([128, 192, 256, 384, 512, 768, 1024], size=256)
    fields, models = [], []
    for n in sizes:
        phi0 = rng.uniform(-0.6, 0.6)
        fields.append(phi0 + 0.01 * rng.standard_normal((n, n)))
        models.append(Model(-0.25, 0, 0.25, 1, rng.uniform(-1, 1), rng.uniform(-4, 4), rng.uniform(0, 0.1)))
    sites = int(sum(int(n) * int(n) for n in sizes))
    ens = Ensemble(fields, Stencil(1e-3, 1, 1), models, precision="f32c", seeds=list(range(256)), graph_steps=50)
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        ens.run(args.inner)
    torch.cuda.synchronize()
    wall = 0.0
    with ClockSampler(torch.cuda.current_device()) as clocks:
        for k in range(args.steps):
            flush.fill_(float(k))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ens.run(args.inner)
            wall += time.perf_counter() - t0
    value = args.steps * args.inner * sites / wall / 1e9
    print(json.dumps({"metric": "ensemble Gsite-updates/s (256 replicas, uneven sizes)", "value": value, "unit": UNIT,
                      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True, "dtype": "f32",
                      "data": "synthetic", "config": {"workload": "ensemble", "replicas": 256, "sites": sites,
                                                      "inner_steps": args.inner, "tasks": ens.ntasks,
                                                      "kernel_form": "fused" if ens.fused else "warp pair"},
                      "clocks": clocks.summary()}), flush=True)
    ens.close()


def run_learned_launches(args):
    """Bare forward passes of the flux network (6 tensor-core convolutions) on one 512^2 field
    of the learned workload, for profilers."""
    import torch
    from activemodelbplus import learned as L
    net = L.FluxNet.load(args.weights)
    net.refresh()
    phi = torch.from_numpy(-0.4 + 0.01 * np.random.default_rng(0).standard_normal((1, 512, 512))).float().cuda()
    params = torch.tensor([[-4.0, -1.0, 0.05]], device="cuda")
    x = L.network_input(phi, params)
    for _ in range(args.learned_launches):
        flux = net.forward(x)
    torch.cuda.synchronize()
    net.check_error()
    print(json.dumps({"learned_launches": args.learned_launches, "flux_rms": float(flux.square().mean().sqrt())}))


def run_learned_steps(args):
    """N macro steps (K = 50 Euler steps each) of the learned stepper on the 512^2 field of the
    learned workload, after 40 untimed ones (graph capture, first checks); wall time per macro
    step, CUDA-synchronised, including its residual checks (adaptive: one per 40 to 320 macro
    steps)."""
    import torch
    from activemodelbplus import learned as L
    from activemodelbplus.integrator import Model, Stencil
    net = L.FluxNet.load(args.weights)
    field = -0.4 + 0.01 * np.random.default_rng(0).standard_normal((512, 512))
    st = L.LearnedStepper(net, field, Stencil(1e-3, 1, 1), Model(-0.25, 0, 0.25, 1, -1, -4, 0.05), K=net.K,
                          check_every=40, tol=0.5, residual_sigma=2.0)
    st.advance(40)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st.advance(args.learned_steps)
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    print(json.dumps({"learned_macro_steps": args.learned_steps, "us_per_macro_step": 1e6 * sec / args.learned_steps,
                      "euler_steps_per_macro_step": net.K, "fallback_spans": st.fallback_spans}))


def learned_comparison(args, seeds: int):
    """The learned coarse stepper (K = 50 Euler steps per network evaluation) against the plain
    FP32 integrator, both from the same seeded 512^2 field (phi = -0.4 + 0.01 N(0,1), numpy seed
    0; a=-0.25 b=0 c=0.25 kappa=1 lambda=-1 zeta=-4 T=0.05, dt=1e-3) to t_end, ``seeds`` noise
    seeds per arm: wall time of each (CUDA-synchronised; the fastest run of each arm counts), the
    S(k) peak position (sub-bin) and mean wavenumber and the droplet count of the end states
    (learned mean against plain mean, with standard errors), and the learned runs' exact
    fixed-point mass drift. Returns (compare record, clocks summary)."""
    import torch
    from activemodelbplus import learned as L
    from activemodelbplus.integrator import Model, Stencil
    net = L.FluxNet.load(args.weights)
    field = -0.4 + 0.01 * np.random.default_rng(0).standard_normal((512, 512))
    model = Model(a=-0.25, b=0, c=0.25, kappa=1, lamb=-1, zeta=-4, T=0.05)
    with ClockSampler(torch.cuda.current_device()) as clocks:
        res = L.compare_with_plain(net, field, Stencil(1e-3, 1, 1), model, t_end=args.t_end, residual_sigma=2.0,
                                   plain_seeds=tuple(range(1, seeds + 1)), learned_runs=seeds)
    return res, clocks.summary()


def learned_summary(res) -> dict:
    """The bench-line digest of a learned-vs-plain comparison record."""
    return {"workload": f"512^2 AMB+ (zeta=-4, lambda=-1, T=0.05) to t={res['t_end']:g}, K=50",
            "speedup": res["speedup"], "plain_seconds": res["plain_seconds_min"],
            "learned_seconds": res["learned_seconds_min"], "plain_path": res["plain_path"],
            "plain_kernel_config": res.get("plain_kernel_config"), "seeds_per_arm": len(res["plain"]),
            "k_peak_plain": res["plain_k_peak_mean"], "k_peak_learned": res["learned_k_peak_mean"],
            "k_peak_rel_err": res["k_peak_rel_err"], "k_peak_rel_err_se": res["k_peak_rel_err_se"],
            "k_avg_rel_err": res["k_avg_rel_err"], "k_avg_rel_err_se": res["k_avg_rel_err_se"],
            "droplets_plain": res["plain_droplets_mean"], "droplets_learned": res["learned_droplets_mean"],
            "droplets_rel_err": res["droplets_rel_err"], "droplets_rel_err_se": res["droplets_rel_err_se"],
            "mass_q_drift_learned_max": res["learned_mass_q_drift_max"],
            "fallback_spans": res["learned_fallback_spans"],
            "max_residual": max(r["max_residual"] for r in res["learned_runs"])}


def run_learned(args):
    """``--learned``: the learned-vs-plain comparison with --learned-seeds seeds per arm, as one
    JSON line whose value is the speed-up."""
    res, clocks = learned_comparison(args, args.learned_seeds)
    out = {"metric": f"learned vs plain FP32 time to t={args.t_end:g} (512^2 AMB+), speed-up", "value": res["speedup"],
           "unit": "x", "higher_is_better": True, "n_gpus": 1, "dtype": "bf16 network / int32 fixed-point field",
           "data": "synthetic", "config": {"workload": "learned_time_to_t", "size": 512, "K": 50,
                                           "t_end": args.t_end, "check_every": res["check_every"],
                                           "max_check_every": res["max_check_every"], "tol": res["tol"]},
           **learned_summary(res),
           "runs_plain": res["plain"], "runs_learned": res["learned_runs"], "clocks": clocks}
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    w = workload(args)
    if args.launches > 0:
        return run_launches(args, w)
    if args.ensemble:
        return run_ensemble(args)
    if args.sweep:
        return run_sweep(args)
    if args.learned:
        return run_learned(args)
    if args.learned_launches > 0:
        return run_learned_launches(args)
    if args.learned_steps > 0:
        return run_learned_steps(args)
    if args.impl == "reference":
        return run_reference_arm(args, w, rank, world)
    import torch
    dist = None
    if world > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        tdist.init_process_group("nccl")
        dist = tdist
    try:
        run_ours(args, w, rank, world, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
