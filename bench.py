#!/usr/bin/env python3
"""Throughput of the Melvin.py per-timestep hot path on GB300.

Workload: decaying 2D turbulence, 2048 x 2048, doubly periodic, fully
spectral (2/3 dealiasing), nu = 5e-5, dt = 2e-4, AB2 with semi-implicit
diffusion (alpha = 0.51), second-order finite-difference Jacobian -- the
configuration the headline metric is quoted on.  One step = velocity from
vorticity, nonlinear term, update, i.e. one pass of the fused timestep
(three kernels) over the resident state.

Arms:
  native     (default) the fused FP64 timestep; also the split-precision
             (FP32 transforms / FP64 state) timestep, an end-to-end run
             through the public API with host buffers, and the CPU
             baseline (the NumPy oracle on the host cores, bounded sample);
  reference  the reference algorithm's CPU implementation (the NumPy
             oracle) on the host cores, same workload.

Multi-GPU (torchrun): replicas only -- every rank advances its own
simulation; the value is the sum over ranks with the max-over-ranks time.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.join(ROOT, "melvin.py_gb300")
if PKG_ROOT not in sys.path:
    sys.path.insert(0, PKG_ROOT)

METRIC = "Mpts·steps/s at 2048² (plain FP64 vs FP32/FP64 split); solves/s + p99 latency"
UNIT = "Mpts·steps/s"
WORKLOAD = {
    "workload": "decaying 2D turbulence 2048x2048, fully spectral, AB2 semi-implicit (alpha=0.51), "
                "FD2 Jacobian, nu=5e-5, dt=2e-4",
    "nx": 2048, "nz": 2048, "lx": "2*pi", "lz": "2*pi", "nu": 5e-5, "dt": 2e-4,
    "integrator_order": 2, "spatial_derivative_order": 2,
}
DATA = "synthetic: seeded vorticity with E(k)~k^4 exp(-(k/10)^2), uniform random phases, unit RMS velocity"
L2_FLUSH_BYTES = 256 << 20


# ---------------------------------------------------------------------------
# process group helpers (replicas only: no data-path collective)
# ---------------------------------------------------------------------------


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def dist_init(backend):
    import torch.distributed as dist

    rank, world, _ = dist_env()
    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend, rank=rank, world_size=world)
    return dist if world > 1 else None


def reduce_max(value: float, dist=None, device=None) -> float:
    """Max of a per-rank scalar over all ranks (identity for one rank)."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist=None):
    if dist is not None:
        dist.barrier()


def aggregate_throughput(npts_per_rank: int, steps: int, world: int, max_seconds: float) -> float:
    """Whole-job Mpts*steps/s: all ranks' points over the slowest rank's time."""
    return world * npts_per_rank * steps / max_seconds / 1e6


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
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
            self._t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------


def make_params(n, precision, device):
    import numpy as np

    import melvin

    return melvin.Parameters({
        "nx": n, "nz": n, "lx": 2 * np.pi, "lz": 2 * np.pi, "final_time": 1.0,
        "initial_dt": WORKLOAD["dt"], "integrator_order": WORKLOAD["integrator_order"],
        "spatial_derivative_order": WORKLOAD["spatial_derivative_order"], "integrator": "semi-implicit",
        "precision": precision, "device": str(device),
    })


def make_run(n, precision, device, w0):
    import torch

    import melvin
    from melvin import BasisFunctions as B, equations

    p = make_params(n, precision, device)
    sim = melvin.Simulation(p, torch)
    bf = [B.COMPLEX_EXP, B.COMPLEX_EXP]
    w = sim.make_variable("w", bf)
    dw = sim.make_derivative("dw")
    w.load(w0, is_physical=True)
    step = equations.vorticity(sim, w, dw, WORKLOAD["nu"])
    return sim, w, dw, step


def kernel_model(n, split):
    """Algorithmic bytes and nominal FFT flops per launch of the three
    fused-step kernels (F = 1 advected field)."""
    nn, nm = (n - 1) // 3, (n - 1) // 3
    S = (2 * nn + 1) * nm  # spectral elements
    Pk = n * nm            # x-pass intermediate elements (kept z modes only)
    ws, wi = 16, (8 if split else 16)
    lg = n.bit_length() - 1
    fft = 5 * n * lg       # nominal flops of one complex length-n FFT
    return {
        "xinv": {"bytes": ws * S + 3 * wi * Pk, "flops": 3 * nm * fft},
        "zstep": {"bytes": 5 * wi * Pk, "flops": (n // 2) * 5 * fft + 12 * n * n},
        "xfwd": {"bytes": 2 * wi * Pk + 4 * ws * S, "flops": nm * fft + 30 * S},
    }


def timed_steps(step, steps, flush):
    """Run `steps` fused steps, each bracketed by CUDA events recorded on the
    launching stream (per-kernel events inside the step), with an L2 flush
    between steps outside the events.  Returns per-step and per-kernel ms."""
    import torch

    nk = step.kernel_count()
    evs = []
    for _ in range(steps):
        flush.zero_()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(nk + 1)]
        for e in ev:
            e.record()  # materialise the events
        step.step_events(ev)
        evs.append(ev)
    torch.cuda.synchronize()
    per_step = [ev[0].elapsed_time(ev[-1]) for ev in evs]
    per_kernel = [[ev[k].elapsed_time(ev[k + 1]) for ev in evs] for k in range(nk)]
    return per_step, per_kernel


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def load_traffic():
    """Per-launch DRAM bytes of the fused-step kernels from the committed
    ncu summary (profiles/fused_step_traffic.json), when present."""
    try:
        with open(os.path.join(ROOT, "profiles", "fused_step_traffic.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def roofline(model, kernel_ms, names, peak_gbs, peak_kind, traffic, key, step_ms):
    """The dominant kernel's algorithmic bytes over its event-timed launch
    duration against the HBM peak, plus the same for the whole step
    (step_achieved / step_frac: the step's algorithmic bytes over its
    event-timed duration)."""
    avg = [statistics.mean(v) for v in kernel_ms]
    k = max(range(len(avg)), key=lambda i: avg[i])
    name = names[k]
    achieved = model[name]["bytes"] / (avg[k] * 1e-3) / 1e9
    tr = traffic.get(key, {}).get(name)
    step_bytes = sum(m["bytes"] for m in model.values())
    step_gbs = step_bytes / (step_ms * 1e-3) / 1e9
    return {
        "kernel": name, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak_gbs, "unit": "GB/s",
        "frac": round(achieved / peak_gbs, 4), "peak_kind": peak_kind,
        "traffic": tr, "algorithmic_bytes": model[name]["bytes"], "avg_ms": round(avg[k], 4),
        "kernel_ms": {names[i]: round(avg[i], 4) for i in range(len(avg))},
        "step_algorithmic_bytes": step_bytes, "step_ms": round(step_ms, 4),
        "step_achieved": round(step_gbs, 1), "step_frac": round(step_gbs / peak_gbs, 4),
    }, k


def fp64_fma_peak(device, iters=1 << 14, reps=5):
    """FP64 FMA throughput of this GPU in TFLOP/s (an FMA counts two flops),
    measured live with the library's probe kernel (mgb_fp64_fma_probe: 4
    CTAs of 256 threads per SM, 8 independent FMA chains per thread): the
    fastest of `reps` event-timed launches after one warm launch."""
    import ctypes as C

    import torch

    from melvin import _native as N

    lib = N.load_library()
    blocks = 4 * torch.cuda.get_device_properties(device).multi_processor_count
    sink = torch.zeros(blocks, dtype=torch.float64, device=device)
    flops = C.c_double()
    best = None
    for r in range(reps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        N.check(lib.mgb_fp64_fma_probe(N.ptr(sink), blocks, iters, C.byref(flops), N.stream_handle(device)))
        e1.record()
        torch.cuda.synchronize()
        if r:
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
    return flops.value / (best * 1e-3) / 1e12


def cpu_step_sample(w0, n, steps):
    """The NumPy oracle (reference algorithm, single thread) on the host."""
    import numpy as np

    import oracle as O
    from oracle import problems as P

    g = O.Grid(n, n, 2 * np.pi, 2 * np.pi)
    pr = P.Problem(g, P.vorticity_specs(WORKLOAD["nu"]), [O.to_spectral(g, w0)], WORKLOAD["dt"])
    pr.step()  # warm
    t0 = time.perf_counter()
    for _ in range(steps):
        pr.step()
    dt = time.perf_counter() - t0
    return n * n * steps / dt / 1e6, dt


def _oracle_member(job):
    """One independent simulation of the oracle (reference algorithm, NumPy,
    one thread) on one host core, time-bounded: returns (grid points x
    steps, seconds, grid).  `kind` "kh": a Kelvin-Helmholtz ensemble member
    (256^2, vorticity + passive scalar, nu = kappa = 1e-4, dt = 5e-4, AB2
    semi-implicit); "ddc": a serving-pool member (double-diffusive convection
    on the Dirichlet grid, Ra_T = 1e6, Pr = 7, Le = 100, R_rho = 2, explicit
    AB2, dt = 0.1 dz^2 / Pr); "rbc": Rayleigh-Benard convection on the
    n x (n/2 + 1) Dirichlet grid (Ra = 1e7, Pr = 1, 4th-order differences,
    AB4/AM4 predictor-corrector, dt = 1e-7)."""
    kind, n, seed, budget = job
    import numpy as np

    import oracle as O
    from oracle import problems as P

    if kind == "kh":
        g = O.Grid(n, n, 2 * np.pi, 2 * np.pi)
        delta = np.random.default_rng(seed).uniform(0.02, 0.1)
        w, c = P.kh_ic(g, delta, seed=seed)
        pr = P.Problem(g, P.kh_specs(1e-4, 1e-4), [O.to_spectral(g, w), O.to_spectral(g, c)], 5e-4)
    elif kind == "rbc":
        g = O.Grid(n, n // 2 + 1, 2.0, 1.0, True, 4)
        pr = P.Problem(g, P.rbc_specs(1.0, 1e7),
                       [np.zeros(g.spectral_shape, complex), O.to_spectral(g, P.conductive_ic(g, seed=seed))],
                       1e-7, "pece", 4)
    else:
        g = O.Grid(n, n + 1, 2.0, 1.0, True, 2)
        t0, s0 = P.conductive_ic(g, seed=2 * seed), P.conductive_ic(g, seed=2 * seed + 1)
        pr = P.Problem(g, P.ddc_dirichlet_specs(7.0, 1e6, 2.0, 100.0),
                       [np.zeros(g.spectral_shape, complex), O.to_spectral(g, t0), O.to_spectral(g, s0)],
                       0.1 * g.dz ** 2 / 7.0, "explicit", 2)
    pr.step()  # warm
    steps, t_start = 0, time.perf_counter()
    while True:
        pr.step()
        steps += 1
        el = time.perf_counter() - t_start
        if el >= budget and steps >= 2:
            return g.nx * g.nz * steps, el, f"{g.nx}x{g.nz}"


def cpu_pool_sample(kind, n, members, budget=6.0):
    """The oracle on min(host cores, members) cores: that many independent
    members at once in a spawn pool, each time-bounded to `budget` seconds.
    Aggregate Mpts.steps/s = total grid points x steps / the slowest
    member's time."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    cores = max(1, min(os.cpu_count() or 1, members))
    # a worker that dies raises BrokenProcessPool here instead of being respawned
    with ProcessPoolExecutor(max_workers=cores, mp_context=mp.get_context("spawn")) as pool:
        res = list(pool.map(_oracle_member, [(kind, n, seed, budget) for seed in range(cores)], timeout=20 * budget))
    pts = sum(r[0] for r in res)
    secs = max(r[1] for r in res)
    return {"value": round(pts / secs / 1e6, 4), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"{cores} independent members at once, one per host core, each about {budget:.0f} s of "
                       f"NumPy oracle steps after a warm step ({kind}, {res[0][2]})") if cores > 1 else
                      (f"one simulation on one host core, about {budget:.0f} s of NumPy oracle steps after a warm "
                       f"step ({kind}, {res[0][2]}; the reference is single-threaded)")}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from melvin import workloads

    n = args.n
    w0 = workloads.decaying_turbulence(n, n, seed=0)
    for _ in range(max(args.warmup - 1, 0)):
        cpu_step_sample(w0, n, 0)
    val, secs = cpu_step_sample(w0, n, args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(val, 4), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(secs / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": dict(WORKLOAD, nx=n, nz=n),
        "cpu_baseline": {"value": round(val, 4), "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"{args.steps} full timesteps at {n}x{n} (NumPy oracle, one thread: "
                                   "pocketfft is single-threaded)"},
        "e2e": {"value": round(val, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_only(args):
    """Warm-up plus timed fused steps of one precision and nothing else (the
    command profiled with ncu)."""
    import torch

    from melvin import workloads

    _, _, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    n = args.n
    w0 = workloads.decaying_turbulence(n, n, seed=0)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)
    sim, w, dw, step = make_run(n, {"fp64": "double"}.get(args.only, args.only), device, w0)
    tiles = _apply_tiles(args, step.plan, 1, lambda: step.autotune())
    for _ in range(args.warmup):
        step.step()
    torch.cuda.synchronize()
    per_step, per_kernel = timed_steps(step, args.steps, flush)
    print(json.dumps({"only": args.only, "n": n, "steps": args.steps, "tiles": tiles,
                      "ms_per_step": round(statistics.mean(per_step), 4),
                      "kernel_ms": [round(statistics.mean(k), 4) for k in per_kernel]}), flush=True)
    return 0


def _timed_run(n, precision, device, w0, steps, warmup, flush, dist, tune=True):
    """Tune the tile variants (unless `tune` is off), warm up, then time
    `steps` fused steps of one precision; returns the per-step and
    per-kernel times, the stepper and the tuning result."""
    import torch

    sim, w, dw, step = make_run(n, precision, device, w0)
    tuned = step.autotune() if tune else None
    for _ in range(warmup):
        step.step()
    torch.cuda.synchronize()
    barrier(dist)
    torch.cuda.synchronize()
    per_step, per_kernel = timed_steps(step, steps, flush)
    torch.cuda.synchronize()
    barrier(dist)
    return per_step, per_kernel, (sim, w, dw, step), tuned


def _apply_tiles(args, plan, nfields, tune):
    """--tiles pins the tile variants, --no-tune keeps the defaults,
    otherwise `tune()` runs the autotuner; returns the selection."""
    if args.tiles:
        plan.set_tiles(nfields, [int(v) for v in args.tiles.split(",")])
    elif not args.no_tune:
        tune()
    return list(plan.get_tiles(nfields))


def _tiles_summary(plan, tuned):
    """The tile variant used per kernel family, and the tuner's gain."""
    from melvin._native import FAMILIES

    tiles = plan.get_tiles(1)
    out = {}
    for fam, name in enumerate(FAMILIES):
        _, shape, radix, _, kind = plan.tile_info(fam, 1, tiles[fam])
        out[name] = {"variant": tiles[fam], "per_cta": shape, "radix": radix,
                     "kind": "registers" if kind else "shared-memory passes"}
    if tuned is not None:
        out["tuned"] = {"default_ms": round(tuned.default_ms_per_step, 4), "ms": round(tuned.ms_per_step, 4),
                        "trials": len(tuned.trials)}
    return out


def _accuracy(n, device, w0, precision, nsteps=100):
    """Relative L2 of the state against the FP64 path after 1 and `nsteps`
    steps from the same initial field, and the max relative error of the
    kinetic-energy trajectory."""
    import numpy as np
    import torch

    _, wa, _, sa = make_run(n, "double", device, w0)
    _, wb, _, sb = make_run(n, precision, device, w0)
    ke_a, ke_b, out = [], [], {}
    for k in range(1, nsteps + 1):
        ke_a.append(float(sa.step(diagnostics=True)[0]))
        ke_b.append(float(sb.step(diagnostics=True)[0]))
        if k in (1, nsteps):
            err = (torch.linalg.vector_norm(wa._sdata - wb._sdata) / torch.linalg.vector_norm(wa._sdata)).item()
            out["rel_l2_1step" if k == 1 else f"rel_l2_{nsteps}steps"] = err
    ke_a, ke_b = np.array(ke_a), np.array(ke_b)
    out["ke_traj_max_rel_err"] = float(np.max(np.abs(ke_b - ke_a) / np.abs(ke_a)))
    return out


def run_native(args):
    import torch

    from melvin import workloads

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    dist = dist_init("nccl")
    n = args.n
    w0 = workloads.decaying_turbulence(n, n, seed=0)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)
    peak, peak_kind = load_peaks()
    traffic = load_traffic()
    names = ["xinv", "zstep", "xfwd"]
    results = {}
    with ClockSampler(local) as clocks:
        t_wall0 = time.perf_counter()
        for key, prec in (("fp64", "double"), ("split", "split"), ("dfloat", "dfloat")):
            per_step, per_kernel, run, tuned = _timed_run(n, prec, device, w0, args.steps, args.warmup, flush, dist,
                                                          tune=not args.no_tune)
            secs = reduce_max(sum(per_step) * 1e-3, dist, device)
            model = kernel_model(n, prec == "split")
            roof, kdom = roofline(model, per_kernel, names, peak, peak_kind, traffic, prec,
                                  secs / args.steps * 1e3)
            results[key] = dict(secs=secs, per_kernel=per_kernel, roof=roof, kdom=kdom, model=model, run=run,
                                tiles=_tiles_summary(run[3].plan, tuned),
                                value=aggregate_throughput(n * n, args.steps, world, secs))
            if key == "fp64":
                wall = time.perf_counter() - t_wall0

        # end to end through the public API with host buffers (FP64)
        sim, w, dw, step = results["fp64"]["run"]
        h_w = torch.empty_like(w._sdata, device="cpu").pin_memory()
        h_dw = torch.empty_like(dw._data, device="cpu").pin_memory()
        h_w.copy_(w._sdata)
        h_dw.copy_(dw._data)
        for _ in range(args.warmup):  # the first call also creates the copy stream
            step.step_host([h_w], [h_dw])
        torch.cuda.synchronize()
        # One interval over the whole loop: a step's history slot comes down
        # on the copy stream while the next step runs, so per-step intervals
        # would not hold it.  The L2 flush before every step is inside.
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            flush.zero_()
            h2d, d2h = step.step_host([h_w], [h_dw])
        torch.cuda.current_stream().wait_event(step.host_done)
        e1.record()
        torch.cuda.synchronize()
        e2e_secs = reduce_max(e0.elapsed_time(e1) * 1e-3, dist, device)

    acc = {}
    if rank == 0:
        acc["split"] = _accuracy(n, device, w0, "split")
        acc["dfloat"] = _accuracy(n, device, w0, "dfloat")

    # the other benchmark configurations, one process and GPU (N = 1 only)
    extra = {}
    if rank == 0 and world == 1 and not args.headline_only:
        del results["split"]["run"], results["dfloat"]["run"]
        torch.cuda.empty_cache()
        cpu_on = not args.no_cpu
        with ClockSampler(local) as extra_clocks:
            extra["rbc"] = rbc_result(device, "double", min(args.steps, 100), args.warmup, cpu_on, 4.0)
            extra["kh_ensemble"] = kh_ensemble_result(device, "split", 256, max(args.steps, 64), args.warmup,
                                                      None, not args.no_tune, cpu_on, 4.0)
            torch.cuda.empty_cache()
            extra["serving"] = serving_result(device, "split", 100, (50.0, 12.0), cpu_on, 4.0)
        extra["clocks"] = extra_clocks.summary()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cv, csecs = cpu_step_sample(w0, n, 2)
        cpu = {"value": round(cv, 4), "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"2 timesteps at {n}x{n} after one warm step ({csecs:.1f} s), NumPy oracle on one host "
                         "core (pocketfft is single-threaded)"}

    if rank == 0:
        r64 = results["fp64"]
        avg_k = [statistics.mean(v) for v in r64["per_kernel"]]
        kd = r64["kdom"]
        fl = r64["model"][names[kd]]["flops"] / (avg_k[kd] * 1e-3) / 1e12
        fma_peak = fp64_fma_peak(device)
        step_fl = sum(m["flops"] for m in r64["model"].values()) / (r64["secs"] / args.steps) / 1e12
        fp64_roof = {"kernel": names[kd], "achieved_tflops": round(fl, 4), "peak_tflops": round(fma_peak, 4),
                     "frac": round(fl / fma_peak, 4), "step_achieved_tflops": round(step_fl, 4),
                     "step_frac": round(step_fl / fma_peak, 4),
                     "note": "nominal 5 N log2 N flops per complex FFT; peak = FP64 FMA rate measured in this run "
                             "by mgb_fp64_fma_probe (FMA = 2 flops)"}

        def sub(key, dtype):
            r = results[key]
            return {"value": round(r["value"], 3), "unit": UNIT, "dtype": dtype,
                    "ms_per_step": round(r["secs"] / args.steps * 1e3, 4),
                    "speedup_vs_fp64": round(r["value"] / r64["value"], 3), "roofline": r["roof"],
                    "tiles": r["tiles"], **acc[key]}

        line = {
            "metric": METRIC, "value": round(r64["value"], 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(r64["secs"] / args.steps * 1e3, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
            "config": dict(WORKLOAD, nx=n, nz=n, l2="flushed (256 MiB write) between timed steps", replicas=world),
            "roofline": r64["roof"],
            "fp64_alu_roof": fp64_roof,
            "tiles": r64["tiles"],
            "e2e": {"value": round(aggregate_throughput(n * n, args.steps, world, e2e_secs), 3), "unit": UNIT,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "path": "Stepper.step_host (FP64): state and history in pinned host memory; each step "
                            "uploads the state and the history slot the update reads (that upload on a second "
                            "stream, overlapping the transforms) and downloads the state and the slot it writes "
                            "(that download on the second stream, overlapping the next step)",
                    "timing": "one interval over all timed steps, the 256 MiB L2 flush before every step "
                              "included"},
            "split": sub("split", "f32 transforms / f64 state and history"),
            "dfloat": sub("dfloat", "double-float (f32 pair) transforms / f64 state and history"),
            "cpu_baseline": cpu,
            "gpu_launches": results["fp64"]["run"][3].kernel_count() * args.steps,
            "clocks": clocks.summary(),
            "wall_s_fp64_timed": round(wall, 3),
        }
        if extra:
            line["rbc"] = extra["rbc"]
            line["kh_ensemble"] = extra["kh_ensemble"]
            line["serving"] = extra["serving"]
            line["configs_clocks"] = extra["clocks"]
        print(json.dumps(line), flush=True)
    barrier(dist)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def kh_ensemble_result(device, precision="split", members=256, steps=200, warmup=3, tiles=None, tune=True,
                       cpu=True, cpu_budget=6.0):
    """Kelvin-Helmholtz ensemble: `members` independent 256x256 runs
    (vorticity + passive scalar, nu = kappa = 1e-4, dt = 5e-4, AB2
    semi-implicit), delta ~ U[0.02, 0.1] per member; all members advance in
    CUDA-graph replays of 8 batched steps, L2 flushed between replays.
    Returns the result dict (value in Mpts.steps/s, the step's algorithmic
    HBM bytes and their fraction of the peak, the CPU baseline)."""
    import numpy as np
    import torch

    import melvin
    from melvin import workloads
    from melvin.ensemble import Ensemble, FieldSpec

    n, graph_steps = 256, 8
    p = melvin.Parameters({"nx": n, "nz": n, "lx": 2 * np.pi, "lz": 2 * np.pi, "final_time": 1.0,
                           "initial_dt": 5e-4, "precision": precision, "device": str(device)})
    ens = Ensemble(p, [FieldSpec(1e-4), FieldSpec(1e-4)], members)
    rng = np.random.default_rng(0)
    deltas = rng.uniform(0.02, 0.1, size=members)
    for b in range(members):
        w, c = workloads.kelvin_helmholtz(n, n, deltas[b], seed=b)
        ens.load_physical(b, [w, c])
    ens.step(5e-4)
    tuned = None
    if tiles:
        ens.plan.set_tiles(2, [int(v) for v in tiles.split(",")])
    elif tune:
        tuned = ens.autotune(5e-4)
    replay = ens.graph(5e-4, graph_steps)
    for _ in range(max(warmup, 1)):
        replay()
    nrep = max(1, steps // graph_steps)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)
    ev = []
    for _ in range(nrep):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        replay()
        e1.record()
        ev.append((e0, e1))
    torch.cuda.synchronize()
    secs = sum(a.elapsed_time(b) for a, b in ev) * 1e-3
    steps_run = nrep * graph_steps
    nn = (n - 1) // 3
    S, Pk = (2 * nn + 1) * nn, n * nn
    wi = 8 if precision == "split" else 16
    bytes_step = members * (16 * 10 * S + wi * 2 * 8 * Pk)
    peak, kind = load_peaks()
    ms = secs / steps_run * 1e3
    out = {
        "members": members, "grid": f"{n}x{n}", "precision": precision, "steps": steps_run,
        "graph_steps": graph_steps, "value": round(members * n * n * steps_run / secs / 1e6, 2), "unit": UNIT,
        "ms_per_ensemble_step": round(ms, 4),
        "roofline": {"bound": "hbm", "algorithmic_bytes_per_step": bytes_step,
                     "step_achieved": round(bytes_step / (ms * 1e-3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                     "step_frac": round(bytes_step / (ms * 1e-3) / 1e9 / peak, 4), "peak_kind": kind},
        "tiles": list(ens.plan.get_tiles(2)),
        "tuned": None if tuned is None else {"default_ms": round(tuned.default_ms_per_step, 4),
                                             "ms": round(tuned.ms_per_step, 4)},
        "l2": "flushed between graph launches",
        "cpu_baseline": cpu_pool_sample("kh", n, members, cpu_budget) if cpu else None,
    }
    del ens, replay
    return out


def run_ensemble(args):
    import torch

    device = torch.device("cuda", dist_env()[2])
    torch.cuda.set_device(device)
    res = kh_ensemble_result(device, args.precision, args.members, args.steps, args.warmup, args.tiles,
                             not args.no_tune, not args.no_cpu)
    print(json.dumps({"workload": "kh-ensemble", "metric": "Mpts·steps/s (ensemble)", **res}), flush=True)
    return 0


def run_mixed_ensemble(args):
    """Kelvin-Helmholtz ensembles of uneven grid sizes in one CUDA graph:
    64 runs at 128x128, 32 at 256x256, 8 at 512x512 and 2 at 1024x1024
    (nu = kappa = 1e-4, AB2 semi-implicit, split precision), each size a
    branch of the graph; against the same ensembles replayed one size after
    the other."""
    import numpy as np
    import torch

    import melvin
    from melvin import workloads
    from melvin.ensemble import Ensemble, EnsembleGroup, FieldSpec

    device = torch.device("cuda", dist_env()[2])
    torch.cuda.set_device(device)
    sizes = [(128, 64, 1e-3), (256, 32, 5e-4), (512, 8, 2.5e-4), (1024, 2, 1.25e-4)]
    graph_steps = 8
    rng = np.random.default_rng(0)
    ens = []
    for n, members, dt in sizes:
        p = melvin.Parameters({"nx": n, "nz": n, "lx": 2 * np.pi, "lz": 2 * np.pi, "final_time": 1.0,
                               "initial_dt": dt, "precision": args.precision, "device": str(device)})
        e = Ensemble(p, [FieldSpec(1e-4), FieldSpec(1e-4)], members)
        for b in range(members):
            w, c = workloads.kelvin_helmholtz(n, n, float(rng.uniform(0.02, 0.1)), seed=b)
            e.load_physical(b, [w, c])
        e.step(dt)
        if not args.no_tune:
            e.autotune(dt)
        ens.append(e)
    dts = [dt for _, _, dt in sizes]
    group = EnsembleGroup(ens)
    together = group.graph(dts, graph_steps)
    apart = [e.graph(dt, graph_steps) for e, dt in zip(ens, dts)]
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)

    def timed(fn):
        for _ in range(max(args.warmup, 1)):
            fn()
        nrep = max(1, args.steps // graph_steps)
        ev = []
        for _ in range(nrep):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            ev.append((e0, e1))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) * 1e-3, nrep * graph_steps

    secs, steps = timed(together)
    secs_apart, _ = timed(lambda: [r() for r in apart])
    pts = sum(n * n * m for n, m, _ in sizes)
    print(json.dumps({
        "workload": "mixed-ensemble", "metric": "Mpts·steps/s (ensembles of uneven sizes, one graph)",
        "ensembles": [{"grid": f"{n}x{n}", "members": m, "dt": dt} for n, m, dt in sizes],
        "precision": args.precision, "steps": steps, "graph_steps": graph_steps,
        "value": round(pts * steps / secs / 1e6, 2), "unit": UNIT,
        "ms_per_step": round(secs / steps * 1e3, 4),
        "one_size_after_another": {"value": round(pts * steps / secs_apart / 1e6, 2),
                                   "ms_per_step": round(secs_apart / steps * 1e3, 4)},
        "tiles": {f"{e.params.nx}": list(e.plan.get_tiles(2)) for e in ens},
        "l2": "flushed between graph launches"}), flush=True)
    return 0


def run_ddc_pool(args):
    """One slot pool of the solve server: 32 double-diffusive convection runs
    on a --n x (--n + 1) Fourier-x / Dirichlet-z grid (Ra_T = 1e6, Pr = 7,
    Le = 100, R_rho = 2, explicit AB2), advanced by batched steps."""
    import torch

    from melvin import serving

    device = torch.device("cuda", dist_env()[2])
    torch.cuda.set_device(device)
    nx, nz, slots = args.n, args.n + 1, 32
    srv = serving.Server(serving.DDCConfig(precision=args.precision), device=str(device))
    pool = serving._Pool(srv, nx, nz, slots)
    for s in range(slots):
        pool.admit(serving.Request(rid=s, nx=nx, nz=nz, r_rho=2.0, nsteps=args.steps, seed=s), srv.cfg)
    members = torch.arange(slots, dtype=torch.int32, device=device)
    for _ in range(args.warmup):
        pool.ens.step(pool.dt, members)
    torch.cuda.synchronize()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)
    ev = []
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        pool.ens.step(pool.dt, members)
        e1.record()
        ev.append((e0, e1))
    torch.cuda.synchronize()
    secs = sum(a.elapsed_time(b) for a, b in ev) * 1e-3
    print(json.dumps({"workload": "ddc-pool", "grid": f"{nx}x{nz}", "slots": slots, "precision": args.precision,
                      "steps": args.steps, "ms_per_step": round(secs / args.steps * 1e3, 4),
                      "value": round(slots * nx * nz * args.steps / secs / 1e6, 2), "unit": UNIT,
                      "l2": "flushed between steps",
                      "cpu_baseline": None if args.no_cpu else cpu_pool_sample("ddc", nx, slots)}), flush=True)
    return 0


def rbc_result(device, precision="double", steps=200, warmup=3, cpu=True, cpu_budget=6.0):
    """Rayleigh-Benard convection, one simulation: 1024 x 513 Fourier-x /
    Dirichlet-z grid, lx = 2, lz = 1, Ra = 1e7, Pr = 1, 4th-order finite
    differences in z, AB4/AM4 predictor-corrector, dt = 1e-7 (at Ra = 1e7
    the reference's dt = 1e-6 of examples/rayleigh_benard_convection.py
    overflows within 500 steps); temperature the conductive profile plus
    1e-3 seeded noise, vorticity zero.  L2 flushed between steps."""
    import torch

    import melvin
    from melvin import BasisFunctions as B, equations, workloads

    nx, nz = 1024, 513
    p = melvin.Parameters({"nx": nx, "nz": nz, "lx": 2.0, "lz": 1.0, "final_time": 1.0, "initial_dt": 1e-7,
                           "discretisation": ["spectral", "fdm"], "integrator": "explicit", "integrator_order": 4,
                           "spatial_derivative_order": 4, "precision": precision, "device": str(device)})
    sim = melvin.Simulation(p, torch)
    bf = [B.COMPLEX_EXP, B.FDM]
    w, dw = sim.make_variable("w", bf), sim.make_derivative("dw")
    t, dt_ = sim.make_variable("tmp", bf), sim.make_derivative("dtmp")
    t.load(workloads.conductive(nx, nz, 2.0, 1.0, seed=0), is_physical=True)
    step = equations.rayleigh_benard(sim, w, dw, t, dt_, 1.0, 1e7, integrator="pece")
    for _ in range(warmup):
        step.step()
    torch.cuda.synchronize()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)
    ev = []
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        step.step()
        e1.record()
        ev.append((e0, e1))
    torch.cuda.synchronize()
    secs = sum(a.elapsed_time(b) for a, b in ev) * 1e-3
    ms = secs / steps * 1e3
    # algorithmic bytes of one explicit evaluation (F = 2, AB4): 17 S + 10 P,
    # S = nn*nz complex128, P = nx*nz in the transform precision; the
    # predictor-corrector evaluates twice
    S = (nx - 1) // 3 * nz * 16
    P = nx * nz * (4 if precision == "split" else 8)
    bytes_step = 2 * (17 * S + 10 * P)
    peak, kind = load_peaks()
    return {"grid": f"{nx}x{nz}", "integrator": "AB4/AM4 predictor-corrector", "dt": 1e-7,
            "precision": precision, "steps": steps, "ms_per_step": round(ms, 4),
            "value": round(nx * nz * steps / secs / 1e6, 2), "unit": UNIT,
            "roofline": {"bound": "hbm", "algorithmic_bytes_per_step": bytes_step,
                         "step_achieved": round(bytes_step / (ms * 1e-3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                         "step_frac": round(bytes_step / (ms * 1e-3) / 1e9 / peak, 4), "peak_kind": kind},
            "l2": "flushed between steps",
            "cpu_baseline": cpu_pool_sample("rbc", nx, 1, cpu_budget) if cpu else None}


def run_rbc(args):
    import torch

    device = torch.device("cuda", dist_env()[2])
    torch.cuda.set_device(device)
    res = rbc_result(device, args.precision, args.steps, args.warmup, not args.no_cpu)
    print(json.dumps({"workload": "rbc", **res}), flush=True)
    return 0


def cpu_serving_sample(reqs, budget=4.0):
    """The oracle's per-core rate on each serving grid (double-diffusive
    convection on the Dirichlet grid, one member per core, the grids run at
    once in one spawn pool, each member time-bounded to `budget` seconds),
    and what it implies for the request mix: with all C cores each solving
    one request at a time, solves/s = C / mean over the requests of
    (grid points x steps / that grid's per-core rate)."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    grids = sorted({r.nx for r in reqs})
    cores = max(1, os.cpu_count() or 1)
    per = max(1, cores // len(grids))
    jobs = [("ddc", n, seed, budget) for n in grids for seed in range(per)]
    with ProcessPoolExecutor(max_workers=min(cores, len(jobs)), mp_context=mp.get_context("spawn")) as pool:
        res = list(pool.map(_oracle_member, jobs, timeout=20 * budget))
    rate = {}
    for (kind, n, seed, _), (pts, secs, _) in zip(jobs, res):
        rate.setdefault(n, []).append(pts / secs)
    rate = {n: sum(v) / len(v) for n, v in rate.items()}  # grid points x steps per second per core
    mean_s = sum(r.nx * r.nz * r.nsteps / rate[r.nx] for r in reqs) / len(reqs)
    pts = sum(r.nx * r.nz * r.nsteps for r in reqs) / len(reqs)
    return {"kind": "port", "cores": cores, "unit": "solves/s",
            "value": round(cores / mean_s, 5),
            "mpts_steps_per_s": round(cores * pts / mean_s / 1e6, 3),
            "per_core_mpts_steps_per_s": {f"{n}x{n + 1}": round(v / 1e6, 3) for n, v in rate.items()},
            "mean_solve_s_one_core": round(mean_s, 1),
            "sample": (f"{per} oracle members per grid at once ({len(jobs)} processes), each about {budget:.0f} s "
                       "of steps; solves/s implied for the same request mix with every core solving one "
                       "request at a time (no queueing)")}


def serving_result(device, precision="split", requests=100, rates=(50.0, 12.0), cpu=True, cpu_budget=4.0,
                   graphs=True):
    """Poisson streams of double-diffusive convection solves (Fourier-x /
    Dirichlet-z, grids 128x129..1024x1025, R_rho ~ U[1.5, 4], 200..2000
    steps, Ra_T = 1e6, Pr = 7, Le = 100) through the continuous-batching
    server, one run per arrival rate: the configuration's 50/s, which is
    above what the GPU finishes for this mix (the tail is the backlog), and
    a lower rate the GPU keeps up with (the tail is the service time).
    Chunks replay as captured CUDA graphs unless `graphs` is off."""
    from melvin import serving

    warm = serving.poisson_requests(8, rate=1000.0, seed=99, steps=(5, 10))
    serving.Server(serving.DDCConfig(precision=precision), device=str(device)).run(warm)
    runs = []
    for rate in rates:
        reqs = serving.poisson_requests(requests, rate=rate, seed=0)
        srv = serving.Server(serving.DDCConfig(precision=precision), device=str(device), graphs=graphs)
        summ = serving.summarize(srv.run(reqs))
        runs.append({"arrival_rate_per_s": rate,
                     **{k: round(v, 4) if isinstance(v, float) else v for k, v in summ.items()},
                     "pools": {f"{k[0]}x{k[1]}": p.ens.nslots for k, p in srv.pools.items()},
                     "admissions_deferred_for_memory": srv.refused, "chunk_graphs": srv.graph_stats()})
        del srv
    head = runs[0]
    return {"precision": precision, "value": head["solves_per_s"], "unit": "solves/s",
            "p50_s": head["p50_s"], "p99_s": head["p99_s"], "runs": runs,
            "cpu_baseline": cpu_serving_sample(serving.poisson_requests(requests, rate=rates[0], seed=0),
                                               cpu_budget) if cpu else None}


def run_serving(args):
    import torch

    device = torch.device("cuda", dist_env()[2])
    torch.cuda.set_device(device)
    res = serving_result(device, args.precision, args.requests, cpu=not args.no_cpu, graphs=not args.no_graphs)
    print(json.dumps({"workload": "ddc-serving", **res}), flush=True)
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["native", "reference"], default="native")
    ap.add_argument("--n", type=int, default=2048, help="grid points per side (default 2048)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-graphs", action="store_true", help="serving: launch every step from the host")
    ap.add_argument("--no-tune", action="store_true", help="keep the default tile variants (no autotuning)")
    ap.add_argument("--tiles", help="pin the tile variants x-inverse,z,x-forward (e.g. 0,1,1) instead of tuning")
    ap.add_argument("--only", choices=["fp64", "split", "dfloat"],
                    help="run only the timed fused steps of one precision")
    ap.add_argument("--workload", choices=["turbulence", "kh-ensemble", "mixed-ensemble", "ddc-pool", "serving", "rbc"],
                    default="turbulence",
                    help="turbulence: the headline line; kh-ensemble / serving: the batched and serving lines; "
                         "rbc: one Rayleigh-Benard simulation on a Dirichlet grid")
    ap.add_argument("--members", type=int, default=256, help="kh-ensemble members")
    ap.add_argument("--requests", type=int, default=200, help="serving requests")
    ap.add_argument("--headline-only", action="store_true",
                    help="default workload: leave out the rbc, kh_ensemble and serving sub-objects")
    ap.add_argument("--precision", help="precision of the kh-ensemble / serving workloads (default split) "
                                        "and of rbc (default double)")
    args = ap.parse_args(argv)
    if args.precision is None:
        args.precision = "double" if args.workload == "rbc" else "split"
    if args.warmup < 3 and args.impl == "native":
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "kh-ensemble":
        return run_ensemble(args)
    if args.workload == "mixed-ensemble":
        return run_mixed_ensemble(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "ddc-pool":
        return run_ddc_pool(args)
    if args.workload == "rbc":
        return run_rbc(args)
    if args.only:
        return run_only(args)
    return run_native(args)


if __name__ == "__main__":
    sys.exit(main())
