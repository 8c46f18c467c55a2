"""Autotuner for the tile variants of the fused timestep.

Each of the three kernels of a fully spectral fused step (the inverse x pass,
the z pass and the forward x pass) is built in a few tile variants: how many
columns (x passes) or pairs of grid rows (z pass) one CTA transforms, and the
largest FFT radix (``mgb_tile_info_get``).  Which variant is fastest depends
on the grid, the precision, the number of advected fields and the batch size,
so the tuner times them on the caller's own :class:`~melvin.Stepper` or
:class:`~melvin.ensemble.Ensemble` and sets the fastest on the plan
(``mgb_plan_set_tiles``).

The search is coordinate descent: starting from the current selection, each
family's variants are tried with the other two fixed, and a change is kept
when it is faster by more than ``min_gain``; two sweeps normally settle.
Every trial starts from the same saved state, and the state is put back at
the end, so tuning can happen at any point of a run.  A CUDA graph captured
before tuning keeps the kernels it captured; capture after tuning.

Variants that differ only in columns or row pairs per CTA give bit-identical
results; the radix-16 variant changes the rounding of the transforms (the FP64
path stays within the 1e-12 parity bound of every variant).

The reference has no counterpart: numpy.fft picks its own factorisation
inside ``rfft2``/``irfft2`` (melvin/SpectralTransformer.py:58,85,132,191).
"""

from __future__ import annotations

import dataclasses
import json
import os
import threading

from . import _native as N

_memo = {}
_memo_lock = threading.Lock()


@dataclasses.dataclass
class TuneResult:
    tiles: tuple | None          # selected variant per family (xinv, zstep, xfwd); None when not tunable
    ms_per_step: float | None    # time of one step with the selection
    default_ms_per_step: float | None
    trials: list                 # [(tiles, ms_per_step)] in the order tried
    key: str
    cached: bool = False

    @property
    def speedup(self):
        if not self.ms_per_step or not self.default_ms_per_step:
            return None
        return self.default_ms_per_step / self.ms_per_step


def variants(plan, nfields):
    """Available variants of each family, one per distinct (shape, radix, kind)."""
    out = []
    for fam in range(len(N.FAMILIES)):
        seen, lst = set(), []
        for v in range(N.TILE_VARIANTS):
            ok, shape, radix, _, kind = plan.tile_info(fam, nfields, v)
            if ok and (shape, radix, kind) not in seen:
                seen.add((shape, radix, kind))
                lst.append(v)
        out.append(lst)
    return out


def describe(plan, nfields):
    """{family: [(variant, available, shape, radix, smem_bytes)]} for reports."""
    return {
        name: [(v, *plan.tile_info(fam, nfields, v)) for v in range(N.TILE_VARIANTS)]
        for fam, name in enumerate(N.FAMILIES)
    }


def cache_key(plan, nfields, batch):
    import torch

    g = plan.grid
    name = torch.cuda.get_device_name(plan.device) if plan.device.type == "cuda" else "cpu"
    return f"{name}|{g.nx}x{g.nz}|sdo{g.sdo}|prec{g.precision}|F{nfields}|B{batch}"


# ---------------------------------------------------------------------------
# targets: what is stepped, how its state is saved and restored
# ---------------------------------------------------------------------------


class _StepperTarget:
    def __init__(self, stepper, dt):
        self.obj = stepper
        self.plan = stepper.plan
        self.nfields = len(stepper.fields)
        self.batch = 1
        self.dt = stepper.sim._integrator._dt if dt is None else float(dt)

    def step(self):
        self.obj.step(self.dt)

    def save(self):
        fs = self.obj.fields
        return ([f.var._sdata.clone() for f in fs], [f.dvar._data.clone() for f in fs],
                [f.dvar._curr_idx for f in fs])

    def restore(self, snap):
        q, h, idx = snap
        for f, a, b, i in zip(self.obj.fields, q, h, idx):
            f.var._sdata.copy_(a)
            f.dvar._data.copy_(b)
            f.dvar._curr_idx = i


class _EnsembleTarget:
    def __init__(self, ens, dt, members):
        self.obj = ens
        self.plan = ens.plan
        self.nfields = ens.F
        self.members = members
        self.batch = ens.nslots if members is None else int(members.numel())
        if dt is None:
            raise ValueError("tuning an Ensemble needs its dt")
        self.dt = float(dt)

    def step(self):
        self.obj.step(self.dt, self.members)

    def save(self):
        e = self.obj
        return e.q.clone(), e.hist.clone(), e.curr, e._stepped

    def restore(self, snap):
        q, h, curr, stepped = snap
        self.obj.q.copy_(q)
        self.obj.hist.copy_(h)
        self.obj.curr, self.obj._stepped = curr, stepped


def _target(obj, dt, members):
    from .ensemble import Ensemble

    if isinstance(obj, Ensemble):
        return _EnsembleTarget(obj, dt, members)
    if hasattr(obj, "fields") and hasattr(obj, "plan"):
        return _StepperTarget(obj, dt)
    raise TypeError(f"cannot tune a {type(obj).__name__}: expected a Stepper or an Ensemble")


def _time_steps(t, steps, reps):
    """Best over `reps` of the mean device time of `steps` steps (ms)."""
    import torch

    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            t.step()
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / steps)
    return best


def search(measure, choices, start, rounds=2, min_gain=0.02):
    """Coordinate descent over the families: `measure(tiles) -> ms`,
    `choices[f]` the variants of family f, `start` the initial selection.
    Returns (best tiles, best ms, default ms, trials)."""
    best = tuple(start)
    trials = []
    t0 = measure(best)
    trials.append((best, t0))
    cur = t0
    for _ in range(rounds):
        changed = False
        for fam, opts in enumerate(choices):
            for v in opts:
                if v == best[fam]:
                    continue
                cand = tuple(v if k == fam else best[k] for k in range(len(best)))
                t = measure(cand)
                trials.append((cand, t))
                if t < cur * (1.0 - min_gain):
                    best, cur, changed = cand, t, True
        if not changed:
            break
    return best, cur, t0, trials


def _load_file(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def tune(obj, dt=None, members=None, steps=4, reps=3, rounds=2, min_gain=0.02, cache_path=None, force=False):
    """Time the tile variants of `obj`'s fused step (a Stepper or an
    Ensemble; `dt` required for an Ensemble, `members` its slot list) and
    set the fastest on its plan.  Results are remembered per device, grid,
    precision, field count and batch size for the life of the process and,
    when `cache_path` (or the environment variable MELVIN_TILE_CACHE) names a
    JSON file, across processes."""
    t = _target(obj, dt, members)
    plan, F = t.plan, t.nfields
    if plan.grid.fdm_z:
        return TuneResult(None, None, None, [], "fdm", cached=False)
    key = cache_key(plan, F, t.batch)
    cache_path = cache_path or os.environ.get("MELVIN_TILE_CACHE")
    if not force:
        with _memo_lock:
            hit = _memo.get(key)
        if hit is None and cache_path:
            hit = _load_file(cache_path).get(key)
        if hit is not None:
            plan.set_tiles(F, hit["tiles"])
            return TuneResult(tuple(hit["tiles"]), hit.get("ms"), hit.get("default_ms"), [], key, cached=True)

    choices = variants(plan, F)
    start = plan.get_tiles(F)
    snap = t.save()

    def measure(tiles):
        plan.set_tiles(F, tiles)
        t.restore(snap)
        t.step()  # first launch of a variant: shared-memory opt-in, instruction cache
        return _time_steps(t, steps, reps)

    try:
        best, ms, ms0, trials = search(measure, choices, start, rounds=rounds, min_gain=min_gain)
    finally:
        t.restore(snap)
    plan.set_tiles(F, best)
    entry = {"tiles": list(best), "ms": ms, "default_ms": ms0}
    with _memo_lock:
        _memo[key] = entry
    if cache_path:
        data = _load_file(cache_path)
        data[key] = entry
        tmp = f"{cache_path}.tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, cache_path)
    return TuneResult(best, ms, ms0, trials, key)
