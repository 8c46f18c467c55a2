"""A solve server with continuous batching.

Requests are double-diffusive convection solves on the Fourier-x /
Dirichlet-z grid (the equations of :func:`melvin.equations.double_diffusive_dirichlet`,
composed from examples/double_diffusive_convection.py:106-120 and
examples/rayleigh_benard_convection.py:97-142), each with its own grid
size, density ratio and step count.

* Every grid size has a slot pool (an :class:`~melvin.ensemble.Ensemble`)
  whose states stay on the GPU for the life of a request.
* Admission is by free device memory: a pool grows by a block of slots only
  when ``torch.cuda.mem_get_info`` shows room for it plus a reserve, and a
  request waits while its pool is full and cannot grow.
* Each engine iteration advances every active slot of every pool by one
  step -- one batched launch sequence per pool, pools on their own CUDA
  streams so their work overlaps -- so requests that arrive while others
  run join the batch at the next step and leave it when they finish.
* Every member's arithmetic is independent of which slot it has and who
  else is in the batch, so a result is the same alone and in the mix.
"""

from __future__ import annotations

import dataclasses
import time

import numpy as np
import torch

from . import _native as N
from .ensemble import Ensemble, FieldSpec
from .Parameters import Parameters
from .workloads import conductive


@dataclasses.dataclass
class Request:
    rid: int
    nx: int
    nz: int
    r_rho: float
    nsteps: int
    arrival: float = 0.0  # seconds after the server start
    seed: int = 0
    # filled by the server
    admitted: float = None
    finished: float = None
    result: np.ndarray = None  # final spectral states (3, rows, cols) when kept
    max_batch: int = 0         # most requests advanced together with this one in one batched launch


@dataclasses.dataclass
class DDCConfig:
    """Physics shared by all requests (Ra_T, Pr, Le) and the numerics."""

    Ra_T: float = 1e6
    Pr: float = 7.0
    Le: float = 100.0
    lx: float = 2.0
    lz: float = 1.0
    order: int = 2          # spatial_derivative_order
    integrator: str = "explicit"
    integrator_order: int = 2
    precision: str = "split"
    dt_factor: float = 0.1  # dt = dt_factor * dz^2 / Pr (explicit diffusion limit)


class _Pool:
    def __init__(self, server, nx, nz, nslots):
        cfg = server.cfg
        self.nx, self.nz = nx, nz
        self.params = Parameters({
            "nx": nx, "nz": nz, "lx": cfg.lx, "lz": cfg.lz, "final_time": 1.0,
            "discretisation": ["spectral", "fdm"], "integrator": cfg.integrator,
            "integrator_order": cfg.integrator_order, "spatial_derivative_order": cfg.order,
            "precision": cfg.precision, "device": str(server.device),
        })
        self.dt = cfg.dt_factor * self.params.dz ** 2 / cfg.Pr
        Pr, RaT = cfg.Pr, cfg.Ra_T
        self.fields = [FieldSpec(Pr, [(1, "ddx", -Pr * RaT), (2, "ddx", 0.0)], N.BC_DIRICHLET_W),
                       FieldSpec(1.0, [], N.BC_DIRICHLET_T),
                       FieldSpec(1.0 / cfg.Le, [], N.BC_DIRICHLET_T)]
        self.ens = Ensemble(self.params, self.fields, nslots, term_coef=np.zeros((nslots, 3, 4)))
        self.free = list(range(nslots))[::-1]
        self.active = {}  # slot -> [request, steps_done]
        self.members = None
        self.stream = torch.cuda.Stream(device=server.device)
        self.event = None
        self.use_graphs = server.use_graphs
        self.mtab = None    # member table: the active slots, rewritten when they change
        self.graphs = {}    # (members, steps, history slot) -> chunk-graph replay
        self.captures = self.replays = 0

    @staticmethod
    def bytes_per_slot(server, nx, nz):
        cfg = server.cfg
        nn = (nx - 1) // 3
        S = nn * nz * 16
        P = nx * nz * (4 if cfg.precision == "split" else 8)
        F, order = 3, cfg.integrator_order
        # state + history + step scratch (psi, 5 physical fields, 3 J, 3 predicted states)
        return F * S + F * order * S + S + 5 * P + 3 * P + 3 * S + (1 << 16)

    def grow(self, nslots):
        """Move the pool into a larger one (between engine iterations)."""
        old = self.ens
        new = Ensemble(self.params, self.fields, nslots, term_coef=np.zeros((nslots, 3, 4)))
        k = old.nslots
        with torch.cuda.stream(self.stream):
            new.q[:k].copy_(old.q)
            new.hist[:k].copy_(old.hist)
            new.term_coef[:k].copy_(old.term_coef)
        new.curr, new._stepped = old.curr, old._stepped
        self.ens = new
        self.free = list(range(k, nslots))[::-1] + self.free
        self.members = None
        self.mtab = None
        self.graphs.clear()  # they hold the old ensemble's buffers

    def admit(self, req, cfg):
        slot = self.free.pop()
        T0 = conductive(self.nx, self.nz, cfg.lx, cfg.lz, seed=2 * req.seed)
        S0 = conductive(self.nx, self.nz, cfg.lx, cfg.lz, seed=2 * req.seed + 1)
        with torch.cuda.stream(self.stream):
            self.ens.load_physical(slot, [np.zeros((self.nx, self.nz)), T0, S0])
            tc = self.ens.term_coef
            tc[slot].zero_()
            tc[slot, 0, 0] = -cfg.Pr * cfg.Ra_T
            tc[slot, 0, 1] = cfg.Pr * cfg.Ra_T / req.r_rho
        self.active[slot] = [req, 0]
        self.members = None

    def launch(self, chunk):
        """Queue up to `chunk` steps of every active slot on the pool's stream
        (no member overshoots its step count); returns the steps queued.

        With graphs on, the chunk is replayed as at most five CUDA graphs of
        16, 8, 4, 2 and 1 steps, each captured once per (member count, step
        count, history slot) over the pool's member table, whose contents
        change with admissions and retirements while its address stays."""
        if not self.active:
            return 0
        slots = sorted(self.active)
        if self.members is None:
            if not self.use_graphs:
                self.members = torch.tensor(slots, dtype=torch.int32, device=self.ens.device)
            else:
                if self.mtab is None:
                    self.mtab = torch.empty(self.ens.nslots, dtype=torch.int32, device=self.ens.device)
                with torch.cuda.stream(self.stream):  # ordered after the chunks that read the old table
                    self.mtab[:len(slots)].copy_(torch.tensor(slots, dtype=torch.int32))
                self.members = self.mtab[:len(slots)]
        k = min(chunk, min(r.nsteps - done for r, done in self.active.values()))
        with torch.cuda.stream(self.stream):
            left = k
            if not self.use_graphs or not self.ens._stepped:
                n0 = k if not self.use_graphs else 1
                for _ in range(n0):
                    self.ens.step(self.dt, self.members)
                left -= n0
            for size in (16, 8, 4, 2, 1):
                while left >= size:
                    key = (len(slots), size, self.ens.curr)
                    replay = self.graphs.get(key)
                    if replay is None:
                        replay = self.graphs[key] = self.ens.chunk_graph(self.dt, size, self.members, self.stream)
                        self.captures += 1
                    replay()
                    self.replays += 1
                    left -= size
            self.event = torch.cuda.Event()
            self.event.record(self.stream)
        for st in self.active.values():
            st[1] += k
            st[0].max_batch = max(st[0].max_batch, len(self.active))
        return k

    def busy(self):
        return self.event is not None and not self.event.query()

    def retire(self, now, keep):
        done = [s for s, (r, k) in self.active.items() if k >= r.nsteps]
        for s in done:
            req = self.active.pop(s)[0]
            req.finished = now
            if keep:
                with torch.cuda.stream(self.stream):
                    req.result = self.ens.q[s].cpu().numpy()
            self.free.append(s)
        if done:
            self.members = None
        return len(done)


class Server:
    def __init__(self, cfg: DDCConfig = None, device="cuda:0", slots_per_block=16, max_slots=256,
                 reserve_bytes=2 << 30, graphs=True):
        self.cfg = cfg or DDCConfig()
        self.use_graphs = bool(graphs)  # replay chunks as captured CUDA graphs
        self.device = torch.device(device)
        self.slots_per_block = slots_per_block
        self.max_slots = max_slots
        self.reserve = reserve_bytes
        self.pools = {}
        self.refused = 0  # admissions deferred for lack of memory

    def graph_stats(self):
        """Chunk graphs captured and replayed over all pools."""
        return {"captures": sum(p.captures for p in self.pools.values()),
                "replays": sum(p.replays for p in self.pools.values())}

    def _pool_for(self, req):
        key = (req.nx, req.nz)
        pool = self.pools.get(key)
        if pool is not None and pool.free:
            return pool
        have = 0 if pool is None else pool.ens.nslots
        if have >= self.max_slots:
            return None
        need = _Pool.bytes_per_slot(self, req.nx, req.nz) * self.slots_per_block
        free, _ = torch.cuda.mem_get_info(self.device)
        if free < need + self.reserve:
            self.refused += 1
            return None
        if pool is None:
            pool = _Pool(self, req.nx, req.nz, self.slots_per_block)
            self.pools[key] = pool
            return pool
        if pool.busy():
            return None  # grow between chunks only
        pool.grow(min(have + self.slots_per_block, self.max_slots))
        return pool

    def run(self, requests, keep_results=False, time_fn=time.perf_counter, chunk=16):
        """Serve `requests` (arrival times relative to the start) until all
        have finished; returns them with admission and finish times.

        Pools run independently: whenever a pool's queued chunk of steps has
        completed, its finished requests retire, waiting requests of its
        size join, and the next chunk (at most `chunk` steps) is queued on
        its stream."""
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        waiting = []
        t0 = time_fn()
        done = 0
        total = len(pending)
        while done < total:
            now = time_fn() - t0
            while pending and pending[0].arrival <= now:
                waiting.append(pending.pop(0))
            # retire finished chunks
            for pool in self.pools.values():
                if pool.event is not None and not pool.busy():
                    done += pool.retire(time_fn() - t0, keep_results)
                    pool.event = None
            # admit into pools that have a free slot (or can be created / grown)
            still = []
            for req in waiting:
                pool = self._pool_for(req)
                if pool is None or not pool.free:
                    still.append(req)
                    continue
                req.admitted = time_fn() - t0
                pool.admit(req, self.cfg)
            waiting = still
            # queue the next chunk of every idle pool
            running = False
            for pool in self.pools.values():
                if pool.event is None and pool.active:
                    pool.launch(chunk)
                running = running or pool.event is not None
            if not running:
                if pending:
                    time.sleep(max(0.0, min(pending[0].arrival - (time_fn() - t0), 0.001)))
            else:
                time.sleep(5e-5)
        return requests


def poisson_requests(n, rate=50.0, seed=0, grids=((128, 129), (256, 257), (512, 513), (1024, 1025)),
                     steps=(200, 2000), r_rho=(1.5, 4.0)):
    """`n` requests with Poisson arrivals at `rate` per second, grid sizes,
    step counts and density ratios drawn uniformly (seeded)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    out = []
    for i in range(n):
        nx, nz = grids[rng.integers(len(grids))]
        out.append(Request(rid=i, nx=int(nx), nz=int(nz), r_rho=float(rng.uniform(*r_rho)),
                           nsteps=int(rng.integers(steps[0], steps[1] + 1)), arrival=float(t[i]), seed=i))
    return out


def summarize(requests):
    tts = np.array([r.finished - r.arrival for r in requests])
    pts = sum(r.nx * r.nz * r.nsteps for r in requests)
    span = max(r.finished for r in requests) - min(r.arrival for r in requests)
    return {
        "requests": len(requests),
        "p50_s": float(np.percentile(tts, 50)),
        "p99_s": float(np.percentile(tts, 99)),
        "mean_s": float(np.mean(tts)),
        "solves_per_s": len(requests) / span,
        "mpts_steps_per_s": pts / span / 1e6,
        "span_s": span,
    }
