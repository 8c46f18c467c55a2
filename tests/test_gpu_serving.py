"""The continuous-batching server: a request's result is the same alone and
in a mix (members' arithmetic does not depend on slot, batch composition
or the shared history slot index; asserted bit-exact), results match the
oracle, and admission is refused when device memory is short."""

import numpy as np
import pytest
import torch

import oracle as O
from oracle import problems as P
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _cfg(precision):
    from melvin.serving import DDCConfig

    return DDCConfig(Ra_T=1e5, precision=precision)


class StepClock:
    """A deterministic server clock: every reading advances it by `tick`
    seconds, so arrivals are ordered by engine iterations, not by how fast
    the GPU happens to run."""

    def __init__(self, tick=1e-3):
        self.t, self.tick = 0.0, tick

    def __call__(self):
        self.t += self.tick
        return self.t


def test_result_same_alone_and_in_mix(cuda):
    """The target arrives a few engine iterations after five other requests,
    three of them on its grid with 400 steps each (25 chunks of 16 steps, at
    most one chunk per pool and iteration), so it is admitted while they run
    and shares their batched launches.  Its result is bit-identical to the
    same request served alone."""
    from melvin.serving import Request, Server

    target = Request(rid=0, nx=64, nz=33, r_rho=2.0, nsteps=40, arrival=0.005, seed=7)
    alone = Server(_cfg("split"), slots_per_block=4).run([target], keep_results=True, time_fn=StepClock())[0]
    assert alone.max_batch == 1
    mix = [Request(rid=i + 1, nx=nx, nz=nz, r_rho=1.5 + 0.5 * i, nsteps=400, arrival=0.0, seed=100 + i)
           for i, (nx, nz) in enumerate([(64, 33), (32, 17), (64, 33), (128, 65), (64, 33)])]
    target2 = Request(rid=0, nx=64, nz=33, r_rho=2.0, nsteps=40, arrival=0.005, seed=7)
    out = Server(_cfg("split"), slots_per_block=4).run(mix + [target2], keep_results=True, time_fn=StepClock())
    assert np.array_equal(target2.result, alone.result)
    assert all(r.finished is not None and r.finished >= r.arrival for r in out)
    # it ran inside a batch: all three same-grid requests were in its launches
    assert target2.max_batch == 4, target2.max_batch
    same = [r for r in mix if (r.nx, r.nz) == (64, 33)]
    assert all(r.admitted < target2.admitted < target2.finished < r.finished for r in same)


def test_chunk_graphs_match_per_step_launches(cuda):
    """Chunks replayed as captured graphs (over a member table rewritten as
    requests join and leave, and a pool that grows) give every request the
    same bits as launching each step from the host."""
    from melvin.serving import Request, Server

    def reqs():
        return [Request(rid=i, nx=nx, nz=nz, r_rho=1.5 + 0.25 * i, nsteps=n, arrival=a, seed=50 + i)
                for i, (nx, nz, n, a) in enumerate([(64, 33, 37, 0.0), (64, 33, 21, 0.002), (32, 17, 45, 0.0),
                                                    (64, 33, 50, 0.004), (64, 33, 19, 0.006), (32, 17, 3, 0.01)])]

    runs = {}
    for graphs in (False, True):
        srv = Server(_cfg("split"), slots_per_block=2, graphs=graphs)
        out = srv.run(reqs(), keep_results=True, time_fn=StepClock())
        runs[graphs] = ({r.rid: r.result for r in out}, srv.graph_stats())
    for rid, res in runs[False][0].items():
        assert np.array_equal(res, runs[True][0][rid]), rid
    assert runs[False][1] == {"captures": 0, "replays": 0}
    st = runs[True][1]
    assert st["captures"] > 0 and st["replays"] > st["captures"], st


def test_served_result_matches_oracle(cuda):
    from melvin.serving import Request, Server

    cfg = _cfg("double")
    req = Request(rid=0, nx=32, nz=17, r_rho=2.5, nsteps=6, seed=3)
    res = Server(cfg, slots_per_block=2).run([req], keep_results=True)[0].result
    g = O.Grid(32, 17, cfg.lx, cfg.lz, True, cfg.order)
    from melvin.workloads import conductive

    t0 = conductive(32, 17, cfg.lx, cfg.lz, seed=6)
    s0 = conductive(32, 17, cfg.lx, cfg.lz, seed=7)
    dt = cfg.dt_factor * (cfg.lz / 17) ** 2 / cfg.Pr
    ref = P.Problem(g, P.ddc_dirichlet_specs(cfg.Pr, cfg.Ra_T, 2.5, cfg.Le),
                    [np.zeros(g.spectral_shape, complex), O.to_spectral(g, t0), O.to_spectral(g, s0)], dt,
                    "explicit", 2)
    for _ in range(6):
        ref.step()
    for f in range(3):
        assert rel_l2(res[f], ref.q[f]) < 1e-12


def test_admission_waits_for_memory(cuda, monkeypatch):
    from melvin.serving import Request, Server

    srv = Server(_cfg("split"), slots_per_block=2)
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda device=None: (1 << 20, 1 << 30))
    assert srv._pool_for(Request(rid=0, nx=64, nz=33, r_rho=2.0, nsteps=1)) is None
    assert srv.refused == 1 and not srv.pools
