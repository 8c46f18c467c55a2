"""Tile variants of the fused step and the autotuner.

* Every available variant of every kernel family keeps the FP64 parity
  bound: 1e-12 relative L2 of every field after every step against the
  reference trajectories (golden vectors), and against the oracle on larger
  grids.
* Variants that differ only in columns or row pairs per CTA give
  bit-identical states; the radix-16 variant stays within 1e-13 (FP64) or
  1e-6 (split precision) of the default.
* The tuner leaves the stepped object's state bit-identical to what it
  was, and the selection it sets steps like the default.
"""

import numpy as np
import pytest
import torch

import oracle as O
from oracle import problems as P
from cases import TRAJ_CASES, params_dict
from conftest import rel_l2
from test_gpu_step import build, stepper_for

pytestmark = pytest.mark.gpu
TOL = 1e-12


def one_family_variants(plan, F):
    """The default selection and every selection that changes one family."""
    from melvin.autotune import variants

    out = [(0, 0, 0)]
    for fam, opts in enumerate(variants(plan, F)):
        for v in opts:
            if v:
                t = [0, 0, 0]
                t[fam] = v
                out.append(tuple(t))
    return out


def radix_changed(plan, F, tiles):
    """The selection changes a family's FFT radix or kind of transform against
    variant 0 (so the rounding changes, not only the CTA work split)."""
    def key(fam, v):
        info = plan.tile_info(fam, F, v)
        return info[2], info[4]

    return any(key(fam, v) != key(fam, 0) for fam, v in enumerate(tiles))


@pytest.mark.parametrize("tag", ["tg32_o2_ab2", "tg32_o4_ab4", "kh64x32", "ddcs32"])
def test_every_variant_matches_reference_trajectory(cuda, golden, tag):
    g, specs, names, integ, order, dt = TRAJ_CASES[tag]
    sim, p, V, D, bf = build(g, names, integ, order, dt)
    step = stepper_for(tag, sim, V, D, integ)
    F = len(names)
    plan = step.plan
    tried = one_family_variants(plan, F)
    assert len(tried) > 3
    default = plan.get_tiles(F)
    try:
        for tiles in tried:
            plan.set_tiles(F, tiles)
            assert plan.get_tiles(F) == tiles
            for n in names:
                V[n].sets(golden[f"{tag}/s0_{n}"])
                D[n]._data.zero_()
                D[n].set_curr_idx(0)
            kes = []
            for s in range(int(golden[f"{tag}/nsteps"])):
                kes.append(float(step.step(diagnostics=True)[0].item()))
                for n in names:
                    err = rel_l2(V[n].gets().cpu().numpy(), golden[f"{tag}/s{s + 1}_{n}"])
                    assert err < TOL, (tiles, s, n, err)
            assert rel_l2(np.array(kes), golden[f"{tag}/ke"]) < TOL, tiles
    finally:
        plan.set_tiles(F, default)


def _turbulence_states(n, precision, F, tiles_list, nsteps=2):
    """Final spectral states after `nsteps` from one initial condition, per
    tile selection; with the oracle's FP64 result for n <= 512."""
    import melvin
    from melvin import BasisFunctions as B, equations, workloads

    g = O.Grid(n, n, 2 * np.pi, 2 * np.pi)
    p = melvin.Parameters(params_dict(g, dt=2e-4, precision=precision))
    sim = melvin.Simulation(p, torch)
    bf = [B.COMPLEX_EXP, B.COMPLEX_EXP]
    w, dw = sim.make_variable("w", bf), sim.make_derivative("dw")
    w0 = workloads.decaying_turbulence(n, n, seed=2)
    if F == 1:
        step = equations.vorticity(sim, w, dw, 5e-5)
        ics = [w0]
        fields = [(w, dw)]
    else:
        c, dc = sim.make_variable("c", bf), sim.make_derivative("dc")
        c0 = workloads.decaying_turbulence(n, n, seed=3)
        step = equations.kelvin_helmholtz(sim, w, dw, c, dc, 5e-5, 1e-4)
        ics = [w0, c0]
        fields = [(w, dw), (c, dc)]
    out = {}
    default = step.plan.get_tiles(F)
    try:
        for tiles in tiles_list:
            step.plan.set_tiles(F, tiles)
            for (v, d), a in zip(fields, ics):
                v.load(a, is_physical=True)
                d._data.zero_()
                d.set_curr_idx(0)
            for _ in range(nsteps):
                step.step(2e-4)
            out[tiles] = [v.gets().clone() for v, _ in fields]
    finally:
        step.plan.set_tiles(F, default)
    return step.plan, g, ics, out


@pytest.mark.parametrize("n,precision,F", [(512, "double", 1), (256, "double", 2), (512, "split", 1),
                                           (256, "split", 2), (2048, "split", 1), (2048, "double", 1),
                                           (512, "dfloat", 1), (2048, "dfloat", 1)])
def test_variants_agree(cuda, n, precision, F):
    import melvin

    g = O.Grid(n, n, 2 * np.pi, 2 * np.pi)
    plan = melvin._native.plan_for(melvin.Parameters(params_dict(g, dt=2e-4, precision=precision)))
    tiles_list = one_family_variants(plan, F)
    plan, g, ics, out = _turbulence_states(n, precision, F, tiles_list)
    base = out[(0, 0, 0)]
    for tiles, st in out.items():
        for a, b in zip(st, base):
            if radix_changed(plan, F, tiles):
                err = (torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)).item()
                assert err < (1e-6 if precision == "split" else 1e-13), (tiles, err)
            else:
                assert torch.equal(a, b), tiles
    if precision != "split" and n <= 512:
        specs = P.vorticity_specs(5e-5) if F == 1 else P.kh_specs(5e-5, 1e-4)
        ref = P.Problem(g, specs, [O.to_spectral(g, a) for a in ics], 2e-4)
        for _ in range(2):
            ref.step()
        for tiles, st in out.items():
            for f in range(F):
                assert rel_l2(st[f].cpu().numpy(), ref.q[f]) < TOL, (tiles, f)


def test_tune_stepper_restores_state(cuda):
    import melvin
    from melvin import BasisFunctions as B, equations, workloads

    g = O.Grid(256, 256, 2 * np.pi, 2 * np.pi)
    p = melvin.Parameters(params_dict(g, dt=1e-3))
    sim = melvin.Simulation(p, torch)
    bf = [B.COMPLEX_EXP, B.COMPLEX_EXP]
    w, dw = sim.make_variable("w", bf), sim.make_derivative("dw")
    w0 = P.taylor_green_ic(g, seed=4)
    w.load(w0, is_physical=True)
    step = equations.vorticity(sim, w, dw, 1e-2)
    ref = P.Problem(g, P.vorticity_specs(1e-2), [O.to_spectral(g, w0)], 1e-3)
    for _ in range(3):
        step.step()
        ref.step()
    before = (w._sdata.clone(), dw._data.clone(), dw._curr_idx)
    default = step.plan.get_tiles(1)
    try:
        res = step.autotune(force=True)
        assert torch.equal(w._sdata, before[0]) and torch.equal(dw._data, before[1]) and dw._curr_idx == before[2]
        assert step.plan.get_tiles(1) == res.tiles
        assert len(res.trials) >= 4 and res.ms_per_step <= res.default_ms_per_step
        again = step.autotune()
        assert again.cached and again.tiles == res.tiles
        for _ in range(2):
            step.step()
            ref.step()
        assert rel_l2(w.gets().cpu().numpy(), ref.q[0]) < TOL
    finally:
        step.plan.set_tiles(1, default)


def test_tune_ensemble_members(cuda):
    import melvin
    from melvin.ensemble import Ensemble, FieldSpec

    n, nb, dt = 128, 6, 5e-4
    g = O.Grid(n, n, 2 * np.pi, 2 * np.pi)
    p = melvin.Parameters({"nx": n, "nz": n, "lx": 2 * np.pi, "lz": 2 * np.pi, "final_time": 1.0,
                           "initial_dt": dt, "precision": "split", "device": "cuda:0"})
    ens = Ensemble(p, [FieldSpec(1e-4), FieldSpec(1e-4)], nb)
    for b in range(nb):
        ens.load_physical(b, list(P.kh_ic(g, 0.05 + 0.01 * b, seed=b)))
    members = torch.tensor([1, 3, 4], dtype=torch.int32, device=cuda)
    ens.step(dt, members)
    q0, h0, c0 = ens.q.clone(), ens.hist.clone(), ens.curr
    default = ens.plan.get_tiles(2)
    for _ in range(4):
        ens.step(dt, members)
    a = ens.q.clone()
    ens.q.copy_(q0)
    ens.hist.copy_(h0)
    ens.curr = c0
    try:
        res = ens.autotune(dt, members, force=True)
        assert torch.equal(ens.q, q0) and torch.equal(ens.hist, h0) and ens.curr == c0
        assert ens.plan.get_tiles(2) == res.tiles
        for _ in range(4):
            ens.step(dt, members)
        err = (torch.linalg.vector_norm(ens.q - a) / torch.linalg.vector_norm(a)).item()
        assert err < 1e-6, (res.tiles, err)
        # slots outside the member list were never touched
        for s in (0, 2, 5):
            assert torch.equal(ens.q[s], q0[s])
    finally:
        ens.plan.set_tiles(2, default)
