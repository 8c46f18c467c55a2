"""Ensembles: every member of a batched step equals the same simulation run
alone (the per-member arithmetic is identical, so to rounding; 1e-12
relative L2 asserted), graph replay equals step-by-step execution, member
lists advance only the listed slots, and per-slot term coefficients act
like per-run equations."""

import numpy as np
import pytest
import torch

import oracle as O
from oracle import problems as P
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def kh_params(nx, nz, precision="double"):
    import melvin

    return melvin.Parameters({"nx": nx, "nz": nz, "lx": 2 * np.pi, "lz": 2 * np.pi, "final_time": 1.0,
                              "initial_dt": 5e-3, "precision": precision, "device": "cuda:0"})


def kh_members(g, B):
    out = []
    for b in range(B):
        w, c = P.kh_ic(g, 0.2 + 0.05 * b, seed=b)
        out.append((w, c))
    return out


@pytest.mark.parametrize("precision", ["double", "split"])
def test_ensemble_members_equal_single_runs(cuda, precision):
    import melvin
    from melvin import BasisFunctions as B, equations
    from melvin.ensemble import Ensemble, FieldSpec

    g = O.Grid(64, 32, 2 * np.pi, 2 * np.pi)
    p = kh_params(64, 32, precision)
    nb = 5
    ics = kh_members(g, nb)
    ens = Ensemble(p, [FieldSpec(1e-3), FieldSpec(2e-3)], nb)
    for b, (w, c) in enumerate(ics):
        ens.load_physical(b, [w, c])
    for _ in range(6):
        ens.step(5e-3)
    for b, (w0, c0) in enumerate(ics):
        sim = melvin.Simulation(p, torch)
        bf = [B.COMPLEX_EXP, B.COMPLEX_EXP]
        w, c = sim.make_variable("w", bf), sim.make_variable("c", bf)
        dw, dc = sim.make_derivative("dw"), sim.make_derivative("dc")
        w.load(w0, is_physical=True)
        c.load(c0, is_physical=True)
        st = equations.kelvin_helmholtz(sim, w, dw, c, dc, 1e-3, 2e-3)
        for _ in range(6):
            st.step(5e-3)
        assert rel_l2(ens.q[b, 0].cpu().numpy(), w.gets().cpu().numpy()) < TOL
        assert rel_l2(ens.q[b, 1].cpu().numpy(), c.gets().cpu().numpy()) < TOL
        if precision == "double":
            ref = P.Problem(g, P.kh_specs(1e-3, 2e-3), [O.to_spectral(g, w0), O.to_spectral(g, c0)], 5e-3)
            for _ in range(6):
                ref.step()
            assert rel_l2(ens.q[b, 0].cpu().numpy(), ref.q[0]) < TOL


def test_graph_replay_equals_steps(cuda):
    from melvin.ensemble import Ensemble, FieldSpec

    g = O.Grid(64, 32, 2 * np.pi, 2 * np.pi)
    p = kh_params(64, 32, "split")
    ics = kh_members(g, 3)
    a = Ensemble(p, [FieldSpec(1e-3), FieldSpec(2e-3)], 3)
    b = Ensemble(p, [FieldSpec(1e-3), FieldSpec(2e-3)], 3)
    for k, (w, c) in enumerate(ics):
        a.load_physical(k, [w, c])
        b.load_physical(k, [w, c])
    a.step(5e-3)
    b.step(5e-3)
    replay = a.graph(5e-3, 4)
    for _ in range(3):
        replay()
    for _ in range(12):
        b.step(5e-3)
    torch.cuda.synchronize()
    assert torch.equal(a.q, b.q)
    assert torch.equal(a.hist, b.hist)


def test_member_list_advances_only_listed_slots(cuda):
    from melvin.ensemble import Ensemble, FieldSpec

    g = O.Grid(64, 32, 2 * np.pi, 2 * np.pi)
    p = kh_params(64, 32)
    ics = kh_members(g, 4)
    ens = Ensemble(p, [FieldSpec(1e-3), FieldSpec(2e-3)], 4)
    for k, (w, c) in enumerate(ics):
        ens.load_physical(k, [w, c])
    before = ens.q.clone()
    members = torch.tensor([3, 1], dtype=torch.int32, device=cuda)
    for _ in range(4):
        ens.step(5e-3, members)
    assert torch.equal(ens.q[0], before[0]) and torch.equal(ens.q[2], before[2])
    ref = Ensemble(p, [FieldSpec(1e-3), FieldSpec(2e-3)], 1)
    ref.load_physical(0, list(ics[3]))
    for _ in range(4):
        ref.step(5e-3)
    assert rel_l2(ens.q[3].cpu().numpy(), ref.q[0].cpu().numpy()) < TOL


def test_per_slot_term_coefficients(cuda):
    """Double-diffusive convection on the Dirichlet grid with a density ratio
    per slot equals runs with that ratio in the equation."""
    import melvin
    from melvin.ensemble import Ensemble, FieldSpec

    Pr, RaT, Le = 7.0, 1e5, 10.0
    ratios = [1.5, 2.5, 4.0]
    g = O.Grid(32, 17, 2.0, 1.0, True, 2)
    p = melvin.Parameters({"nx": 32, "nz": 17, "lx": 2.0, "lz": 1.0, "final_time": 1.0, "initial_dt": 2e-6,
                           "discretisation": ["spectral", "fdm"], "integrator": "explicit", "device": "cuda:0"})
    fields = [FieldSpec(Pr, [(1, "ddx", -Pr * RaT), (2, "ddx", 0.0)], 2), FieldSpec(1.0, [], 4),
              FieldSpec(1.0 / Le, [], 4)]
    tco = np.zeros((3, 3, 4))
    for k, r in enumerate(ratios):
        tco[k, 0, 0] = -Pr * RaT
        tco[k, 0, 1] = Pr * RaT / r
    ens = Ensemble(p, fields, 3, term_coef=tco)
    t0 = P.conductive_ic(g, seed=1)
    s0 = P.conductive_ic(g, seed=2)
    for k in range(3):
        ens.load_physical(k, [np.zeros((32, 17)), t0, s0])
    for _ in range(5):
        ens.step(2e-6)
    for k, r in enumerate(ratios):
        ref = P.Problem(g, P.ddc_dirichlet_specs(Pr, RaT, r, Le),
                        [np.zeros(g.spectral_shape, complex), O.to_spectral(g, t0), O.to_spectral(g, s0)], 2e-6,
                        "explicit", 2)
        for _ in range(5):
            ref.step()
        for f in range(3):
            assert rel_l2(ens.q[k, f].cpu().numpy(), ref.q[f]) < TOL, (k, f)


def _mixed_group(seed_shift=0):
    import melvin
    from melvin import _native as N
    from melvin.ensemble import Ensemble, EnsembleGroup, FieldSpec

    out = []
    for n, nb in ((64, 3), (128, 2)):
        g = O.Grid(n, n, 2 * np.pi, 2 * np.pi)
        ens = Ensemble(kh_params(n, n, "split"), [FieldSpec(1e-3), FieldSpec(2e-3)], nb)
        for b in range(nb):
            ens.load_physical(b, list(P.kh_ic(g, 0.2 + 0.05 * b, seed=b + seed_shift)))
        out.append(ens)
    p = melvin.Parameters({"nx": 64, "nz": 65, "lx": 2.0, "lz": 1.0, "final_time": 1.0, "initial_dt": 1e-6,
                           "discretisation": ["spectral", "fdm"], "integrator": "explicit", "precision": "split",
                           "device": "cuda:0"})
    Pr, RaT = 7.0, 1e5
    fields = [FieldSpec(Pr, [(1, "ddx", -Pr * RaT), (2, "ddx", Pr * RaT / 2.0)], N.BC_DIRICHLET_W),
              FieldSpec(1.0, [], N.BC_DIRICHLET_T), FieldSpec(0.01, [], N.BC_DIRICHLET_T)]
    ddc = Ensemble(p, fields, 2)
    from melvin.workloads import conductive
    for b in range(2):
        ddc.load_physical(b, [np.zeros((64, 65)), conductive(64, 65, 2.0, 1.0, seed=b), conductive(64, 65, 2.0, 1.0,
                                                                                                   seed=9 + b)])
    out.append(ddc)
    return EnsembleGroup(out), [5e-3, 5e-3, 1e-6]


def test_group_graph_equals_individual_steps(cuda):
    grp_a, dts = _mixed_group()
    for e, d in zip(grp_a.ensembles, dts):
        e.step(d)
    replay = grp_a.graph(dts, 4)
    replay()
    replay()
    grp_b, _ = _mixed_group()
    for e, d in zip(grp_b.ensembles, dts):
        for _ in range(9):
            e.step(d)
    torch.cuda.synchronize()
    for ea, eb in zip(grp_a.ensembles, grp_b.ensembles):
        assert ea.curr == eb.curr
        assert torch.equal(ea.q, eb.q)
        assert torch.equal(ea.hist, eb.hist)


def test_group_rejects_shared_plans(cuda):
    from melvin.ensemble import Ensemble, EnsembleGroup, FieldSpec

    a = Ensemble(kh_params(64, 64), [FieldSpec(1e-3)], 2)
    b = Ensemble(kh_params(64, 64), [FieldSpec(1e-3)], 3)
    with pytest.raises(ValueError):
        EnsembleGroup([a, b])


@pytest.mark.parametrize("precision", ["double", "split"])
def test_dirichlet_member_bits_independent_of_batch_size(cuda, precision):
    """The Dirichlet-grid x-forward pass narrows its tile (column pairs per
    CTA) when a launch is small.  A member's arithmetic does not depend on
    the tile: one run alone (a quarter-width tile) and the same run inside a
    160-member batch (the full tile) are bit-identical."""
    import melvin
    from melvin import _native as N
    from melvin.ensemble import Ensemble, FieldSpec
    from melvin.workloads import conductive

    p = melvin.Parameters({"nx": 64, "nz": 65, "lx": 2.0, "lz": 1.0, "final_time": 1.0, "initial_dt": 1e-6,
                           "discretisation": ["spectral", "fdm"], "integrator": "explicit", "precision": precision,
                           "device": "cuda:0"})
    Pr, RaT = 7.0, 1e5
    fields = [FieldSpec(Pr, [(1, "ddx", -Pr * RaT), (2, "ddx", Pr * RaT / 2.0)], N.BC_DIRICHLET_W),
              FieldSpec(1.0, [], N.BC_DIRICHLET_T), FieldSpec(0.01, [], N.BC_DIRICHLET_T)]
    ic = [np.zeros((64, 65)), conductive(64, 65, 2.0, 1.0, seed=1), conductive(64, 65, 2.0, 1.0, seed=2)]
    alone = Ensemble(p, fields, 1)
    alone.load_physical(0, ic)
    batch = Ensemble(p, fields, 160)
    for b in range(160):
        batch.load_physical(b, ic if b == 0 else [np.zeros((64, 65)), conductive(64, 65, 2.0, 1.0, seed=10 + b),
                                                  conductive(64, 65, 2.0, 1.0, seed=400 + b)])
    for _ in range(6):
        alone.step(1e-6)
        batch.step(1e-6)
    assert torch.equal(alone.q[0], batch.q[0])
    assert torch.equal(alone.hist[0], batch.hist[0])
