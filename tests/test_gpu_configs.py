"""The benchmark configurations run free on the GPU against the oracle
(the reference algorithm restated in NumPy, golden-pinned), at their own
grid sizes and step counts -- no restart from the oracle state.

* Taylor-Green 256^2 (nu = 1e-2, dt = 1e-3, AB2 semi-implicit, FP64), 1000
  steps: the vorticity after every step and the kinetic-energy history at
  1e-12 relative L2.  A free-running trajectory keeps the per-step bound:
  rounding differences of 2e-16 per element injected every step grow to
  no more than 1e-14 over the 1000 steps of this dissipative flow
  (measured with the oracle against itself).  Also the reference example's
  known answer (examples/taylor_green_vortex.py:97-106): the kinetic
  energy decays as exp(-4 nu t) for this mode.
* Rayleigh-Benard 1024x513 (Ra = 1e7, Pr = 1, 4th-order differences,
  AB4/AM4 predictor-corrector, dt = 1e-7), 50 steps: FP64 and double-float
  at 1e-12 per step, split precision at 1e-5 after the 50 steps.
* Decaying turbulence 2048^2 (nu = 5e-5, dt = 2e-4, AB2 semi-implicit),
  100 steps: FP64 and double-float at 1e-12 per step against the oracle;
  split precision within 1e-5 of the FP64 path after 1 and 100 steps,
  kinetic-energy trajectory within 1e-6 relative at every step.
* Kelvin-Helmholtz ensemble: 256 members at 256^2 (vorticity + passive
  scalar, nu = kappa = 1e-4, dt = 5e-4, delta ~ U[0.02, 0.1]), split
  precision, 400 steps as CUDA-graph replays of the batched step: the
  members with the thinnest and the thickest shear layer within 1e-5 of
  the oracle.  FP32-sized rounding (6e-8 per element per step, injected into
  the oracle) grows to 1.6e-6 over these 400 steps at delta = 0.02.
"""

import numpy as np
import pytest
import torch

import oracle as O
from oracle import problems as P
from cases import params_dict
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12
SPLIT_TOL = 1e-5
KE_SPLIT_TOL = 1e-6


def _spectral_run(g, precision, w0, nu, dt, order=2):
    import melvin
    from melvin import BasisFunctions as B, equations

    sim = melvin.Simulation(melvin.Parameters(params_dict(g, "semi-implicit", order, dt, precision)), torch)
    bf = [B.COMPLEX_EXP, B.COMPLEX_EXP]
    w, dw = sim.make_variable("w", bf), sim.make_derivative("dw")
    w.load(w0, is_physical=True)
    return w, equations.vorticity(sim, w, dw, nu)


def test_taylor_green_256_free_running_1000_steps(cuda):
    g = O.Grid(256, 256, 2 * np.pi, 2 * np.pi)
    nu, dt, nsteps = 1e-2, 1e-3, 1000
    w0 = P.taylor_green_ic(g, seed=0)
    w, step = _spectral_run(g, "double", w0, nu, dt)
    ref = P.Problem(g, P.vorticity_specs(nu), [O.to_spectral(g, w0)], dt)
    ke_gpu, ke_ref, worst = [], [], 0.0
    for s in range(nsteps):
        ke_gpu.append(step.step(diagnostics=True)[0].clone())
        vel = ref.step()
        ke_ref.append(O.kinetic_energy(g, vel["ux_p"], vel["uz_p"]))
        err = rel_l2(w.gets().cpu().numpy(), ref.q[0])
        worst = max(worst, err)
        assert err < TOL, (s, err)
    ke_gpu = torch.stack(ke_gpu).cpu().numpy()
    assert rel_l2(ke_gpu, np.array(ke_ref)) < TOL
    # the known answer of the reference example: KE(t)/KE(0) = exp(-4 nu t)
    # for the sin x sin z mode (to the seeded 1e-3 noise and the first-order
    # time error of the alpha = 0.51 scheme)
    t = (nsteps - 1) * dt  # the last sample is the velocity at the start of the last step
    assert abs(ke_gpu[-1] / ke_gpu[0] / np.exp(-4 * nu * t) - 1) < 1e-6
    print(f"TG 256^2: worst per-step rel L2 over {nsteps} steps {worst:.2e}")


@pytest.fixture(scope="module")
def rbc_runs(cuda):
    """RBC 1024x513 in FP64, double-float and split, stepped in lockstep
    with the oracle for 50 steps; returns the per-step errors."""
    import melvin
    from melvin import BasisFunctions as B, equations, workloads

    nx, nz, dt, nsteps = 1024, 513, 1e-7, 50
    g = O.Grid(nx, nz, 2.0, 1.0, True, 4)
    t0 = workloads.conductive(nx, nz, 2.0, 1.0, seed=0)
    runs = {}
    for prec in ("double", "dfloat", "split"):
        sim = melvin.Simulation(melvin.Parameters(params_dict(g, "explicit", 4, dt, prec)), torch)
        bf = [B.COMPLEX_EXP, B.FDM]
        w, dw, t, dtt = (sim.make_variable("w", bf), sim.make_derivative("dw"), sim.make_variable("t", bf),
                         sim.make_derivative("dt"))
        t.load(t0, is_physical=True)
        runs[prec] = (w, t, equations.rayleigh_benard(sim, w, dw, t, dtt, 1.0, 1e7, integrator="pece"))
    ref = P.Problem(g, P.rbc_specs(1.0, 1e7), [np.zeros(g.spectral_shape, complex), O.to_spectral(g, t0)], dt,
                    "pece", 4)
    errs = {p: [] for p in runs}
    for _ in range(nsteps):
        ref.step()
        for prec, (w, t, step) in runs.items():
            step.step()
            errs[prec].append((rel_l2(w.gets().cpu().numpy(), ref.q[0]), rel_l2(t.gets().cpu().numpy(), ref.q[1])))
    return errs


@pytest.mark.parametrize("precision", ["double", "dfloat"])
def test_rbc_1024x513_pece_50_steps_fp64_class(rbc_runs, precision):
    for s, (ew, et) in enumerate(rbc_runs[precision]):
        assert ew < TOL and et < TOL, (s, ew, et)


def test_rbc_1024x513_pece_50_steps_split(rbc_runs):
    ew, et = rbc_runs["split"][-1]
    assert ew < SPLIT_TOL and et < SPLIT_TOL, (ew, et)


@pytest.fixture(scope="module")
def turbulence_runs(cuda):
    """2048^2 decaying turbulence, 100 steps: FP64, double-float and split
    in lockstep with the oracle; per-step errors and kinetic energies."""
    from melvin import workloads

    n, nu, dt, nsteps = 2048, 5e-5, 2e-4, 100
    g = O.Grid(n, n, 2 * np.pi, 2 * np.pi)
    w0 = workloads.decaying_turbulence(n, n, seed=0)
    runs = {p: _spectral_run(g, p, w0, nu, dt) for p in ("double", "dfloat", "split")}
    ref = P.Problem(g, P.vorticity_specs(nu), [O.to_spectral(g, w0)], dt)
    out = {p: {"err_ref": [], "err_fp64": [], "ke": []} for p in runs}
    for _ in range(nsteps):
        ref.step()
        for p, (w, step) in runs.items():
            out[p]["ke"].append(step.step(diagnostics=True)[0].clone())
        w64 = runs["double"][0].gets()
        for p, (w, step) in runs.items():
            out[p]["err_ref"].append(rel_l2(w.gets().cpu().numpy(), ref.q[0]))
            out[p]["err_fp64"].append((torch.linalg.vector_norm(w.gets() - w64) / torch.linalg.vector_norm(w64)).item())
    for p in out:
        out[p]["ke"] = torch.stack(out[p]["ke"]).cpu().numpy()
    return out


@pytest.mark.parametrize("precision", ["double", "dfloat"])
def test_turbulence_2048_100_steps_fp64_class(turbulence_runs, precision):
    errs = turbulence_runs[precision]["err_ref"]
    for s, e in enumerate(errs):
        assert e < TOL, (s, e)


def test_turbulence_2048_100_steps_split(turbulence_runs):
    r, r64 = turbulence_runs["split"], turbulence_runs["double"]
    assert r["err_fp64"][0] < SPLIT_TOL, r["err_fp64"][0]
    assert r["err_fp64"][-1] < SPLIT_TOL, r["err_fp64"][-1]
    assert r["err_ref"][-1] < SPLIT_TOL, r["err_ref"][-1]
    ke_err = np.max(np.abs(r["ke"] - r64["ke"]) / np.abs(r64["ke"]))
    assert ke_err < KE_SPLIT_TOL, ke_err
    print(f"split 2048^2: rel L2 vs FP64 {r['err_fp64'][0]:.2e} (1 step), {r['err_fp64'][-1]:.2e} (100 steps); "
          f"KE trajectory {ke_err:.2e}")


def test_kh_ensemble_256_members_400_steps_split(cuda):
    import melvin
    from melvin import workloads
    from melvin.ensemble import Ensemble, FieldSpec

    n, members, dt, nsteps, graph_steps = 256, 256, 5e-4, 400, 8
    g = O.Grid(n, n, 2 * np.pi, 2 * np.pi)
    p = melvin.Parameters({"nx": n, "nz": n, "lx": 2 * np.pi, "lz": 2 * np.pi, "final_time": 1.0,
                           "initial_dt": dt, "precision": "split", "device": "cuda:0"})
    ens = Ensemble(p, [FieldSpec(1e-4), FieldSpec(1e-4)], members)
    deltas = np.random.default_rng(0).uniform(0.02, 0.1, size=members)
    ics = [workloads.kelvin_helmholtz(n, n, deltas[b], seed=b) for b in range(members)]
    for b, (w, c) in enumerate(ics):
        ens.load_physical(b, [w, c])
    ens.step(dt)
    replay = ens.graph(dt, graph_steps)
    for _ in range((nsteps - 1) // graph_steps):
        replay()
    for _ in range((nsteps - 1) % graph_steps):
        ens.step(dt)
    torch.cuda.synchronize()
    for b in (int(np.argmin(deltas)), int(np.argmax(deltas))):
        w0, c0 = ics[b]
        ref = P.Problem(g, P.kh_specs(1e-4, 1e-4), [O.to_spectral(g, w0), O.to_spectral(g, c0)], dt)
        for _ in range(nsteps):
            ref.step()
        for f in range(2):
            err = rel_l2(ens.q[b, f].cpu().numpy(), ref.q[f])
            assert err < SPLIT_TOL, (b, deltas[b], f, err)
