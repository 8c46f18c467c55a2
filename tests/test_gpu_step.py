"""Timestepping parity: the fused step and the reference-style per-verb
loop against the reference trajectories (golden vectors) and the oracle.

Tolerances: FP64 paths 1e-12 relative L2 of every field after every step
(the parity bound of the FP64 path); the split-precision path (FP32
transforms, FP64 state) is checked against the FP64 oracle at 1e-5 after
the trajectory."""

import numpy as np
import pytest
import torch

import oracle as O
from oracle import problems as P
from cases import TRAJ_CASES, params_dict
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-12


def build(g, names, integ, order, dt, precision="double"):
    import melvin
    from melvin import BasisFunctions as B

    p = melvin.Parameters(params_dict(g, "explicit" if integ == "pece" else integ, order, dt, precision))
    sim = melvin.Simulation(p, torch)
    bf = [B.COMPLEX_EXP, B.FDM if g.fdm_z else B.COMPLEX_EXP]
    V = {n: sim.make_variable(n, bf) for n in names + ["psi", "ux", "uz"]}
    D = {n: sim.make_derivative("d" + n) for n in names}
    sim.init_laplacian_solver(bf)
    return sim, p, V, D, bf


def stepper_for(tag, sim, V, D, integ):
    from melvin import equations

    kw = {"integrator": integ}
    if tag.startswith("tg"):
        return equations.vorticity(sim, V["w"], D["w"], 1e-2, **kw)
    if tag.startswith("kh"):
        return equations.kelvin_helmholtz(sim, V["w"], D["w"], V["c"], D["c"], 1e-3, 2e-3, **kw)
    if tag.startswith("ddcs"):
        return equations.double_diffusive_spectral(sim, V["w"], D["w"], V["tmp"], D["tmp"], V["xi"], D["xi"],
                                                   7.0, 1.1, 1.0 / 3.0, **kw)
    if tag.startswith("rbc"):
        return equations.rayleigh_benard(sim, V["w"], D["w"], V["tmp"], D["tmp"], 1.0, 1e5, **kw)
    if tag.startswith("ddcd"):
        return equations.double_diffusive_dirichlet(sim, V["w"], D["w"], V["T"], D["T"], V["S"], D["S"],
                                                    7.0, 1e5, 2.0, 10.0, **kw)
    raise KeyError(tag)


@pytest.mark.parametrize("precision", ["double", "dfloat"])
@pytest.mark.parametrize("tag", list(TRAJ_CASES))
def test_fused_step_matches_reference_trajectory(cuda, golden, tag, precision):
    """FP64 and double-float transforms both hold the 1e-12 per-step bound."""
    g, specs, names, integ, order, dt = TRAJ_CASES[tag]
    sim, p, V, D, bf = build(g, names, integ, order, dt, precision)
    for n in names:
        V[n].sets(golden[f"{tag}/s0_{n}"])
    step = stepper_for(tag, sim, V, D, integ)
    kes = []
    for s in range(int(golden[f"{tag}/nsteps"])):
        diag = step.step(diagnostics=True)
        kes.append(float(diag[0].item()))
        for n in names:
            err = rel_l2(V[n].gets().cpu().numpy(), golden[f"{tag}/s{s + 1}_{n}"])
            assert err < TOL, (s, n, err)
    assert rel_l2(np.array(kes), golden[f"{tag}/ke"]) < TOL


def _reference_loop_body(tag, sim, p, V, D, integ):
    """The example loop bodies written against this package's API."""
    from melvin.utility import calc_velocity_from_vorticity

    solver = sim.get_laplacian_solver()
    integ_ = sim._integrator
    calc_velocity_from_vorticity(V["w"], V["psi"], V["ux"], V["uz"], solver)
    ux, uz = V["ux"].getp(), V["uz"].getp()
    if tag.startswith("tg"):
        w = V["w"]
        D["w"][:] = -w.vec_dot_nabla(ux, uz)
        integ_.integrate(w, D["w"], 1e-2 * w.lap())
    elif tag.startswith("kh"):
        for n, k in (("w", 1e-3), ("c", 2e-3)):
            D[n][:] = -V[n].vec_dot_nabla(ux, uz)
            integ_.integrate(V[n], D[n], k * V[n].lap())
    elif tag.startswith("ddcs"):
        w, tmp, xi = V["w"], V["tmp"], V["xi"]
        lin = 7.0 * w.lap()
        D["w"][:] = -w.vec_dot_nabla(ux, uz) + 7.0 * xi.sddx() - 7.0 * tmp.sddx()
        integ_.integrate(w, D["w"], lin)
        D["tmp"][:] = -tmp.vec_dot_nabla(ux, uz) - V["uz"][:]
        integ_.integrate(tmp, D["tmp"], tmp.lap())
        D["xi"][:] = -xi.vec_dot_nabla(ux, uz) - V["uz"][:] / 1.1
        integ_.integrate(xi, D["xi"], (1.0 / 3.0) * xi.lap())
        tmp[:, 0] = 0.0
        xi[:, 0] = 0.0
    elif tag.startswith("rbc") and integ == "explicit":
        w, tmp = V["w"], V["tmp"]
        diff = 1.0 * w.snabla2()
        D["w"][:] = -w.vec_dot_nabla(ux, uz) - 1.0 * 1e5 * tmp.sddx()
        integ_.integrate(w, D["w"], diff)
        diff = tmp.snabla2()
        D["tmp"][:] = -tmp.vec_dot_nabla(ux, uz)
        integ_.integrate(tmp, D["tmp"], diff)
        e = p.spatial_derivative_order // 2
        w[1:, :e] = 0.0
        w[1:, -e:] = 0.0
        tmp[0, :e] = 1.0
        tmp[0, -e:] = 0.0
        tmp[1:, :e] = 0.0
        tmp[1:, -e:] = 0.0
        w[0, :] = 0.0
    else:
        pytest.skip("no per-verb form written for this case")


@pytest.mark.parametrize("tag", ["tg32_o2_ab2", "tg32_o4_ab4", "kh64x32", "ddcs32", "rbc32x17_o4_ab4",
                                 "rbc32x17_o2_ab2"])
def test_per_verb_loop_matches_reference_trajectory(cuda, golden, tag):
    g, specs, names, integ, order, dt = TRAJ_CASES[tag]
    sim, p, V, D, bf = build(g, names, integ, order, dt)
    for n in names:
        V[n].load(golden[f"{tag}/init_{n}"], is_physical=True)
        assert rel_l2(V[n].gets().cpu().numpy(), golden[f"{tag}/s0_{n}"]) < TOL
    for s in range(int(golden[f"{tag}/nsteps"])):
        _reference_loop_body(tag, sim, p, V, D, integ)
        for n in names:
            err = rel_l2(V[n].gets().cpu().numpy(), golden[f"{tag}/s{s + 1}_{n}"])
            assert err < TOL, (s, n, err)


def test_taylor_green_256_matches_oracle(cuda):
    """Config-1 grid (256^2, nu=1e-2, dt=1e-3, AB2 semi-implicit): per-step
    relative L2 against the oracle for the first 20 steps."""
    import melvin
    from melvin import BasisFunctions as B, equations

    g = O.Grid(256, 256, 2 * np.pi, 2 * np.pi)
    p = melvin.Parameters(params_dict(g, dt=1e-3))
    sim = melvin.Simulation(p, torch)
    bf = [B.COMPLEX_EXP, B.COMPLEX_EXP]
    w, dw = sim.make_variable("w", bf), sim.make_derivative("dw")
    w0 = P.taylor_green_ic(g, seed=0)
    w.load(w0, is_physical=True)
    ref = P.Problem(g, P.vorticity_specs(1e-2), [O.to_spectral(g, w0)], 1e-3)
    step = equations.vorticity(sim, w, dw, 1e-2)
    for s in range(20):
        # restart the GPU from the oracle state each step: per-step error
        w.sets(ref.q[0])
        dw._data.copy_(torch.as_tensor(ref.h[0].data, device=cuda))
        dw.set_curr_idx(ref.h[0].curr)
        step.step()
        ref.step()
        assert rel_l2(w.gets().cpu().numpy(), ref.q[0]) < TOL, s


@pytest.mark.parametrize("tag", ["tg32_o2_ab2", "kh64x32", "rbc32x17_o4_ab4", "rbc32x17_pece4", "ddcd32x17"])
def test_split_precision_close_to_fp64(cuda, golden, tag):
    g, specs, names, integ, order, dt = TRAJ_CASES[tag]
    sim, p, V, D, bf = build(g, names, integ, order, dt, precision="split")
    for n in names:
        V[n].sets(golden[f"{tag}/s0_{n}"])
    step = stepper_for(tag, sim, V, D, integ)
    nsteps = int(golden[f"{tag}/nsteps"])
    for _ in range(nsteps):
        step.step()
    for n in names:
        err = rel_l2(V[n].gets().cpu().numpy(), golden[f"{tag}/s{nsteps}_{n}"])
        assert err < 1e-5, (n, err)


@pytest.mark.parametrize(
    "nx,nz,fdm,precision,integ,order,tol",
    [(2048, 2048, False, "double", "semi-implicit", 2, TOL),
     (2048, 2048, False, "dfloat", "semi-implicit", 2, TOL),
     (2048, 2048, False, "split", "semi-implicit", 2, 1e-5),
     (256, 4096, False, "dfloat", "semi-implicit", 2, TOL),
     (1024, 513, True, "dfloat", "pece", 4, TOL),
     (4096, 256, False, "double", "semi-implicit", 4, TOL),
     (1024, 513, True, "double", "pece", 4, TOL),
     (1024, 513, True, "split", "pece", 4, 1e-5),
     (1024, 1025, True, "split", "explicit", 2, 1e-5)],
)
def test_fused_step_large_grids(cuda, nx, nz, fdm, precision, integ, order, tol):
    """One fused step at the benchmark grid sizes against the oracle
    (shared-memory footprints, grid shapes and tile edges of the big
    configurations)."""
    import melvin
    from melvin import BasisFunctions as B, equations, workloads

    lx, lz = (2 * np.pi, 2 * np.pi) if not fdm else (2.0, 1.0)
    sdo = 4 if order == 4 else 2
    g = O.Grid(nx, nz, lx, lz, fdm, sdo)
    p = melvin.Parameters(params_dict(g, "explicit" if integ == "pece" else integ, order, 1e-7 if fdm else 2e-4,
                                      precision))
    sim = melvin.Simulation(p, torch)
    bf = [B.COMPLEX_EXP, B.FDM if fdm else B.COMPLEX_EXP]
    if fdm:
        w, dw, t, dt_ = sim.make_variable("w", bf), sim.make_derivative("dw"), sim.make_variable("t", bf), \
            sim.make_derivative("dt")
        t0 = workloads.conductive(nx, nz, lx, lz, seed=3)
        t.load(t0, is_physical=True)
        step = equations.rayleigh_benard(sim, w, dw, t, dt_, 1.0, 1e7, integrator=integ)
        ref = P.Problem(g, P.rbc_specs(1.0, 1e7), [np.zeros(g.spectral_shape, complex), O.to_spectral(g, t0)],
                        1e-7, integ, order)
        for _ in range(2):
            step.step()
            ref.step()
        assert rel_l2(w.gets().cpu().numpy(), ref.q[0]) < tol
        assert rel_l2(t.gets().cpu().numpy(), ref.q[1]) < tol
    else:
        w, dw = sim.make_variable("w", bf), sim.make_derivative("dw")
        w0 = workloads.decaying_turbulence(nx, nz, seed=1)
        w.load(w0, is_physical=True)
        step = equations.vorticity(sim, w, dw, 5e-5)
        ref = P.Problem(g, P.vorticity_specs(5e-5), [O.to_spectral(g, w0)], 2e-4, "semi-implicit", order)
        for _ in range(2):
            step.step()
            ref.step()
        assert rel_l2(w.gets().cpu().numpy(), ref.q[0]) < tol


@pytest.mark.parametrize("tag", ["tg32_o2_ab2", "tg32_o4_ab4", "kh64x32"])
def test_step_host_matches_device_step(cuda, golden, tag):
    """Stepper.step_host (state and history in pinned host memory, only the
    read history slots uploaded, on a second stream that the update waits
    for) leaves the host tensors bit-identical to the device-resident step,
    history included, over steps that cycle through every history slot."""
    g, specs, names, integ, order, dt = TRAJ_CASES[tag]
    runs = []
    for _ in range(2):
        sim, p, V, D, bf = build(g, names, integ, order, dt)
        for n in names:
            V[n].sets(golden[f"{tag}/s0_{n}"])
        runs.append((V, D, stepper_for(tag, sim, V, D, integ)))
    (Va, Da, sa), (Vb, Db, sb) = runs
    hs = [Vb[n]._sdata.cpu().pin_memory() for n in names]
    hh = [Db[n]._data.cpu().pin_memory() for n in names]
    for n in names:  # the device staging copies start stale: only the host tensors are the state
        Vb[n]._sdata.zero_()
        Db[n]._data.fill_(float("nan"))
    nsteps = 2 * order + 1
    for _ in range(nsteps):
        sa.step(dt)
        up, down = sb.step_host(hs, hh, dt)
    torch.cuda.synchronize()
    S = Va[names[0]]._sdata.numel() * 16
    assert up == len(names) * order * S and down == 2 * len(names) * S, (up, down)
    for i, n in enumerate(names):
        assert torch.equal(hs[i], Va[n]._sdata.cpu()), n
        assert torch.equal(hh[i], Da[n]._data.cpu()), n
        assert Db[n]._curr_idx == Da[n]._curr_idx
