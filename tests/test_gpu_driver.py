"""The device-driven Simulation loop (melvin.driver.DeviceRun) against the
Simulation's own host loop, which runs the reference's tickers: the CFL
check Integrator.set_dt on per-verb velocities every cfl_cadence loops, the
kinetic-energy tracker every tracker_cadence loops, time-based dumps, and
the stop at final_time.

Both runs use the same fused step, so the states must be bit-identical and
t, dt, the loop counter and the ticker counters equal; the kinetic-energy
samples come from the fused step's own reduction on the device and from a
separate per-verb velocity on the host, so they agree to 1e-12.
"""

import functools

import numpy as np
import pytest
import torch

import oracle as O
from oracle import problems as P

pytestmark = pytest.mark.gpu


def make_tg(n=64, dt=0.06, final_time=3.0, cfl_cadence=10, tracker_cadence=5, dump_cadence=None, nu=1e-2,
            precision="double"):
    import melvin
    from melvin import BasisFunctions as B, equations
    from melvin.utility import calc_kinetic_energy

    prm = {"nx": n, "nz": n, "lx": 2 * np.pi, "lz": 2 * np.pi, "final_time": final_time, "initial_dt": dt,
           "cfl_cadence": cfl_cadence, "tracker_cadence": tracker_cadence, "precision": precision,
           "device": "cuda:0"}
    if dump_cadence is not None:
        prm["dump_cadence"] = dump_cadence
    p = melvin.Parameters(prm)
    sim = melvin.Simulation(p, torch)
    bf = [B.COMPLEX_EXP, B.COMPLEX_EXP]
    V = {k: sim.make_variable(k, bf) for k in ("w", "psi", "ux", "uz")}
    dw = sim.make_derivative("dw")
    sim.init_laplacian_solver(bf)
    g = O.Grid(n, n, 2 * np.pi, 2 * np.pi)
    V["w"].load(P.taylor_green_ic(g, seed=3), is_physical=True)
    if dump_cadence is not None:
        sim.config_dump([V["w"]], [dw])
    sim.config_cfl(V["ux"], V["uz"])
    sim.config_scalar_trackers({"kinetic_energy": functools.partial(calc_kinetic_energy, V["ux"], V["uz"], torch, p)})
    step = equations.vorticity(sim, V["w"], dw, nu)
    return sim, step, V, dw


def make_rbc(nx=32, nz=17, dt=1e-5, final_time=2e-4, precision="double", integrator="explicit", order=2):
    import melvin
    from melvin import BasisFunctions as B, equations, workloads
    from melvin.utility import calc_kinetic_energy

    p = melvin.Parameters({"nx": nx, "nz": nz, "lx": 2.0, "lz": 1.0, "final_time": final_time, "initial_dt": dt,
                           "discretisation": ["spectral", "fdm"], "integrator": "explicit",
                           "integrator_order": order, "spatial_derivative_order": order, "cfl_cadence": 3,
                           "tracker_cadence": 2, "precision": precision, "device": "cuda:0"})
    sim = melvin.Simulation(p, torch)
    bf = [B.COMPLEX_EXP, B.FDM]
    V = {k: sim.make_variable(k, bf) for k in ("w", "psi", "ux", "uz", "tmp")}
    dw, dt_ = sim.make_derivative("dw"), sim.make_derivative("dtmp")
    sim.init_laplacian_solver(bf)
    V["tmp"].load(workloads.conductive(nx, nz, 2.0, 1.0, seed=5), is_physical=True)
    # a convection roll, so that max(ux) > 0 from the start (the reference's
    # CFL check takes the signed maximum, which breaches for a field at rest)
    X, Z = np.meshgrid(np.linspace(0, 2.0, nx, endpoint=False), np.linspace(0, 1.0, nz), indexing="ij")
    V["w"].load(50.0 * np.sin(np.pi * X) * np.sin(np.pi * Z), is_physical=True)
    sim.config_cfl(V["ux"], V["uz"])
    sim.config_scalar_trackers({"kinetic_energy": functools.partial(calc_kinetic_energy, V["ux"], V["uz"], torch, p)})
    step = equations.rayleigh_benard(sim, V["w"], dw, V["tmp"], dt_, 1.0, 1e5, integrator=integrator)
    return sim, step, V, dw


def host_loop(sim, step, V, max_steps=None):
    """The reference's loop with the fused body: velocities for the tickers
    from the per-verb path, then the step, then end_loop."""
    from melvin.utility import calc_velocity_from_vorticity

    solver = sim.get_laplacian_solver()
    n = 0
    while sim.is_running() and (max_steps is None or n < max_steps):
        calc_velocity_from_vorticity(V["w"], V["psi"], V["ux"], V["uz"], solver)
        step.step()
        sim.end_loop()
        n += 1
    return n


def compare(a, b, fields, ke_rtol=1e-12):
    sa, sb = a[0], b[0]
    assert sa._loop_counter == sb._loop_counter
    assert sa._t == sb._t
    assert sa._integrator._dt == sb._integrator._dt
    assert sa._cfl_ticker._counter == sb._cfl_ticker._counter
    assert sa._cfl_ticker.times_fired == sb._cfl_ticker.times_fired
    ta, tb = sa._trackers[0], sb._trackers[0]
    assert ta._times == tb._times
    np.testing.assert_allclose(np.array(tb._values, dtype=float), np.array(ta._values, dtype=float), rtol=ke_rtol)
    for k in fields:
        assert torch.equal(a[2][k]._sdata, b[2][k]._sdata), k
    assert a[3]._curr_idx == b[3]._curr_idx


def test_device_run_matches_host_loop_with_cfl_shrinks(cuda):
    from melvin.driver import DeviceRun

    a = make_tg()
    b = make_tg()
    na = host_loop(a[0], a[1], a[2])
    nb = DeviceRun(b[0], b[1], horizon=7).run(chunk=16)
    assert na == nb > 40
    assert a[0]._integrator._dt < 0.06  # the CFL check shrank dt
    compare(a, b, ["w"])


def test_device_run_in_pieces_equals_one_run(cuda):
    from melvin.driver import DeviceRun

    a = make_tg(final_time=1.5)
    b = make_tg(final_time=1.5)
    host_loop(a[0], a[1], a[2])
    run = DeviceRun(b[0], b[1])
    total = 0
    for m in (3, 1, 7, 50):
        total += run.run(max_steps=m, chunk=4)
    total += run.run()
    assert total == a[0]._loop_counter
    compare(a, b, ["w"])


def test_cfl_breach_raises_at_the_same_iteration(cuda):
    from melvin.driver import DeviceRun

    a = make_tg(dt=0.2)
    b = make_tg(dt=0.2)
    with pytest.raises(Exception, match="CFL condition breached"):
        host_loop(a[0], a[1], a[2])
    with pytest.raises(Exception, match="CFL condition breached"):
        DeviceRun(b[0], b[1]).run(chunk=8)
    assert a[0]._loop_counter == b[0]._loop_counter == 1
    assert a[0]._t == b[0]._t
    assert torch.equal(a[2]["w"]._sdata, b[2]["w"]._sdata)


def test_dumps_fire_at_the_host_loop_times(cuda, tmp_path, monkeypatch):
    from melvin.driver import DeviceRun

    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    monkeypatch.chdir(tmp_path / "a")
    a = make_tg(final_time=1.2, dump_cadence=0.25)
    host_loop(a[0], a[1], a[2])
    monkeypatch.chdir(tmp_path / "b")
    b = make_tg(final_time=1.2, dump_cadence=0.25)
    DeviceRun(b[0], b[1]).run(chunk=32)
    fa = sorted(p.name for p in (tmp_path / "a").iterdir())
    fb = sorted(p.name for p in (tmp_path / "b").iterdir())
    assert fa == fb and len(fa) >= 4
    for name in fa:
        da, db = np.load(tmp_path / "a" / name), np.load(tmp_path / "b" / name)
        for k in ("t", "loop_counter", "curr_idx", "w", "dw"):
            np.testing.assert_array_equal(da[k], db[k], err_msg=f"{name}:{k}")
    compare(a, b, ["w"])


@pytest.mark.parametrize("integrator,order", [("explicit", 2), ("pece", 4)])
def test_device_run_dirichlet_grid(cuda, integrator, order):
    from melvin.driver import DeviceRun

    a = make_rbc(integrator=integrator, order=order)
    b = make_rbc(integrator=integrator, order=order)
    na = host_loop(a[0], a[1], a[2])
    nb = DeviceRun(b[0], b[1], horizon=5).run(chunk=6)
    assert na == nb >= 20
    compare(a, b, ["w", "tmp"])


def test_device_run_split_precision(cuda):
    from melvin.driver import DeviceRun

    a = make_tg(n=128, dt=0.03, precision="split", final_time=1.0)
    b = make_tg(n=128, dt=0.03, precision="split", final_time=1.0)
    host_loop(a[0], a[1], a[2])
    DeviceRun(b[0], b[1]).run()
    # the fused step's velocity is FP32 here, the host tickers' per-verb one FP64
    compare(a, b, ["w"], ke_rtol=1e-5)


# ---- the Nusselt tracker (examples/double_diffusive_convection.py:20-23, 80-89) ----


def _ddc_sim(n=64, dt=None, final_time=None, precision="double", fdm=False):
    """Fully spectral double-diffusive convection (the example's equations
    and trackers), or Rayleigh-Benard on the Dirichlet grid; both with the
    kinetic-energy and Nusselt trackers and the CFL check."""
    import melvin
    from melvin import BasisFunctions as B, equations, workloads
    from melvin.utility import calc_kinetic_energy, calc_nusselt_number

    nz = n // 2 + 1 if fdm else n
    # 250 steps; the Dirichlet grid's explicit diffusion needs dt below ~1.2e-4 at 64x33
    dt = dt if dt is not None else (2e-5 if fdm else 2e-4)
    final_time = final_time if final_time is not None else 250 * dt
    lx, lz = (2.0, 1.0) if fdm else (4.0, 2.0)
    prm = {"nx": n, "nz": nz, "lx": lx, "lz": lz, "final_time": final_time, "initial_dt": dt, "cfl_cadence": 4,
           "tracker_cadence": 3, "precision": precision, "device": "cuda:0"}
    if fdm:
        prm.update({"discretisation": ["spectral", "fdm"], "integrator": "explicit"})
    p = melvin.Parameters(prm)
    sim = melvin.Simulation(p, torch)
    bf = [B.COMPLEX_EXP, B.FDM if fdm else B.COMPLEX_EXP]
    names = ("w", "psi", "ux", "uz", "tmp") + (() if fdm else ("xi",))
    V = {k: sim.make_variable(k, bf) for k in names}
    D = {k: sim.make_derivative("d" + k) for k in ("w", "tmp", "xi")}
    sim.init_laplacian_solver(bf)
    g = O.Grid(n, nz, lx, lz, fdm)
    X, Z = np.meshgrid(np.arange(n) * lx / n, np.arange(nz) * lz / (nz - 1 if fdm else nz), indexing="ij")
    if fdm:
        V["tmp"].load(workloads.conductive(n, nz, lx, lz, seed=2), is_physical=True)
        V["w"].load(40.0 * np.sin(np.pi * X) * np.sin(np.pi * Z), is_physical=True)
        step = equations.rayleigh_benard(sim, V["w"], D["w"], V["tmp"], D["tmp"], 1.0, 1e4)
    else:
        rng = np.random.default_rng(5)
        V["w"].load(3.0 * np.sin(2 * np.pi * X / lx) * np.cos(2 * np.pi * Z / lz) + 0.1 * rng.standard_normal((n, nz)),
                    is_physical=True)
        V["tmp"].load(np.cos(2 * np.pi * X / lx) * np.sin(2 * np.pi * Z / lz) + 0.05 * rng.standard_normal((n, nz)),
                      is_physical=True)
        V["xi"].load(0.5 * np.sin(4 * np.pi * Z / lz) + 0.05 * rng.standard_normal((n, nz)), is_physical=True)
        step = equations.double_diffusive_spectral(sim, V["w"], D["w"], V["tmp"], D["tmp"], V["xi"], D["xi"],
                                                   7.0, 1.1, 1.0 / 3.0)
    sim.config_cfl(V["ux"], V["uz"])
    sim.config_scalar_trackers({
        "kinetic_energy.npz": functools.partial(calc_kinetic_energy, V["ux"], V["uz"], torch, p),
        "nusselt_number.npz": functools.partial(calc_nusselt_number, V["tmp"], V["uz"], torch, p),
    })
    return sim, step, V, D["w"], g


def _host_loop_with_tmp(sim, step, V):
    """host_loop, with the temperature's physical field refreshed at the start
    of each iteration (the example's loop body does it through
    tmp.vec_dot_nabla)."""
    from melvin.utility import calc_velocity_from_vorticity

    solver = sim.get_laplacian_solver()
    n = 0
    while sim.is_running():
        calc_velocity_from_vorticity(V["w"], V["psi"], V["ux"], V["uz"], solver)
        V["tmp"].to_physical()
        step.step()
        sim.end_loop()
        n += 1
    return n


@pytest.mark.parametrize("fdm,precision,tol", [(False, "double", 1e-12), (True, "double", 1e-12),
                                               (False, "split", 2e-6)])
def test_step_flux_diagnostic_vs_oracle(cuda, fdm, precision, tol):
    """diag[3] = mean(tmp * uz) of the start-of-step fields against the
    oracle's physical temperature and velocity, within `tol` times
    mean(|tmp * uz|) (the mean itself may cancel)."""
    sim, step, V, dw, g = _ddc_sim(precision=precision, fdm=fdm)
    w_s, t_s = V["w"].gets().cpu().numpy(), V["tmp"].gets().cpu().numpy()
    vel = O.velocity_from_vorticity(g, O.PoissonSolver(g), w_s)
    prod = O.to_physical(g, t_s) * vel["uz_p"]
    want, scale = float(np.mean(prod)), float(np.mean(np.abs(prod)))
    want_ke = O.kinetic_energy(g, vel["ux_p"], vel["uz_p"])
    step.set_flux_field(V["tmp"])
    d = step.step(diagnostics=True).cpu().numpy()
    assert abs(d[3] - want) <= tol * scale, (d[3], want, scale)
    assert abs(d[0] - want_ke) <= tol * abs(want_ke)
    step.set_flux_field(None)
    assert step.step(diagnostics=True)[3].item() == 0.0


@pytest.mark.parametrize("fdm", [False, True])
def test_device_run_nusselt_tracker(cuda, fdm):
    from melvin.driver import DeviceRun

    a = _ddc_sim(fdm=fdm)
    b = _ddc_sim(fdm=fdm)
    na = _host_loop_with_tmp(a[0], a[1], a[2])
    nb = DeviceRun(b[0], b[1], horizon=9).run(chunk=16)
    assert na == nb > 100
    sa, sb = a[0], b[0]
    assert sa._loop_counter == sb._loop_counter and sa._t == sb._t
    assert sa._integrator._dt == sb._integrator._dt
    for ta, tb in zip(sa._trackers, sb._trackers):
        assert ta._times == tb._times and len(ta._times) > 30
        np.testing.assert_allclose(np.array(tb._values, dtype=float), np.array(ta._values, dtype=float),
                                   rtol=1e-12, atol=1e-14)
    nu = np.array(sb._trackers[1]._values, dtype=float)
    assert np.all(np.isfinite(nu)) and np.ptp(nu) > 0
    for k in ("w", "tmp"):
        assert torch.equal(a[2][k]._sdata, b[2][k]._sdata), k


def test_device_run_rejects_unknown_tracker(cuda):
    from melvin.driver import DeviceRun

    sim, step, V, dw, g = _ddc_sim()
    sim._trackers[0]._filename = "enstrophy.npz"
    sim._tracker_fns[0] = lambda: 0.0
    with pytest.raises(ValueError, match="only the kinetic energy and the Nusselt number"):
        DeviceRun(sim, step)
