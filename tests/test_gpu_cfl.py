"""Integrator.set_dt (melvin/Integrator.py:35-44) on the GPU against the
reference's own outcomes (golden vectors from tests/golden/make_golden.py).

The reference's CFL limit is min(dx/max(ux), dz/max(uz)) with the SIGNED
maximum and Python's builtin min, so:
  * a velocity whose signed maximum is far below its absolute maximum gets a
    much larger limit (an absolute maximum would breach these cases);
  * an all-negative ux gives a negative limit, which always breaches;
  * a NaN in ux is caught (min keeps a NaN first argument), a NaN in uz
    alone is not (min drops a NaN second argument).
Every outcome -- the dt left after the 0.9 shrink loop, or the breach -- must
be identical: the maxima are exact reductions, and the shrink loop repeats
the reference's multiplications, so dts are compared bit for bit.
Three paths are checked: the device maxima of mgb_diagnostics, the host
Integrator.set_dt on arbitrary velocities, and the CFL check of a whole
loop iteration (velocity from vorticity, step, end_loop) both on the host
loop and on the device-driven loop (melvin.driver.DeviceRun)."""

import numpy as np
import pytest
import torch

from cases import CFL_E2E_GRIDS, CFL_GRIDS, params_dict

pytestmark = pytest.mark.gpu


def _sim(g, dt=1e-3, cfl_cadence=10, final_time=1.0):
    import melvin
    from melvin import BasisFunctions as B

    d = params_dict(g, "explicit" if g.fdm_z else "semi-implicit", 2, dt)
    d.update(final_time=final_time, cfl_cadence=cfl_cadence)
    sim = melvin.Simulation(melvin.Parameters(d), torch)
    bf = [B.COMPLEX_EXP, B.FDM if g.fdm_z else B.COMPLEX_EXP]
    return sim, bf


def _outcome(fn):
    try:
        return fn()
    except Exception as e:
        assert str(e) == "CFL condition breached", e
        return np.nan


@pytest.mark.parametrize("tag", list(CFL_GRIDS))
def test_device_maxima_match_reference(cuda, golden, tag):
    sim, bf = _sim(CFL_GRIDS[tag])
    for s in golden[f"{tag}/sets"]:
        d = sim._integrator.diagnostics(golden[f"{tag}/{s}/ux"], golden[f"{tag}/{s}/uz"]).cpu().numpy()
        np.testing.assert_array_equal(d[1:3], golden[f"{tag}/{s}/max"], err_msg=str(s))


@pytest.mark.parametrize("tag", list(CFL_GRIDS))
def test_set_dt_matches_reference(cuda, golden, tag):
    sim, bf = _sim(CFL_GRIDS[tag])
    integ = sim._integrator
    ux, uz = sim.make_variable("ux", bf), sim.make_variable("uz", bf)
    for s in golden[f"{tag}/sets"]:
        ux.setp(golden[f"{tag}/{s}/ux"])
        uz.setp(golden[f"{tag}/{s}/uz"])
        got = []
        for dt in golden[f"{tag}/{s}/dts"]:
            integ.override_dt(float(dt))
            got.append(_outcome(lambda: (integ.set_dt(ux, uz), integ.get_dt())[1]))
        np.testing.assert_array_equal(got, golden[f"{tag}/{s}/dt_out"], err_msg=str(s))


def _iteration(g, w0, dt, device_loop):
    """One loop iteration from vorticity w0 at initial dt with the CFL ticker
    on; returns the dt after end_loop (NaN on a breach)."""
    from melvin import equations
    from melvin.driver import DeviceRun
    from melvin.utility import calc_velocity_from_vorticity

    sim, bf = _sim(g, dt=float(dt), final_time=1e6)
    V = {k: sim.make_variable(k, bf) for k in ("w", "psi", "ux", "uz", "tmp")}
    dw, dtmp = sim.make_derivative("dw"), sim.make_derivative("dtmp")
    sim.init_laplacian_solver(bf)
    V["w"].load(w0, is_physical=True)
    sim.config_cfl(V["ux"], V["uz"])
    if g.fdm_z:
        step = equations.rayleigh_benard(sim, V["w"], dw, V["tmp"], dtmp, 1.0, 1e3)
    else:
        step = equations.vorticity(sim, V["w"], dw, 1e-2)

    def host():
        calc_velocity_from_vorticity(V["w"], V["psi"], V["ux"], V["uz"], sim.get_laplacian_solver())
        step.step()
        sim.end_loop()
        return sim._integrator.get_dt()

    def device():
        assert DeviceRun(sim, step).run(max_steps=1) == 1
        return sim._integrator.get_dt()

    return _outcome(device if device_loop else host)


@pytest.mark.parametrize("device_loop", [False, True])
@pytest.mark.parametrize("tag", list(CFL_E2E_GRIDS))
def test_loop_iteration_cfl_matches_reference(cuda, golden, tag, device_loop):
    g = CFL_E2E_GRIDS[tag]
    got = [_iteration(g, golden[f"{tag}/init_w"], dt, device_loop) for dt in golden[f"{tag}/dts"]]
    np.testing.assert_array_equal(got, golden[f"{tag}/dt_out"])
    # the jet's signed maximum is far below its absolute maximum: an
    # absolute-value CFL would breach every ratio from 0.3 on
    if tag == "cfl_e2e_fs32":
        assert golden[f"{tag}/max"][0] < 0.25 * np.abs(golden[f"{tag}/ux"]).max()
