"""Checkpoint and host I/O of the Simulation / Variable API.

* Simulation.dump / load (melvin/Simulation.py:155-197): a run that stops,
  is loaded from one of its dumps into a fresh Simulation and continues
  ends bit-identical to the run that never stopped (state, history slot
  index, t, dt, loop counter).  The reference's load cannot read its own
  dumps (the pickled params need allow_pickle); these dumps are pickle-free.
* Variable.load of a spectral array of another resolution
  (melvin/Variable.py:67-85,142-151) keeps the overlapping low modes:
  against the reference's own output where its resampling works (a real
  spectrum from a finer grid), and against that rule for complex spectra in
  both directions (the reference resamples into a real array).
* Variable.save (melvin/Variable.py:130-133) writes the physical field to
  ``<name><counter:04d>.npy``.
"""

import numpy as np
import pytest
import torch

import oracle as O
from oracle import problems as P

pytestmark = pytest.mark.gpu


def _tg(n=32, final_time=0.2, dt=0.01, dump_cadence=0.05):
    import melvin
    from melvin import BasisFunctions as B, equations

    p = melvin.Parameters({"nx": n, "nz": n, "lx": 2 * np.pi, "lz": 2 * np.pi, "final_time": final_time,
                           "initial_dt": dt, "dump_cadence": dump_cadence, "device": "cuda:0"})
    sim = melvin.Simulation(p, torch)
    bf = [B.COMPLEX_EXP, B.COMPLEX_EXP]
    V = {k: sim.make_variable(k, bf) for k in ("w", "psi", "ux", "uz")}
    dw = sim.make_derivative("dw")
    sim.init_laplacian_solver(bf)
    sim.config_dump([V["w"]], [dw])
    return sim, V, dw, equations.vorticity(sim, V["w"], dw, 1e-2)


def _loop(sim, V, step, stop_loop=None):
    from melvin.utility import calc_velocity_from_vorticity

    while sim.is_running() and (stop_loop is None or sim._loop_counter < stop_loop):
        calc_velocity_from_vorticity(V["w"], V["psi"], V["ux"], V["uz"], sim.get_laplacian_solver())
        step.step()
        sim.end_loop()


def test_dump_load_continue_is_bit_identical(cuda, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    g = O.Grid(32, 32, 2 * np.pi, 2 * np.pi)
    w0 = P.taylor_green_ic(g, seed=4)
    sim, V, dw, step = _tg()
    V["w"].load(w0, is_physical=True)
    _loop(sim, V, step)
    final = (V["w"].gets().cpu().numpy(), dw.get_all().cpu().numpy(), dw.get_curr_idx(), sim._t,
             sim._integrator._dt, sim._loop_counter)
    assert (tmp_path / "dump0002.npz").exists()
    with np.load(tmp_path / "dump0002.npz", allow_pickle=False) as d:
        stop = int(d["loop_counter"])
    assert 0 < stop < final[5]

    # a fresh simulation resumes from the third dump
    sim2, V2, dw2, step2 = _tg()
    sim2.load(2)
    assert sim2._loop_counter == stop
    _loop(sim2, V2, step2)
    got = (V2["w"].gets().cpu().numpy(), dw2.get_all().cpu().numpy(), dw2.get_curr_idx(), sim2._t,
           sim2._integrator._dt, sim2._loop_counter)
    assert np.array_equal(got[0], final[0])
    assert np.array_equal(got[1], final[1])
    assert got[2:] == final[2:]


def test_load_resamples_like_the_reference(cuda, golden):
    import melvin
    from melvin import BasisFunctions as B

    p = melvin.Parameters({"nx": 32, "nz": 32, "lx": 2 * np.pi, "lz": 2 * np.pi, "final_time": 1.0,
                           "device": "cuda:0"})
    sim = melvin.Simulation(p, torch)
    v = sim.make_variable("v", [B.COMPLEX_EXP, B.COMPLEX_EXP])
    v.load(golden["load_resample/in_spec"], is_physical=False)
    assert np.array_equal(v.gets().cpu().numpy(), golden["load_resample/out_spec"])


def _modes(a):
    """{(n, m): value} of a fully spectral array (rows 0..nn, -nn..-1)."""
    rows, cols = a.shape
    nn = (rows - 1) // 2
    return {(r if r <= nn else r - rows, m): a[r, m] for r in range(rows) for m in range(cols)}


@pytest.mark.parametrize("n_from,n_to", [(64, 32), (32, 64), (64, 64)])
def test_load_resample_keeps_complex_low_modes(cuda, n_from, n_to):
    import melvin
    from melvin import BasisFunctions as B

    def par(n):
        return melvin.Parameters({"nx": n, "nz": n, "lx": 2 * np.pi, "lz": 2 * np.pi, "final_time": 1.0,
                                  "device": "cuda:0"})

    src = par(n_from)
    rng = np.random.default_rng(n_from * 100 + n_to)
    a = rng.standard_normal(src.spectral_shape) + 1j * rng.standard_normal(src.spectral_shape)
    sim = melvin.Simulation(par(n_to), torch)
    v = sim.make_variable("v", [B.COMPLEX_EXP, B.COMPLEX_EXP])
    v.load(a, is_physical=False)
    got = _modes(v.gets().cpu().numpy())
    have = _modes(a)
    for k, val in got.items():
        assert val == have.get(k, 0.0), k


def test_variable_save_writes_the_physical_field(cuda, tmp_path, monkeypatch):
    import melvin
    from melvin import BasisFunctions as B

    monkeypatch.chdir(tmp_path)
    p = melvin.Parameters({"nx": 32, "nz": 16, "lx": 2.0, "lz": 1.0, "final_time": 1.0, "device": "cuda:0"})
    sim = melvin.Simulation(p, torch)
    v = sim.make_variable("temp", [B.COMPLEX_EXP, B.COMPLEX_EXP])
    field = np.random.default_rng(5).standard_normal((32, 16))
    v.setp(field)
    v.save(7)
    assert np.array_equal(np.load(tmp_path / "temp0007.npy"), field)
