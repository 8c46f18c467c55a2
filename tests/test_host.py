"""Host-side logic that needs no GPU: parameters and derived shapes, basis
factors, tickers, the derivative ring buffer, equation assembly rules."""

import numpy as np
import pytest
import torch

import oracle as O


def test_parameters_derived_shapes_match_reference_rules():
    from melvin import Parameters

    for nx, nz, disc in [(256, 256, ["spectral", "spectral"]), (1024, 513, ["spectral", "fdm"]),
                         (2048, 1024, ["spectral", "spectral"])]:
        p = Parameters({"nx": nx, "nz": nz, "lx": 2.0, "lz": 1.0, "final_time": 1.0, "discretisation": disc})
        g = O.Grid(nx, nz, 2.0, 1.0, disc[1] == "fdm")
        assert p.spectral_shape == g.spectral_shape
        assert p.physical_shape == (nx, nz)
        assert p.dx == g.dx and p.dz == g.dz
        assert p.initial_dt == 0.2 * min(p.dx, p.dz)
        assert p.dump_cadence == 0.1
        assert p.alpha == 0.51 and p.integrator_order == 2 and p.cfl_cutoff == 0.5


def test_parameters_validation_exits_on_missing_keys():
    from melvin import Parameters

    with pytest.raises(SystemExit):
        Parameters({"nx": 16})
    with pytest.raises(ValueError):
        Parameters({"nx": 16, "nz": 16, "lx": 1, "lz": 1, "final_time": 1, "precision": "half"})


def test_basis_factors():
    from melvin.BasisFunctions import BasisFunctions as B, calc_diff_factor, gen_diff2_factors

    assert calc_diff_factor(B.COMPLEX_EXP, 2.0) == 1j * np.pi
    assert calc_diff_factor(B.FDM, 2.0) == 0
    f2 = gen_diff2_factors(1.0)
    assert f2[B.COMPLEX_EXP] == -((2 * np.pi) ** 2) and f2[B.FDM] == 0


def test_ticker_fires_like_reference():
    from melvin import Ticker

    fired = []
    t = Ticker(3, lambda tk: fired.append(tk.times_fired), is_loop_counter=True)
    for loop in range(1, 11):
        t.tick(0.0, loop)
    # fires when counter < loop: at loops 1, 4, 7, 10
    assert fired == [0, 1, 2, 3]
    tt = Ticker(0.5, lambda tk: fired.append("t"), is_loop_counter=False)
    tt.tick(0.1, 1)
    tt.tick(0.6, 2)
    assert tt.times_fired == 2
    assert tt.dump() == {"counter": 1.0, "times_fired": 2}


def test_time_derivative_ring_buffer_on_host_memory():
    from melvin import Parameters, TimeDerivative

    p = Parameters({"nx": 16, "nz": 16, "lx": 1, "lz": 1, "final_time": 1, "integrator_order": 4,
                    "device": "cpu"})
    d = TimeDerivative(p, None)
    h = O.History(4, p.spectral_shape)
    rng = np.random.default_rng(0)
    for _ in range(6):
        v = rng.standard_normal(p.spectral_shape) + 0j
        d[:] = torch.as_tensor(v)
        h.set(v)
        for k in range(0, -4, -1):
            np.testing.assert_array_equal(d.get(k).numpy(), h.get(k))
        d.advance()
        h.advance()
    assert d.get_curr_idx() == h.curr


def test_term_validation():
    from melvin.stepper import Term

    with pytest.raises(ValueError):
        Term("psi", "d3dx3", 1.0)
    t = Term("psi", "ddx", -2)
    assert t.coef == -2.0


def test_parameters_save_round_trip(tmp_path):
    """Parameters.save (melvin/Parameters.py:94-96) writes the dictionary the
    parameters were built from as JSON; building from the file again gives
    the same derived values."""
    import json

    from melvin import Parameters

    d = {"nx": 1024, "nz": 513, "lx": 2.0, "lz": 1.0, "final_time": 0.5, "Ra": 1e7, "Pr": 1.0,
         "discretisation": ["spectral", "fdm"], "integrator": "explicit", "integrator_order": 4,
         "spatial_derivative_order": 4, "initial_dt": 1e-7}
    p = Parameters(d)
    fname = tmp_path / "params.json"
    p.save(str(fname))
    with open(fname) as f:
        back = json.load(f)
    assert back == d
    q = Parameters(back)
    for k in ("spectral_shape", "physical_shape", "nn", "dx", "dz", "initial_dt", "dump_cadence",
              "integrator", "integrator_order", "spatial_derivative_order", "discretisation"):
        assert getattr(q, k) == getattr(p, k), k
    assert q.Ra == 1e7 and q.Pr == 1.0
    # the default file name is the reference's
    import os

    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        Parameters(d).save()
        assert (tmp_path / "params.json").exists()
    finally:
        os.chdir(cwd)
