"""Host logic of the device-driven loop (no GPU): which scalar trackers run
on the device and with what, as the examples bind them
(examples/double_diffusive_convection.py:80-89), and the Nusselt-number
function itself on plain arrays."""

import functools

import numpy as np
import pytest

pytest.importorskip("torch")

from melvin import utility  # noqa: E402
from melvin.driver import DeviceRun  # noqa: E402


class _Tracker:
    def __init__(self, filename):
        self._filename = filename


class _Var:
    """Stand-in Variable: getp() returns a fixed physical array."""

    def __init__(self, arr):
        self._arr = arr

    def getp(self):
        import torch

        return torch.as_tensor(self._arr)


def test_kinetic_energy_tracker_by_function_or_file_name():
    fn = functools.partial(utility.calc_kinetic_energy, "ux", "uz", None, None)
    assert DeviceRun._classify(_Tracker("anything.npz"), fn) == ("ke", None)
    assert DeviceRun._classify(_Tracker("kinetic_energy.npz"), lambda: 0.0) == ("ke", None)
    assert DeviceRun._classify(_Tracker("out/kinetic_energy"), None) == ("ke", None)


def test_nusselt_tracker_names_its_field():
    tmp, uz = object(), object()
    kind, var = DeviceRun._classify(_Tracker("nusselt_number.npz"),
                                    functools.partial(utility.calc_nusselt_number, tmp, uz, None, None))
    assert kind == "nusselt" and var is tmp


def test_other_trackers_are_refused():
    with pytest.raises(ValueError, match="only the kinetic energy and the Nusselt number"):
        DeviceRun._classify(_Tracker("enstrophy.npz"), lambda: 0.0)
    # a Nusselt tracker is recognised by its function, not by its file name
    with pytest.raises(ValueError):
        DeviceRun._classify(_Tracker("nusselt_number.npz"), lambda: 0.0)


def test_calc_nusselt_number_is_one_minus_mean_flux():
    rng = np.random.default_rng(0)
    t, w = rng.standard_normal((8, 6)), rng.standard_normal((8, 6))
    assert utility.calc_nusselt_number(_Var(t), _Var(w)) == pytest.approx(1.0 - np.mean(t * w), rel=1e-15)
