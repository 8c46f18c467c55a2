"""Scalar time series saved as ``.npz`` (melvin/ScalarTracker.py)."""

import numpy as np


class ScalarTracker:
    def __init__(self, params, xp, filename):
        self._params = params
        self._filename = filename
        self._values = []
        self._times = []

    def append(self, t, val):
        self._times.append(t)
        self._values.append(float(val))

    def save(self, _index):
        np.savez(self._filename, t=np.array(self._times), values=np.array(self._values))
