"""History of time derivatives (melvin/TimeDerivative.py).

A ring buffer of ``integrator_order`` spectral slots, zero at start;
``dvar[:] = f`` writes slot ``curr``, ``get(k)`` reads slot ``curr + k``
(negative k wraps), ``advance`` rotates ``curr``.
"""

import numpy as np
import torch


class TimeDerivative:
    def __init__(self, params, xp=None, dump_name="", array_factory=None):
        self._params = params
        self._curr_idx = 0
        self._device = torch.device(getattr(params, "device", "cuda"))
        self._data = torch.zeros(
            (params.integrator_order, params.spectral_shape[0], params.spectral_shape[1]),
            dtype=torch.complex128, device=self._device,
        )
        self._dump_name = dump_name

    def __setitem__(self, index, value):
        if isinstance(value, np.ndarray):
            value = torch.as_tensor(value, device=self._device)
        self._data[self._curr_idx][index] = value

    def __getitem__(self, index):
        return self._data[self._curr_idx][index]

    def get_curr_idx(self):
        return self._curr_idx

    def set_curr_idx(self, curr_idx):
        self._curr_idx = int(curr_idx)

    def advance(self):
        self._curr_idx = (self._curr_idx + 1) % self._params.integrator_order

    def get(self, idx=0):
        return self._data[self._curr_idx + idx]

    def get_all(self):
        return self._data

    def set(self, data, idx=0):
        self._data[self._curr_idx + idx] = torch.as_tensor(data, device=self._device)

    def load(self, data):
        if isinstance(data, str):
            raise NotImplementedError
        arr = torch.as_tensor(np.asarray(data), device=self._device).to(torch.complex128)
        if tuple(arr.shape) != tuple(self._data.shape):
            raise ValueError(f"history of shape {tuple(arr.shape)} does not match {tuple(self._data.shape)}")
        self._data.copy_(arr)

    def get_name(self):
        return self._dump_name
