"""Host <-> device transfers (melvin/DataTransferer.py).

Arrays live on the CUDA device as torch tensors whatever ``xp`` module the
caller passed; ``from_host`` accepts numpy arrays, Python scalars or
tensors, ``to_host`` returns numpy arrays.
"""

import numpy as np
import torch


class DataTransferer:
    def __init__(self, xp=None, device="cuda"):
        self._device = torch.device(device)

    def from_host(self, data, dtype=None):
        if isinstance(data, torch.Tensor):
            t = data.to(self._device)
        else:
            t = torch.as_tensor(np.asarray(data), device=self._device)
        if dtype is not None:
            t = t.to(dtype)
        return t

    def to_host(self, data):
        if isinstance(data, torch.Tensor):
            return data.detach().cpu().numpy()
        return np.asarray(data)
